"""Strain derivatives (return_derivatives) and WFOverlap through the C ABI (gwf_strain_derivs,
gwf_overlap) against the oracle.

Tolerances: derivative arrays |dD| <= 1e-6 max|D| per (arm, parameter, event) row, overlap
integrals relative 1e-9 (norms) and 1e-7 sqrt(n1 n2) (cross term). Both are FP64; the phase
2 pi f tcoal (up to ~1e9 rad) carries ~1e-7 rad of rounding in either implementation, which
bounds the agreement of complex values point by point.
"""
import numpy as np
import pytest
import torch

import oracle as O
from gwfast_gb300 import synthetic
from gwfast_gb300 import waveforms as W

from test_gpu_parity import MODELS, events, oracle_det

pytestmark = pytest.mark.gpu

D_TOL = 1e-6


@pytest.mark.parametrize('earth', [False, True])
@pytest.mark.parametrize('det', [('Virgo', 10.), ('ETS', 5.)])
@pytest.mark.parametrize('model', ['TF2', 'PhenomD', 'PhenomHM'])
def test_strain_derivatives(gpu_lib, model, det, earth):
    mk, om, kind = MODELS[model]
    ev = events(kind, 3, seed=21)
    res = 200
    net = synthetic.make_network(mk(), dets=(det,), earth=earth)
    sig = list(net.signals.values())[0]
    Fa, Da = sig.FisherMatr(dict(ev), res=res, return_derivatives=True)
    p = O.to_params(ev)
    od = oracle_det(det[0], det[1], earth)
    Do = O.strain_derivs_arms(od, om, p, res)
    assert len(Da) == len(Do) == len(Fa)
    f, S = O.event_grid(od, om, p, res)
    for a, (D, Dr) in enumerate(zip(Da, Do)):
        Dr = Dr.numpy()
        assert D.shape == Dr.shape == (11, 3, res)
        scale = np.abs(Dr).max(axis=-1, keepdims=True)
        rel = np.abs(D - Dr) / np.where(scale > 0, scale, 1.)
        # the IMR models cut the waveform (IMRPhenomHM: each mode) at Mf = 0.2, which is also the
        # last grid point: whether that point lands on the near or the far side of a cut is decided
        # by the last bit of M f in either implementation, so the last point is compared only for
        # TaylorF2 and, for IMRPhenomD, where neither side is cut to zero
        err = rel[..., :-1].max()
        last = rel[..., -1]
        assert err < D_TOL, (a, err)
        if om.name == 'TF2':
            assert last.max() < D_TOL, (a, last.max())
        elif om.name == 'PhenomD':
            zero_one = (np.abs(D[..., -1]) == 0) | (np.abs(Dr[..., -1]) == 0)
            assert np.all((last < D_TOL) | zero_one), (a, last.max())
        # the returned Fisher is the Gram of the returned derivatives
        Fg = O._gram(torch.as_tensor(D), S, f).numpy()
        d = np.sqrt(np.einsum('nii->ni', Fg))
        ferr = (np.abs(np.moveaxis(Fa[a], -1, 0) - Fg) / (d[:, :, None] * d[:, None, :])).max()
        assert ferr < 1e-6, (a, ferr)


def test_strain_derivatives_network_and_reparametrisation(gpu_lib):
    """DetNet.FisherMatr(return_derivatives=True): keys per arm, 'net' Fisher, chain rule to (m1, m2, chiS, chiA)."""
    ev = events('bbh', 2, seed=5)
    res = 150
    net = synthetic.make_network(W.IMRPhenomD(), dets=(('L1', 10.), ('ETS', 5.)), earth=True)
    allF, allD = net.FisherMatr(dict(ev), res=res, return_derivatives=True)
    assert set(allD) == {'L1', 'ETS_0', 'ETS_1', 'ETS_2'}
    assert set(allF) == {'L1', 'ETS_0', 'ETS_1', 'ETS_2', 'net'}
    np.testing.assert_allclose(allD['ETS_2'], -(allD['ETS_0'] + allD['ETS_1']), rtol=0, atol=1e-30)
    Fnet = np.moveaxis(net.FisherMatr(dict(ev), res=res), -1, 0)
    d = np.sqrt(np.einsum('nii->ni', Fnet))
    err = (np.abs(np.moveaxis(allF['net'], -1, 0) - Fnet) / (d[:, :, None] * d[:, None, :])).max()
    assert err < 1e-9
    _, allD2 = net.FisherMatr(dict(ev), res=res, return_derivatives=True, use_chi1chi2=False)
    np.testing.assert_allclose(allD2['L1'][9], allD['L1'][9] + allD['L1'][10], rtol=1e-12, atol=0)
    np.testing.assert_allclose(allD2['L1'][10], allD['L1'][9] - allD['L1'][10], rtol=1e-12, atol=0)


PAIRS = [('TF2', 'TF2', 'bns'), ('PhenomD', 'PhenomD', 'bbh'), ('TF2', 'PhenomD', 'bbh'), ('PhenomD', 'PhenomHM', 'bbh')]


@pytest.mark.parametrize('pair', PAIRS, ids=['-'.join(p[:2]) for p in PAIRS])
def test_overlap(gpu_lib, pair):
    m1, m2, kind = pair
    mk1, om1, _ = MODELS[m1]
    mk2, om2, _ = MODELS[m2]
    ev1 = events(kind, 4, seed=31)
    ev2 = {k: np.array(v, copy=True) for k, v in ev1.items()}
    ev2['Mc'] = ev2['Mc'] * (1. + 2e-4)
    ev2['dL'] = ev2['dL'] * 1.01
    ev2['chi1z'] = ev2['chi1z'] + 0.01
    res = 300
    dets = (('L1', 10.), ('ETS', 5.))
    net = synthetic.make_network(mk1(), dets=dets, earth=True)
    sigs = list(net.signals.values())
    ov_net = net.WFOverlap(mk1(), mk2(), dict(ev1), dict(ev2), res=res)
    p1, p2 = O.to_params(ev1), O.to_params(ev2)
    tot = np.zeros((3, 4))
    for (name, fmin), s in zip(dets, sigs):
        ov, s1, s2 = s.WFOverlap(mk1(), mk2(), dict(ev1), dict(ev2), res=res, return_separate=True)
        o_ov, o_n1, o_n2 = (x.numpy().reshape(-1) for x in O.overlap_parts(oracle_det(name, fmin, True), om1, p1, om2,
                                                                            p2, res))
        assert np.max(np.abs(s1 ** 2 - o_n1) / o_n1) < 1e-9, name
        assert np.max(np.abs(s2 ** 2 - o_n2) / o_n2) < 1e-9, name
        assert np.max(np.abs(ov - o_ov) / np.sqrt(o_n1 * o_n2)) < 1e-7, name
        tot += np.stack([o_ov, o_n1, o_n2])
    ref = tot[0] / np.sqrt(tot[1] * tot[2])
    assert np.max(np.abs(ov_net - ref)) < 1e-7
    assert np.all(np.abs(ov_net) <= 1. + 1e-12)


def test_overlap_identity_and_fmax(gpu_lib):
    """Overlap of a waveform with itself is 1; with a detector fmax the grid follows gwfast's choice."""
    ev = events('bbh', 5, seed=41)
    res = 250
    net = synthetic.make_network(W.IMRPhenomD(), dets=(('H1', 10.),), earth=False)
    s = list(net.signals.values())[0]
    ov = s.WFOverlap(W.IMRPhenomD(), W.IMRPhenomD(), dict(ev), dict(ev), res=res)
    np.testing.assert_allclose(ov, 1., rtol=0, atol=1e-13)
    spec = synthetic.detector_spec('H1', 10.)
    f, S = spec['psd_path']
    from gwfast_gb300.signal import GWSignal
    sf = GWSignal(W.TaylorF2_RestrictedPN(), psd_path=(f, S), detector_shape='L', det_lat=spec['det_lat'],
                  det_long=spec['det_long'], det_xax=spec['det_xax'], is_ASD=False, fmin=10., fmax=60.)
    ev2 = {k: np.array(v, copy=True) for k, v in ev.items()}
    ev2['Mc'] = ev2['Mc'] * 1.5
    ov, s1, s2 = sf.WFOverlap(W.TaylorF2_RestrictedPN(), W.IMRPhenomD(), dict(ev), dict(ev2), res=res,
                              return_separate=True)
    od = O.Detector(spec['det_lat'], spec['det_long'], spec['det_xax'], 'L', fmin=10., fmax=60., psd_f=f, psd_S=S)
    o = [x.numpy().reshape(-1) for x in O.overlap_parts(od, O.Model('TF2'), O.to_params(ev), O.Model('PhenomD'),
                                                        O.to_params(ev2), res)]
    np.testing.assert_allclose(s1 ** 2, o[1], rtol=1e-9)
    np.testing.assert_allclose(s2 ** 2, o[2], rtol=1e-9)
    assert np.max(np.abs(ov - o[0]) / np.sqrt(o[1] * o[2])) < 1e-7


# the tidal, eccentric and NSBH models: (descriptor, oracle model, event kind)
def _tidal_events(n, seed, nsbh=False, ecc=False):
    rng = np.random.default_rng(seed + 7)
    if nsbh:
        m1, m2 = rng.uniform(5., 15., n), rng.uniform(1.2, 2., n)
        ev = events('bns', n, seed)
        ev['Mc'], ev['eta'] = (m1 * m2) ** 0.6 / (m1 + m2) ** 0.2, m1 * m2 / (m1 + m2) ** 2
        ev['chi1z'], ev['chi2z'] = rng.uniform(-0.5, 0.9, n), np.zeros(n)
        ev['Lambda1'], ev['Lambda2'] = np.zeros(n), rng.uniform(10., 2000., n)
        return ev
    ev = events('bns', n, seed)
    ev['Lambda1'], ev['Lambda2'] = rng.uniform(50., 1500., n), rng.uniform(50., 1500., n)
    if ecc:
        ev['ecc'] = rng.uniform(0.01, 0.15, n)
    return ev


MODELS_X = {
    'TF2_tidal_quadmon': (lambda: W.TaylorF2_RestrictedPN(is_tidal=True, use_QuadMonTid=True),
                          O.Model('TF2', tidal=True, quadmon=True), {}),
    'TF2_tidal_ecc_vlso': (lambda: W.TaylorF2_RestrictedPN(is_tidal=True, is_eccentric=True, phiref_vlso=True),
                           O.Model('TF2', tidal=True, ecc=True, vlso=True), dict(ecc=True)),
    'NRTidalv2': (lambda: W.IMRPhenomD_NRTidalv2(), O.Model('PhenomD_NRTidalv2'), {}),
    'NSBH': (lambda: W.IMRPhenomNSBH(verbose=False), O.Model('PhenomNSBH'), dict(nsbh=True)),
}


@pytest.mark.parametrize('model', list(MODELS_X))
def test_strain_derivatives_tidal_models(gpu_lib, model):
    """return_derivatives for the 12-14 parameter models: the (P, N, R) arrays against the oracle (the
    last point of the IMR-based models excluded: it sits on their cut or taper end, see
    test_gpu_nrtidal and test_gpu_nsbh), and the returned Fisher is the Gram of the returned arrays."""
    mk, om, kw = MODELS_X[model]
    ev = _tidal_events(3, 23, **kw)
    res = 200
    wf = mk()
    net = synthetic.make_network(wf, dets=(('ETS', 5.),), earth=True)
    sig = list(net.signals.values())[0]
    evd = dict(ev)
    Fa, Da = sig.FisherMatr(evd, res=res, return_derivatives=True)
    P = wf.nParams
    p = O.to_params(evd, om.params)
    od = oracle_det('ETS', 5., True)
    om.prepare(p)
    Do = O.strain_derivs_arms(od, om, p, res)
    f, S = O.event_grid(od, om, p, res)
    last = None if om.name == 'TF2' else -1
    for a, (D, Dr) in enumerate(zip(Da, Do)):
        Dr = Dr.numpy()
        assert D.shape == Dr.shape == (P, 3, res)
        scale = np.abs(Dr[..., :last]).max(axis=-1, keepdims=True)
        rel = np.abs(D[..., :last] - Dr[..., :last]) / np.where(scale > 0, scale, 1.)
        assert rel.max() < D_TOL, (a, rel.max())
        Fg = O._gram(torch.as_tensor(D), S, f).numpy()
        d = np.sqrt(np.abs(np.einsum('nii->ni', Fg)))
        ferr = (np.abs(np.moveaxis(Fa[a], -1, 0) - Fg) / (d[:, :, None] * d[:, None, :])).max()
        assert ferr < 1e-6, (a, ferr)


PAIRS_X = [('TF2_tidal_quadmon', 'TF2_tidal_ecc_vlso', 1e-7), ('NRTidalv2', 'NRTidalv2', 1e-5),
           ('NSBH', 'NSBH', 1e-5)]


@pytest.mark.parametrize('pair', PAIRS_X, ids=['-'.join(p[:2]) for p in PAIRS_X])
def test_overlap_tidal_models(gpu_lib, pair):
    """WFOverlap with the tidal, eccentric and NSBH models against the oracle. The IMR-based models'
    last grid point (cut or taper end, decided by rounding) moves their integrals by up to ~1e-6,
    hence the looser tolerance there."""
    m1, m2, tol = pair
    mk1, om1, kw1 = MODELS_X[m1]
    mk2, om2, kw2 = MODELS_X[m2]
    ev1 = _tidal_events(3, 31, **{**kw1, **kw2})
    ev2 = {k: np.array(v, copy=True) for k, v in ev1.items()}
    ev2['Mc'] = ev2['Mc'] * (1. + 1e-4)
    ev2['dL'] = ev2['dL'] * 1.01
    res = 300
    dets = (('L1', 10.), ('ETS', 5.))
    net = synthetic.make_network(mk1(), dets=dets, earth=True)
    sigs = list(net.signals.values())
    e1, e2 = dict(ev1), dict(ev2)
    ov_net = net.WFOverlap(mk1(), mk2(), e1, e2, res=res)
    p1, p2 = O.to_params(e1, om1.params), O.to_params(e2, om2.params)
    for (name, fmin), s in zip(dets, sigs):
        ov, s1, s2 = s.WFOverlap(mk1(), mk2(), dict(ev1), dict(ev2), res=res, return_separate=True)
        o_ov, o_n1, o_n2 = (x.numpy().reshape(-1) for x in O.overlap_parts(oracle_det(name, fmin, True), om1, p1, om2,
                                                                            p2, res))
        assert np.max(np.abs(s1 ** 2 - o_n1) / o_n1) < tol, name
        assert np.max(np.abs(s2 ** 2 - o_n2) / o_n2) < tol, name
        assert np.max(np.abs(ov - o_ov) / np.sqrt(o_n1 * o_n2)) < max(tol, 1e-7), name
    assert np.all(np.abs(ov_net) <= 1. + 1e-12)
