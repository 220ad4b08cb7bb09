"""TaylorF2 options through the C ABI against the oracle, which tests/test_oracle_golden.py pins to
gwfast's own TaylorF2 with the same options: orbital eccentricity (the ecc Fisher parameter, 12
parameters; with the tidal terms 14), the spin-induced quadrupole moments of tidal bodies
(use_QuadMonTid), the phase referenced at the last stable orbit (phiref_vlso), fRef_ecc, and the
cut at twice the Kerr-remnant ISCO (which_ISCO='Kerr').

Tolerances as for the other FP64 models: SNR relative 1e-10, Fisher |dF_ab| <= 1e-9 sqrt(F_aa F_bb);
the FP32 form of the 11-parameter options against the FP64 kernel as in test_gpu_fp32.
"""
import numpy as np
import pytest

import oracle as O
from gwfast_gb300 import _lib, fisherTools, synthetic
from gwfast_gb300 import waveforms as W

from test_gpu_parity import fisher_err, oracle_det

pytestmark = pytest.mark.gpu

SNR_TOL = 1e-10
F_TOL = 1e-9


def ecc_events(n, seed, tidal=False, chimax=0.05):
    ev = synthetic.bns_events(n, seed=seed, chimax=chimax)
    rng = np.random.default_rng(seed + 1)
    ev['ecc'] = rng.uniform(0.005, 0.2, n)
    if tidal:
        ev['Lambda1'], ev['Lambda2'] = rng.uniform(50., 1500., n), rng.uniform(50., 1500., n)
        ev['Lambda1'][-1] = 0.6   # one star on the polynomial branch of the quadrupole relation
    return ev


def run_per_arm(wf, om, ev, det, earth, res, P):
    net = synthetic.make_network(wf, dets=(det,), earth=earth)
    snrs = net.SNR(dict(ev), res=res, return_all=True)
    evd = dict(ev)
    Fs = net.FisherMatr(evd, res=res, return_all=True)
    p = O.to_params(evd, om.params)
    od = oracle_det(det[0], det[1], earth)
    arms = O.snr_arms(od, om, p, res)
    Fo = O.fisher_arms(od, om, p, res)
    names = [det[0]] if od.shape == 'L' else ['%s_%d' % (det[0], i) for i in range(3)]
    for nm, a, F in zip(names, arms, Fo):
        assert np.max(np.abs(snrs[nm] - a.numpy()) / a.numpy()) < SNR_TOL, nm
        Fk = np.moveaxis(Fs[nm], -1, 0)
        assert Fk.shape[1:] == (P, P)
        err = fisher_err(Fk, F.numpy())
        assert err < F_TOL, (nm, err)


@pytest.mark.parametrize('earth', [False, True])
@pytest.mark.parametrize('det', [('L1', 10.), ('ETS', 5.)])
def test_eccentric_per_arm(gpu_lib, det, earth):
    wf = W.TaylorF2_RestrictedPN(is_eccentric=True)
    assert wf.nParams == 12 and wf.ParNums['ecc'] == 11
    run_per_arm(wf, O.Model('TF2', ecc=True), ecc_events(5, seed=91), det, earth, 400, 12)


@pytest.mark.parametrize('det', [('Virgo', 10.), ('ETS', 5.)])
def test_tidal_eccentric_options_per_arm(gpu_lib, det):
    wf = W.TaylorF2_RestrictedPN(is_tidal=True, is_eccentric=True, use_QuadMonTid=True, phiref_vlso=True,
                                 fRef_ecc=8.)
    assert wf.nParams == 14 and wf.ParNums['ecc'] == 13
    om = O.Model('TF2', tidal=True, ecc=True, quadmon=True, vlso=True, fref_ecc=8.)
    run_per_arm(wf, om, ecc_events(5, seed=93, tidal=True, chimax=0.3), det, True, 400, 14)


@pytest.mark.parametrize('opts', [dict(use_QuadMonTid=True), dict(phiref_vlso=True, use_3p5PN_SpinHO=True)],
                         ids=['quadmon', 'vlso'])
def test_tidal_options_per_arm(gpu_lib, opts):
    wf = W.TaylorF2_RestrictedPN(is_tidal=True, **opts)
    om = O.Model('TF2', tidal=True, quadmon=opts.get('use_QuadMonTid', False), vlso=opts.get('phiref_vlso', False),
                 spin_ho=opts.get('use_3p5PN_SpinHO', False))
    ev = ecc_events(5, seed=95, tidal=True, chimax=0.3)
    del ev['ecc']
    run_per_arm(wf, om, ev, ('ETS', 5.), True, 400, 13)


def test_eccentric_network_detector_reference_and_covariance(gpu_lib):
    """L1 (10 Hz) + ETS (5 Hz): without fRef_ecc each detector references ecc at its own lowest grid
    frequency, so the shared source record is completed per detector; 12 x 12 and 14 x 14 inversions."""
    res = 500
    dets = (('L1', 10.), ('ETS', 5.))
    for tidal in (False, True):
        wf = W.TaylorF2_RestrictedPN(is_eccentric=True, is_tidal=tidal)
        om = O.Model('TF2', ecc=True, tidal=tidal)
        ev = ecc_events(6, seed=97, tidal=tidal)
        net = synthetic.make_network(wf, dets=dets, earth=True)
        evd = dict(ev)
        F = net.FisherMatr(evd, res=res)
        P = wf.nParams
        assert F.shape == (P, P, 6)
        p = O.to_params(evd, om.params)
        Fo = sum(O.fisher(oracle_det(n, fm, True), om, p, res) for n, fm in dets).numpy()
        assert fisher_err(np.moveaxis(F, -1, 0), Fo) < F_TOL
        snr = net.SNR(dict(ev), res=res)
        so = O.network_snr([oracle_det(n, fm, True) for n, fm in dets], om, p, res).numpy()
        assert np.max(np.abs(snr - so) / so) < SNR_TOL
        cov, eps, cond = fisherTools.CovMatr(F, return_cond=True)
        covo, _ = O.cov_matr_fast(np.moveaxis(F, -1, 0))
        s = np.sqrt(np.einsum('iin->ni', cov))
        so_ = np.sqrt(np.einsum('nii->ni', covo))
        err = (np.abs(s - so_) / so_).max(axis=1)
        assert np.all(err < np.maximum(1e-9, 1e-14 * cond)), (tidal, err, cond)


def test_zero_eccentricity_and_inputs(gpu_lib):
    """ecc = 0: the eccentric phase and its column vanish (the rest equals plain TaylorF2); a missing
    ecc raises as in gwfast; the eccentric forms run on the FP64 path only."""
    ev = synthetic.bns_events(4, seed=5)
    ev['ecc'] = np.zeros(4)
    net = synthetic.make_network(W.TaylorF2_RestrictedPN(is_eccentric=True), dets=(('ETS', 5.),), earth=True)
    F = np.moveaxis(net.FisherMatr(dict(ev), res=300), -1, 0)
    assert np.all(np.isfinite(F)) and np.all(F[:, 11, :] == 0.) and np.all(F[:, :, 11] == 0.)
    net0 = synthetic.make_network(W.TaylorF2_RestrictedPN(), dets=(('ETS', 5.),), earth=True)
    F0 = np.moveaxis(net0.FisherMatr({k: v for k, v in ev.items() if k != 'ecc'}, res=300), -1, 0)
    assert fisher_err(F[:, :11, :11], F0) < 1e-13
    with pytest.raises(ValueError):
        net.FisherMatr({k: v for k, v in ev.items() if k != 'ecc'}, res=300)
    ev['ecc'] = np.full(4, 0.05)
    with pytest.raises(_lib.GWFError):
        net.FisherMatr(dict(ev), res=300, precision='fp32')


@pytest.mark.parametrize('opts', [dict(which_ISCO='Kerr', use_3p5PN_SpinHO=True), dict(phiref_vlso=True)],
                         ids=['kerr', 'vlso'])
def test_tf2_options_fp64_and_fp32(gpu_lib, opts):
    """The 11-parameter options (Kerr-ISCO cut, phiref_vlso) on the FP64 kernel against the oracle, and
    the FP32 split-precision form against the FP64 kernel."""
    wf = W.TaylorF2_RestrictedPN(**opts)
    om = O.Model('TF2', kerr=opts.get('which_ISCO') == 'Kerr', vlso=opts.get('phiref_vlso', False),
                 spin_ho=opts.get('use_3p5PN_SpinHO', False))
    ev = synthetic.bbh_events(6, seed=99, mmax=40., chimax=0.9) if 'which_ISCO' in opts else synthetic.bns_events(6, seed=99)
    run_per_arm(wf, om, ev, ('ETS', 5.), True, 400, 11)
    fc = wf.fcut(**ev)
    p = O.to_params(dict(ev))
    np.testing.assert_allclose(fc, om.fcut_of(p).numpy().reshape(-1), rtol=1e-13)
    ev = synthetic.bbh_events(256, seed=98, mmax=40., chimax=0.9) if 'which_ISCO' in opts else synthetic.bns_events(256, seed=98)
    net = synthetic.make_network(wf, dets=(('ETS', 5.),), earth=True)
    F64 = np.moveaxis(net.FisherMatr(dict(ev), res=2000), -1, 0)
    F32 = np.moveaxis(net.FisherMatr(dict(ev), res=2000, precision='fp32'), -1, 0)
    d = np.sqrt(np.abs(np.einsum('nii->ni', F64)))
    e = (np.abs(F32 - F64) / (d[:, :, None] * d[:, None, :])).max(axis=(1, 2))
    assert np.median(e) < 1e-5, np.median(e)
