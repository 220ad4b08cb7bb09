"""FP64 CUDA path against the oracle, through the C ABI (gwf_snr / gwf_fisher / gwf_cov).

Tolerances: SNR relative error <= 1e-10; Fisher entries |dF_ab| <= 1e-9 sqrt(F_aa F_bb)
(both computed in float64; the residual is rounding plus the last-grid-point cut of the
IMR models, see test_oracle_golden).
"""
import numpy as np
import pytest
import torch

import oracle as O
from gwfast_gb300 import fisherTools, synthetic
from gwfast_gb300 import waveforms as W

pytestmark = pytest.mark.gpu

MODELS = {
    'TF2': (lambda: W.TaylorF2_RestrictedPN(), O.Model('TF2'), 'bns'),
    'TF2_spinHO': (lambda: W.TaylorF2_RestrictedPN(use_3p5PN_SpinHO=True), O.Model('TF2', spin_ho=True), 'bns'),
    'PhenomD': (lambda: W.IMRPhenomD(), O.Model('PhenomD'), 'bbh'),
    'PhenomHM': (lambda: W.IMRPhenomHM(), O.Model('PhenomHM'), 'bbh'),
}
SNR_TOL = 1e-10
F_TOL = 1e-9
F_TOL_HM = 5e-9   # six-mode sum: the oracle solves the 5x5 collocation system, the kernel uses Newton-Hermite form


def events(kind, n, seed):
    if kind == 'bns':
        return synthetic.bns_events(n, seed=seed)
    return synthetic.bbh_events(n, seed=seed, mmax=150., qmin=0.1, chimax=0.9)


def oracle_det(name, fmin, earth):
    spec = synthetic.detector_spec(name, fmin)
    f, S = spec['psd_path']
    return O.Detector(spec['det_lat'], spec['det_long'], spec['det_xax'], spec['detector_shape'], fmin=fmin,
                      psd_f=f, psd_S=S, earth=earth)


def fisher_err(F, Fr):
    d = np.sqrt(np.abs(np.einsum('nii->ni', Fr)))
    return (np.abs(F - Fr) / (d[:, :, None] * d[:, None, :])).max()


@pytest.mark.parametrize('earth', [False, True])
@pytest.mark.parametrize('det', [('Virgo', 10.), ('ETS', 5.)])
@pytest.mark.parametrize('model', list(MODELS))
def test_snr_and_fisher_per_arm(gpu_lib, model, det, earth):
    mk, om, kind = MODELS[model]
    ev = events(kind, 5, seed=7)
    res = 300
    net = synthetic.make_network(mk(), dets=(det,), earth=earth)
    snrs = net.SNR(dict(ev), res=res, return_all=True)
    Fs = net.FisherMatr(dict(ev), res=res, return_all=True)
    p = O.to_params(ev)
    od = oracle_det(det[0], det[1], earth)
    arms = O.snr_arms(od, om, p, res)
    Fo = O.fisher_arms(od, om, p, res)
    names = [det[0]] if od.shape == 'L' else ['%s_%d' % (det[0], i) for i in range(3)]
    for nm, a, F in zip(names, arms, Fo):
        s = snrs[nm]
        assert np.max(np.abs(s - a.numpy()) / a.numpy()) < SNR_TOL, nm
        err = fisher_err(np.moveaxis(Fs[nm], -1, 0), F.numpy())
        assert err < (F_TOL_HM if om.is_hm else F_TOL), (nm, err)


@pytest.mark.parametrize('model', ['TF2', 'PhenomD', 'PhenomHM'])
def test_network_total(gpu_lib, model):
    """DetNet.FisherMatr default path (triangle total via two Gram sets) against the oracle sum over arms."""
    mk, om, kind = MODELS[model]
    ev = events(kind, 4, seed=11)
    res = 250
    dets = synthetic.NETWORK_LHET
    net = synthetic.make_network(mk(), dets=dets, earth=True)
    F = np.moveaxis(net.FisherMatr(dict(ev), res=res), -1, 0)
    snr = net.SNR(dict(ev), res=res)
    p = O.to_params(ev)
    Fo = sum(O.fisher(oracle_det(n, fm, True), om, p, res) for n, fm in dets).numpy()
    so = O.network_snr([oracle_det(n, fm, True) for n, fm in dets], om, p, res).numpy()
    assert fisher_err(F, Fo) < (F_TOL_HM if om.is_hm else F_TOL)
    assert np.max(np.abs(snr - so) / so) < SNR_TOL


def test_identities_full_size(gpu_lib):
    """F_dLdL = (SNR/dL)^2 and F_PhicPhic = SNR^2 hold for a 22-mode model at full grid size."""
    ev = synthetic.bbh_events(64, seed=3)
    net = synthetic.make_network(W.IMRPhenomD(), earth=True)
    F = net.FisherMatr(dict(ev), res=2000)
    snr = net.SNR(dict(ev), res=2000)
    assert np.allclose(F[2, 2], (snr / ev['dL']) ** 2, rtol=1e-11)
    assert np.allclose(F[8, 8], snr ** 2, rtol=1e-11)
    assert np.all(np.abs(F - np.swapaxes(F, 0, 1)) <= 1e-14 * np.abs(F).max(axis=(0, 1)))


def test_triangle_null_stream_consistency(gpu_lib):
    """Per-arm triangle Fishers sum to the detector total computed with the two-Gram identity."""
    ev = synthetic.bbh_events(16, seed=5)
    net = synthetic.make_network(W.IMRPhenomD(), dets=(('ETS', 5.),), earth=True)
    Fa = net.FisherMatr(dict(ev), res=800, return_all=True)
    Ft = net.FisherMatr(dict(ev), res=800)
    S = Fa['ETS_0'] + Fa['ETS_1'] + Fa['ETS_2']
    assert fisher_err(np.moveaxis(Ft, -1, 0), np.moveaxis(S, -1, 0)) < 1e-12


def test_covariance_against_oracle(gpu_lib):
    ev = synthetic.bbh_events(32, seed=9)
    net = synthetic.make_network(W.IMRPhenomD(), earth=True)
    F = net.FisherMatr(dict(ev), res=1000)
    cov, eps, cond = fisherTools.CovMatr(F, return_cond=True)
    Fn = np.moveaxis(F, -1, 0)
    cref, eref = O.cov_matr_fast(Fn)
    # two float64 inversions agree to ~ eps_machine x condition number of the equilibrated matrix
    tol = np.maximum(1e-9, 1e-13 * cond)
    s = np.sqrt(np.einsum('nii->ni', np.moveaxis(cov, -1, 0)))
    sr = np.sqrt(np.einsum('nii->ni', cref))
    ok = cond < 1e12
    assert ok.sum() >= 16
    assert np.all((np.abs(s - sr) / sr).max(axis=1)[ok] < tol[ok])
    # residual of the equilibrated system, diag(w) (Cov F - 1) diag(1/w), is rounding-level x condition number
    w = 1. / np.sqrt(np.einsum('nii->ni', Fn))
    C = np.moveaxis(cov, -1, 0)
    Req = (C @ Fn - np.eye(11)) * (1. / w)[:, :, None] * w[:, None, :]
    assert np.all(np.abs(Req).max(axis=(1, 2))[ok] < 1e-13 * cond[ok] + 1e-12)
    assert np.allclose(eps, eref, rtol=0.5, atol=1e-9) or np.all(eps[ok] < 100 * eref[ok] + 1e-9)
    # gwfast's own mpmath path on a few events
    C3, e3, c3 = O.cov_matr(Fn[:4])
    s3 = np.sqrt(np.einsum('nii->ni', C3))
    good = c3 < 1e12
    assert np.all((np.abs(s[:4] - s3) / s3).max(axis=1)[good] < tol[:4][good])
    assert np.allclose(cond[:4][good], c3[good], rtol=1e-4)


def test_per_event_grid_and_linear_spacing(gpu_lib):
    """res_per_event and spacing='lin' through the ABI against the oracle."""
    from gwfast_gb300 import _lib
    from gwfast_gb300.signal import event_array
    ev = synthetic.bbh_events(3, seed=13)
    net = synthetic.make_network(W.IMRPhenomD(), dets=(('L1', 10.),), earth=False)
    sig = net.signals['L1']
    p = event_array(ev)
    ctx = _lib.context(0)
    res = np.array([120, 333, 77], dtype=np.int32)
    out = np.empty((3, 11, 11))
    ctx.fisher([sig.det_id], W.IMRPhenomD().gpu_desc(), p, 0, res_ev=res, per_arm=False, out_net=out)
    od = oracle_det('L1', 10., False)
    P = O.to_params(ev)
    for i in range(3):
        Pi = {k: v[i:i + 1] for k, v in P.items()}
        Fo = O.fisher(od, O.Model('PhenomD'), Pi, int(res[i])).numpy()
        assert fisher_err(out[i:i + 1], Fo) < F_TOL
    Fl = np.moveaxis(sig.FisherMatr(dict(ev), res=200, spacing='lin'), -1, 0)
    f, S = O.event_grid(od, O.Model('PhenomD'), P, 200, spacing='lin')
    D = O.strain_jacobian(od, O.Model('PhenomD'), f, P, 0.)
    D[O.TC_INDEX] = D[O.TC_INDEX] / O.DAY_S
    assert fisher_err(Fl, O._gram(D, S, f).numpy()) < F_TOL


def test_errors_are_reported(gpu_lib):
    from gwfast_gb300 import _lib
    with pytest.raises(ValueError):
        synthetic.make_network(W.IMRPhenomD()).SNR({'Mc': np.array([30.])})
    ctx = _lib.context(0)
    with pytest.raises(_lib.GWFError):
        ctx.snr([999], W.IMRPhenomD().gpu_desc(), np.zeros((11, 2)), 100, out_net=np.empty(2))
    with pytest.raises(_lib.GWFError):
        ctx.add_detector(0., 0., 0., 'L', False, 10., None, np.array([2., 1.]), np.array([1., 1.]))


@pytest.mark.parametrize('model', ['TF2', 'PhenomD', 'PhenomHM'])
def test_snr_derivatives(gpu_lib, model):
    """return_SNR_derivatives: per-arm 4 trapz(Re(h conj(dh/dtheta)) / S) against the oracle, and the
    identities sum_arms 4 trapz(Re(h conj(dh/ddL)) / S) = -dL F_dLdL and the Phicoal one = 0 (the
    network entry is divided by DetNet.SNR, which for IMRPhenomHM is gwfast's SNR without the
    h+ hx cross term, so the identity is checked on the undivided sum)."""
    mk, om, kind = MODELS[model]
    ev = events(kind, 4, seed=17)
    res = 300
    dets = (('L1', 10.), ('ETS', 5.))
    net = synthetic.make_network(mk(), dets=dets, earth=True)
    allF, allDer = net.FisherMatr(dict(ev), res=res, return_SNR_derivatives=True)
    p = O.to_params(ev)
    worst = 0.0
    for name, fmin in dets:
        od = oracle_det(name, fmin, True)
        ref = O.snr_derivs_arms(od, om, p, res)
        snr = O.snr_arms(od, om, p, res)
        keys = [name] if od.shape == 'L' else ['%s_%d' % (name, i) for i in range(3)]
        for k, r, sn in zip(keys, ref, snr):
            Fd = np.sqrt(np.abs(np.einsum('iin->in', allF[k])))
            scale = sn.numpy()[None] / 2. * Fd          # Cauchy-Schwarz bound of each entry
            worst = max(worst, np.max(np.abs(allDer[k] - r.numpy()) / scale))
    print('%s SNR derivatives: max normalised error %.2e' % (model, worst))
    assert worst < (F_TOL_HM if model == 'PhenomHM' else F_TOL)
    snr_net = net.SNR(dict(ev))   # the divisor of the 'net' entry: DetNet.SNR at its default res, as gwfast
    d = allDer['net']
    assert np.allclose(d[2] * snr_net, -ev['dL'] * allF['net'][2, 2], rtol=1e-9)
    assert np.all(np.abs(d[8]) < 1e-9 * np.sqrt(np.einsum('iin->in', allF['net'])[8]))


def test_snr_derivatives_fp32(gpu_lib):
    ev = synthetic.bbh_events(256, seed=19)
    net = synthetic.make_network(W.IMRPhenomD(), earth=True)
    F64, D64 = net.FisherMatr(dict(ev), res=1000, return_SNR_derivatives=True)
    F32, D32 = net.FisherMatr(dict(ev), res=1000, return_SNR_derivatives=True, precision='fp32')
    Fd = np.sqrt(np.abs(np.einsum('iin->in', F64['net'])))
    err = np.max(np.abs(D32['net'] - D64['net']) / Fd)
    print('fp32 dSNR/dtheta max error relative to sqrt(F_aa): %.2e' % err)
    assert err < 1e-5
