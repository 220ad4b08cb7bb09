"""Tidal TaylorF2 (13 Fisher parameters: ... chi2z, LambdaTilde, deltaLambda) through the C ABI against the
oracle, which tests/test_oracle_golden.py pins to gwfast's own tidal TaylorF2.

Tolerances as for the 11-parameter FP64 path: SNR relative 1e-10, Fisher |dF_ab| <= 1e-9 sqrt(F_aa F_bb).
"""
import numpy as np
import pytest

import oracle as O
from gwfast_gb300 import _lib, fisherTools, synthetic
from gwfast_gb300 import waveforms as W

from test_gpu_parity import fisher_err, oracle_det

pytestmark = pytest.mark.gpu


def tidal_events(n, seed, from_components=True):
    ev = synthetic.bns_events(n, seed=seed)
    rng = np.random.default_rng(seed + 1)
    l1, l2 = rng.uniform(50., 1500., n), rng.uniform(50., 1500., n)
    if from_components:
        ev['Lambda1'], ev['Lambda2'] = l1, l2
    else:
        from gwfast_gb300 import gwfastUtils as U
        ev['LambdaTilde'], ev['deltaLambda'] = U.Lamt_delLam_from_Lam12(l1, l2, ev['eta'])
    return ev


@pytest.mark.parametrize('earth', [False, True])
@pytest.mark.parametrize('det', [('Virgo', 10.), ('ETS', 5.)])
def test_tidal_snr_and_fisher_per_arm(gpu_lib, det, earth):
    ev = tidal_events(4, seed=51)
    res = 400
    wf = W.TaylorF2_RestrictedPN(is_tidal=True)
    assert wf.nParams == 13 and wf.ParNums['deltaLambda'] == 12
    net = synthetic.make_network(wf, dets=(det,), earth=earth)
    snrs = net.SNR(dict(ev), res=res, return_all=True)
    evd = dict(ev)
    Fs = net.FisherMatr(evd, res=res, return_all=True)
    assert 'LambdaTilde' in evd and 'deltaLambda' in evd      # the dict gains the Fisher parameters
    om = O.Model('TF2', tidal=True)
    p = O.to_params(evd, om.params)
    od = oracle_det(det[0], det[1], earth)
    arms = O.snr_arms(od, om, p, res)
    Fo = O.fisher_arms(od, om, p, res)
    names = [det[0]] if od.shape == 'L' else ['%s_%d' % (det[0], i) for i in range(3)]
    for nm, a, F in zip(names, arms, Fo):
        assert np.max(np.abs(snrs[nm] - a.numpy()) / a.numpy()) < 1e-10, nm
        Fk = np.moveaxis(Fs[nm], -1, 0)
        assert Fk.shape == (4, 13, 13)
        err = fisher_err(Fk, F.numpy())
        assert err < 1e-9, (nm, err)


def test_tidal_network_covariance_and_inputs(gpu_lib):
    """Network total, 13 x 13 covariance on the GPU, and LambdaTilde/deltaLambda given directly."""
    ev = tidal_events(6, seed=61)
    res = 500
    dets = (('L1', 10.), ('ETS', 5.))
    wf = W.TaylorF2_RestrictedPN(is_tidal=True)
    net = synthetic.make_network(wf, dets=dets, earth=True)
    evd = dict(ev)
    F = net.FisherMatr(evd, res=res)
    assert F.shape == (13, 13, 6)
    om = O.Model('TF2', tidal=True)
    p = O.to_params(evd, om.params)
    Fo = sum(O.fisher(oracle_det(n, fm, True), om, p, res) for n, fm in dets).numpy()
    assert fisher_err(np.moveaxis(F, -1, 0), Fo) < 1e-9
    cov, eps, cond = fisherTools.CovMatr(F, return_cond=True)
    assert cov.shape == (13, 13, 6)
    covo, epso = O.cov_matr_fast(np.moveaxis(F, -1, 0))
    s = np.sqrt(np.einsum('iin->ni', cov))
    so = np.sqrt(np.einsum('nii->ni', covo))
    # two FP64 inversions of matrices with equilibrated condition numbers of 1e9-1e14 agree to about
    # cond x 1e-16 (the tidal parameters are nearly degenerate with the masses)
    err = (np.abs(s - so) / so).max(axis=1)
    print('tidal covariance: cond', cond, 'sigma difference', err)
    assert np.all(err < np.maximum(1e-9, 1e-14 * cond))
    # the same events given as (LambdaTilde, deltaLambda)
    ev2 = {k: v for k, v in ev.items() if k not in ('Lambda1', 'Lambda2')}
    ev2['LambdaTilde'], ev2['deltaLambda'] = evd['LambdaTilde'], evd['deltaLambda']
    F2 = net.FisherMatr(dict(ev2), res=res)
    assert fisher_err(np.moveaxis(F2, -1, 0), np.moveaxis(F, -1, 0)) < 1e-12


def test_tidal_fp32_is_rejected(gpu_lib):
    ev = tidal_events(2, seed=3)
    net = synthetic.make_network(W.TaylorF2_RestrictedPN(is_tidal=True), dets=(('L1', 10.),), earth=False)
    with pytest.raises(_lib.GWFError):
        net.FisherMatr(dict(ev), res=100, precision='fp32')
