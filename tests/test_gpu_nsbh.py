"""IMRPhenomNSBH (13 Fisher parameters) through the C ABI against the oracle, which
tests/test_oracle_golden.py pins to gwfast's own IMRPhenomNSBH.

The model interpolates xi_tide (arXiv:1509.00512 eq. 8) on a 200^3 table, which gwfast tabulates
with numpy's companion-matrix roots and this build on the device with an exact real-root
isolation; the table itself is compared with numpy's roots at random nodes and cell interiors.

The grid ends at M f = 0.2, where gwfast cuts the waveform (M f < 0.2): whether the last point
falls on the kept side is decided by the rounding of M G fcut, in gwfast and here alike. Unlike
IMRPhenomD's, this model's amplitude there (and its tangent in LambdaTilde, for the
non-disruptive mergers) is large enough to move the Fisher matrix by ~1e-6 of sqrt(F_aa F_bb), so
each event is compared with the oracle taken both ways and has to match one of them.

Tolerances as for the other FP64 models: SNR relative 1e-10, Fisher |dF_ab| <= 1e-9 sqrt(F_aa F_bb).
"""
import numpy as np
import pytest
import torch

import oracle as O
from gwfast_gb300 import _lib, fisherTools, synthetic
from gwfast_gb300 import waveforms as W

from test_gpu_parity import fisher_err, oracle_det

pytestmark = pytest.mark.gpu

SNR_TOL = 1e-10
F_TOL = 1e-9


def nsbh_events(n, seed):
    """BH 5-20 Msun with spin in [-0.5, 0.95], NS 1.2-2 Msun without spin, Lambda2 in [1, 3000] (one
    event below 1): the set spans disruptive, mildly disruptive and non-disruptive mergers."""
    rng = np.random.default_rng(seed)
    m1, m2 = rng.uniform(5., 20., n), rng.uniform(1.2, 2., n)
    ev = {'Mc': (m1 * m2) ** 0.6 / (m1 + m2) ** 0.2, 'eta': m1 * m2 / (m1 + m2) ** 2,
          'chi1z': rng.uniform(-0.5, 0.95, n), 'chi2z': np.zeros(n), 'dL': rng.uniform(0.05, 0.5, n),
          'theta': np.arccos(rng.uniform(-1, 1, n)), 'phi': rng.uniform(0, 2 * np.pi, n),
          'iota': np.arccos(rng.uniform(-1, 1, n)), 'psi': rng.uniform(0, np.pi, n), 'tcoal': rng.uniform(0, 1, n),
          'Phicoal': rng.uniform(0, 2 * np.pi, n)}
    ev['Lambda1'] = np.zeros(n)
    ev['Lambda2'] = rng.uniform(1., 3000., n)
    ev['Lambda2'][-1] = 0.7
    return ev


def oracle_both(fn):
    """fn(model) with the last grid point kept and cut."""
    return [fn(O.Model('PhenomNSBH', cut_last=np.full((1,), c))) for c in (False, True)]


def fisher_err_per_event(F, Fr):
    d = np.sqrt(np.abs(np.einsum('nii->ni', Fr)))
    return (np.abs(F - Fr) / (d[:, :, None] * d[:, None, :])).max(axis=(1, 2))


def test_xitide_table(gpu_lib):
    """The device table at random nodes (exactly numpy's roots, as gwfast tabulates them) and the
    trilinear interpolation at random interior points, against the oracle."""
    ctx = _lib.context(0)
    rng = np.random.default_rng(3)
    n = 400
    ii, jj, kk = (rng.integers(0, 200, n) for _ in range(3))
    g = O.XI_GRID
    node = ctx.xitide(g[0][ii], g[1][jj], g[2][kk])
    ref = np.array([O.xitide_node(a, b, c) for a, b, c in zip(ii, jj, kk)])
    err = np.abs(node - ref) / ref
    # at spin 1 the polynomial has a double root, which numpy's eigenvalues split by ~1e-8 relative
    assert np.max(err[kk < 199]) < 1e-12
    kk1 = np.full(20, 199)
    node1 = ctx.xitide(g[0][ii[:20]], g[1][jj[:20]], g[2][kk1])
    ref1 = np.array([O.xitide_node(a, b, c) for a, b, c in zip(ii[:20], jj[:20], kk1)])
    assert np.max(np.abs(node1 - ref1) / ref1) < 1e-6
    C, q, chi = rng.uniform(0.1, 0.5, n), rng.uniform(1., 100., n), rng.uniform(-1., 0.98, n)
    val = ctx.xitide(C, q, chi)
    ref = O.xitide_interp(torch.as_tensor(C), torch.as_tensor(q), torch.as_tensor(chi)).numpy()
    assert np.max(np.abs(val - ref) / ref) < 1e-12
    # outside the compactness and mass-ratio ranges gwfast extrapolates; outside the spin range: NaN
    out = ctx.xitide(np.array([0.05, 0.3]), np.array([3., 120.]), np.array([0.2, 0.2]))
    assert np.all(np.isfinite(out))
    assert np.isnan(ctx.xitide(np.array([0.3]), np.array([3.]), np.array([1.5])))[0]


@pytest.mark.parametrize('earth', [False, True])
@pytest.mark.parametrize('det', [('L1', 10.), ('ETS', 5.)])
def test_nsbh_snr_and_fisher_per_arm(gpu_lib, det, earth):
    ev = nsbh_events(6, seed=101)
    res = 400
    wf = W.IMRPhenomNSBH(verbose=False)
    assert wf.nParams == 13 and wf.objType == 'NSBH'
    net = synthetic.make_network(wf, dets=(det,), earth=earth)
    snrs = net.SNR(dict(ev), res=res, return_all=True)
    evd = dict(ev)
    Fs = net.FisherMatr(evd, res=res, return_all=True)
    p = O.to_params(evd, O.PARAMS_TIDAL)
    od = oracle_det(det[0], det[1], earth)
    arms = oracle_both(lambda m: O.snr_arms(od, m, p, res))
    Fo = oracle_both(lambda m: O.fisher_arms(od, m, p, res))
    names = [det[0]] if od.shape == 'L' else ['%s_%d' % (det[0], i) for i in range(3)]
    for k, nm in enumerate(names):
        se = np.minimum(*(np.abs(snrs[nm] - a[k].numpy()) / a[k].numpy() for a in arms))
        assert se.max() < SNR_TOL, (nm, se)
        Fk = np.moveaxis(Fs[nm], -1, 0)
        fe = np.minimum(*(fisher_err_per_event(Fk, F[k].numpy()) for F in Fo))
        assert fe.max() < F_TOL, (nm, fe)


def test_nsbh_network_and_covariance(gpu_lib):
    ev = nsbh_events(5, seed=103)
    res = 500
    dets = (('L1', 10.), ('ETS', 5.))
    net = synthetic.make_network(W.IMRPhenomNSBH(verbose=False), dets=dets, earth=True)
    evd = dict(ev)
    F = net.FisherMatr(evd, res=res)
    assert F.shape == (13, 13, 5)
    p = O.to_params(evd, O.PARAMS_TIDAL)
    # every detector's grid ends at the same M f, so an event's last point is on the same side in all
    Fo = oracle_both(lambda m: sum(O.fisher(oracle_det(n, fm, True), m, p, res) for n, fm in dets).numpy())
    assert np.minimum(*(fisher_err_per_event(np.moveaxis(F, -1, 0), x) for x in Fo)).max() < F_TOL
    snr = net.SNR(dict(ev), res=res)
    so = oracle_both(lambda m: O.network_snr([oracle_det(n, fm, True) for n, fm in dets], m, p, res).numpy())
    assert np.minimum(*(np.abs(snr - x) / x for x in so)).max() < SNR_TOL
    cov, eps, cond = fisherTools.CovMatr(F, return_cond=True)
    assert np.all(np.isfinite(cov))
    with pytest.raises(_lib.GWFError):
        net.FisherMatr(dict(ev), res=100, precision='fp32')
