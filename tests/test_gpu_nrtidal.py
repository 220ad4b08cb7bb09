"""IMRPhenomD_NRTidalv2 (13 Fisher parameters) through the C ABI against the oracle, which
tests/test_oracle_golden.py pins to gwfast's own IMRPhenomD_NRTidalv2.

The grid of every event ends at fcut = 1.2 f_merger, on the end of the Planck taper: there the
taper formula gives 1 when M f equals 1.2 f_merger to the last bit and 0 otherwise, in gwfast as
here. Which way an event falls depends on the rounding of f_merger and of the grid's last point in
either implementation, so each event is compared with the oracle taken both ways (last-point
taper 0 and 1) and has to match one of them.

Tolerances as for the other FP64 models: SNR relative 1e-10, Fisher |dF_ab| <= 1e-9 sqrt(F_aa F_bb).
"""
import numpy as np
import pytest

import oracle as O
from gwfast_gb300 import _lib, fisherTools, synthetic
from gwfast_gb300 import gwfastUtils as U
from gwfast_gb300 import waveforms as W

from test_gpu_parity import oracle_det

pytestmark = pytest.mark.gpu

SNR_TOL = 1e-10
F_TOL = 1e-9


def nrt_events(n, seed, from_components=True):
    """BNS with spins up to 0.3 (the spin-induced moments matter) and Lambda in [50, 1500]; the last
    two events have one star with Lambda < 1 (the polynomial branch of the quadrupole relation)."""
    ev = synthetic.bns_events(n, seed=seed, chimax=0.3)
    rng = np.random.default_rng(seed + 1)
    l1, l2 = rng.uniform(50., 1500., n), rng.uniform(50., 1500., n)
    l1[-1], l2[-2] = 0.5, 0.8
    if from_components:
        ev['Lambda1'], ev['Lambda2'] = l1, l2
    else:
        ev['LambdaTilde'], ev['deltaLambda'] = U.Lamt_delLam_from_Lam12(l1, l2, ev['eta'])
    return ev


def oracle_both(fn):
    """fn(model) evaluated with the last-point taper at 0 and at 1, stacked on a new first axis."""
    out = []
    for last in (False, True):
        out.append(fn(O.Model('PhenomD_NRTidalv2', taper_last=np.full((1,), last))))
    return out


def snr_err_per_event(s, ref):
    return np.abs(s - ref) / ref


def fisher_err_per_event(F, Fr):
    d = np.sqrt(np.abs(np.einsum('nii->ni', Fr)))
    return (np.abs(F - Fr) / (d[:, :, None] * d[:, None, :])).max(axis=(1, 2))


@pytest.mark.parametrize('earth', [False, True])
@pytest.mark.parametrize('det', [('L1', 10.), ('ETS', 5.)])
def test_nrtidal_snr_and_fisher_per_arm(gpu_lib, det, earth):
    ev = nrt_events(6, seed=71)
    res = 400
    wf = W.IMRPhenomD_NRTidalv2()
    assert wf.nParams == 13 and wf.is_tidal
    net = synthetic.make_network(wf, dets=(det,), earth=earth)
    snrs = net.SNR(dict(ev), res=res, return_all=True)
    evd = dict(ev)
    Fs = net.FisherMatr(evd, res=res, return_all=True)
    om0 = O.Model('PhenomD_NRTidalv2')
    p = O.to_params(evd, om0.params)
    od = oracle_det(det[0], det[1], earth)
    arms = oracle_both(lambda m: O.snr_arms(od, m, p, res))
    Fo = oracle_both(lambda m: O.fisher_arms(od, m, p, res))
    names = [det[0]] if od.shape == 'L' else ['%s_%d' % (det[0], i) for i in range(3)]
    for k, nm in enumerate(names):
        se = np.minimum(*(snr_err_per_event(snrs[nm], a[k].numpy()) for a in arms))
        assert se.max() < SNR_TOL, (nm, se)
        Fk = np.moveaxis(Fs[nm], -1, 0)
        assert Fk.shape == (6, 13, 13)
        fe = np.minimum(*(fisher_err_per_event(Fk, F[k].numpy()) for F in Fo))
        assert fe.max() < F_TOL, (nm, fe)


def test_nrtidal_network_covariance_and_inputs(gpu_lib):
    """Network total, 13 x 13 covariance, and (LambdaTilde, deltaLambda) given directly."""
    ev = nrt_events(5, seed=81)
    res = 500
    dets = (('L1', 10.), ('H1', 10.), ('ETS', 5.))
    net = synthetic.make_network(W.IMRPhenomD_NRTidalv2(), dets=dets, earth=True)
    evd = dict(ev)
    F = net.FisherMatr(evd, res=res)
    snr = net.SNR(dict(ev), res=res)
    assert F.shape == (13, 13, 5)
    p = O.to_params(evd, O.PARAMS_TIDAL)
    # every detector's grid ends on the same fcut, so an event's last-point taper is the same in all
    Fo = oracle_both(lambda m: sum(O.fisher(oracle_det(n, fm, True), m, p, res) for n, fm in dets).numpy())
    so = oracle_both(lambda m: O.network_snr([oracle_det(n, fm, True) for n, fm in dets], m, p, res).numpy())
    Fk = np.moveaxis(F, -1, 0)
    assert np.minimum(*(fisher_err_per_event(Fk, x) for x in Fo)).max() < F_TOL
    assert np.minimum(*(snr_err_per_event(snr, x) for x in so)).max() < SNR_TOL
    cov, eps, cond = fisherTools.CovMatr(F, return_cond=True)
    assert cov.shape == (13, 13, 5)
    covo, _ = O.cov_matr_fast(Fk)
    s = np.sqrt(np.einsum('iin->ni', cov))
    so_ = np.sqrt(np.einsum('nii->ni', covo))
    err = (np.abs(s - so_) / so_).max(axis=1)
    assert np.all(err < np.maximum(1e-9, 1e-14 * cond)), (err, cond)
    ev2 = {k: v for k, v in ev.items() if k not in ('Lambda1', 'Lambda2')}
    ev2['LambdaTilde'], ev2['deltaLambda'] = evd['LambdaTilde'], evd['deltaLambda']
    F2 = net.FisherMatr(dict(ev2), res=res)
    d = np.sqrt(np.einsum('iin->in', F))
    # the grid end comes from Lambda1, Lambda2 either way (converted on the GPU from the pair given)
    assert (np.abs(F2 - F) / (d[:, None] * d[None, :])).max() < 1e-12


def test_nrtidal_fp32_is_rejected(gpu_lib):
    ev = nrt_events(2, seed=3)
    net = synthetic.make_network(W.IMRPhenomD_NRTidalv2(), dets=(('L1', 10.),), earth=False)
    with pytest.raises(_lib.GWFError):
        net.FisherMatr(dict(ev), res=100, precision='fp32')


def test_kat_gw170817(gpu_lib):
    """gwfast's GW170817 example: IMRPhenomD_NRTidalv2, L1 + H1 + Virgo with the O2 ASD tables, fmin
    10 Hz, no Earth rotation, default resolution: network SNR 33.16 and, with deltaLambda fixed, a
    90 % sky area of 19.9 deg^2. The SNRs are compared with gwfast's own to 1e-6 (the last-point
    taper, 0 or 1 by rounding, is worth ~1e-7 of the SNR), the Fisher matrix with the oracle."""
    from gwfast_gb300 import gwfastGlobals as glob
    from gwfast_gb300.network import DetNet
    from gwfast_gb300.signal import GWSignal
    from test_oracle_golden import gw170817
    g, ev, tabs = gw170817()
    sigs = {}
    for d, (f, asd) in tabs.items():
        c = glob.detectors[d]
        sigs[d] = GWSignal(W.IMRPhenomD_NRTidalv2(), psd_path=(f, asd), detector_shape=c['shape'], det_lat=c['lat'],
                           det_long=c['long'], det_xax=c['xax'], verbose=False, is_ASD=True, useEarthMotion=False,
                           fmin=10.)
    net = DetNet(sigs, verbose=False)
    snrs = net.SNR(dict(ev), return_all=True)
    for d in tabs:
        assert abs(snrs[d][0] - g['snr_' + d][0]) < 1e-6 * g['snr_' + d][0], d
    snr = net.SNR(dict(ev))
    assert abs(snr[0] - g['snr_net'][0]) < 1e-6 * snr[0]
    assert round(float(snr[0]), 2) == 33.16
    evd = dict(ev)
    F = net.FisherMatr(evd)
    assert F.shape == (13, 13, 1)
    p = O.to_params(evd, O.PARAMS_TIDAL)
    dets = [O.Detector(*O.DETECTORS[d][:3], O.DETECTORS[d][3], fmin=10., psd_f=f, psd_S=asd * asd, earth=False)
            for d, (f, asd) in tabs.items()]
    Fo = oracle_both(lambda m: sum(O.fisher(det, m, p, 1000) for det in dets).numpy())
    assert np.minimum(*(fisher_err_per_event(np.moveaxis(F, -1, 0), x) for x in Fo)).max() < F_TOL
    Ff, pf = fisherTools.fixParams(F, W.IMRPhenomD_NRTidalv2().ParNums, ['deltaLambda'])
    cov, _ = fisherTools.CovMatr(Ff)
    area = fisherTools.compute_localization_region(cov, pf, ev['theta'])
    assert abs(area[0] - g['sky_area'][0]) < 2e-3 * g['sky_area'][0]
    assert round(float(area[0]), 1) == 19.9
