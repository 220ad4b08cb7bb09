"""FP32 split-precision Fisher against the FP64 kernel (and so against the oracle).

Error measures: Fisher entries relative to sqrt(F_aa F_bb), and the marginalised 1-sigma
errors sqrt(diag(Cov)) from the FP64 equilibrated-Cholesky inversion of each.
"""
import numpy as np
import pytest

from gwfast_gb300 import fisherTools, synthetic
from gwfast_gb300 import waveforms as W

pytestmark = pytest.mark.gpu


def entry_err(F, Fr):
    d = np.sqrt(np.abs(np.einsum('nii->ni', Fr)))
    return np.abs(F - Fr) / (d[:, :, None] * d[:, None, :])


def sigma_err(F32, F64):
    c32, _, _ = fisherTools.CovMatr(np.moveaxis(F32, 0, -1), return_cond=True)
    c64, _, cond = fisherTools.CovMatr(np.moveaxis(F64, 0, -1), return_cond=True)
    s32 = np.sqrt(np.einsum('iin->ni', c32))
    s64 = np.sqrt(np.einsum('iin->ni', c64))
    return np.abs(s32 - s64) / s64, cond


@pytest.mark.parametrize('earth', [True, False])
def test_phenomd_network_fp32(gpu_lib, earth):
    ev = synthetic.bbh_events(512, seed=1001)
    net = synthetic.make_network(W.IMRPhenomD(), earth=earth)
    F64 = np.moveaxis(net.FisherMatr(dict(ev), res=2000), -1, 0)
    F32 = np.moveaxis(net.FisherMatr(dict(ev), res=2000, precision='fp32'), -1, 0)
    e = entry_err(F32, F64)
    se, cond = sigma_err(F32, F64)
    worst = se.max(axis=1)
    print('PhenomD fp32 entry err max %.2e median %.2e; sigma err median %.2e p95 %.2e max %.2e; frac<=1e-3 %.4f'
          % (e.max(), np.median(e.max(axis=(1, 2))), np.median(worst), np.percentile(worst, 95), worst.max(),
             np.mean(worst <= 1e-3)))
    assert np.median(e.max(axis=(1, 2))) < 1e-5
    assert np.mean(worst <= 1e-3) >= 0.95


@pytest.mark.parametrize('det,cond_ok', [(('Virgo', 10.), 1e12), (('ETS', 5.), 1e13)])
def test_taylorf2_fp32(gpu_lib, det, cond_ok):
    """TaylorF2 BNS on one detector with Earth rotation, FP32 against FP64.

    A single detector measures the sky position and polarisation only through the Earth-rotation
    modulation of its pattern functions, so the 11-parameter Fisher matrices of one L-shaped detector
    have equilibrated condition numbers from 3e10 up to 2e17. Above ~1e16 they are numerically
    singular in float64: the FP64 inversion itself gives a non-positive variance there, so sigma is
    NaN in either precision (8 of these 256 events on Virgo). Those NaN sigmas are counted and must all
    come from such matrices. The FP32 sigma errors grow with the condition number: within 1e-3 below
    cond 1e12 on one L (7.2e-4 measured; up to 3.5e-3 between 1e12 and 1e13, so single L-shaped
    detectors need the FP64 recomputation threshold at 1e12 or lower) and below 1e13 on the triangle
    (2.9e-4 measured)."""
    ev = synthetic.bns_events(256, seed=1000)
    net = synthetic.make_network(W.TaylorF2_RestrictedPN(), dets=(det,), earth=True)
    F64 = np.moveaxis(net.FisherMatr(dict(ev), res=2000), -1, 0)
    F32 = np.moveaxis(net.FisherMatr(dict(ev), res=2000, precision='fp32'), -1, 0)
    e = entry_err(F32, F64)
    c32, _, _ = fisherTools.CovMatr(np.moveaxis(F32, 0, -1), return_cond=True)
    c64, _, cond = fisherTools.CovMatr(np.moveaxis(F64, 0, -1), return_cond=True)
    v32, v64 = np.einsum('iin->ni', c32), np.einsum('iin->ni', c64)
    nan32, nan64 = np.any(~(v32 > 0), axis=1), np.any(~(v64 > 0), axis=1)
    worst = (np.abs(np.sqrt(np.abs(v32)) - np.sqrt(np.abs(v64))) / np.sqrt(np.abs(v64))).max(axis=1)
    ok = (cond < cond_ok) & ~nan32 & ~nan64
    print('TF2 %s fp32 entry err max %.2e; NaN sigma: %d (fp64) %d (fp32), smallest cond of those %.2e; '
          'sigma err below cond %.0e (%d events): median %.2e max %.2e'
          % (det[0], e.max(), nan64.sum(), nan32.sum(), cond[nan32 | nan64].min() if (nan32 | nan64).any() else np.nan,
             cond_ok, ok.sum(), np.median(worst[ok]), worst[ok].max()))
    assert np.median(e.max(axis=(1, 2))) < 1e-5
    assert np.all(cond[nan32 | nan64] > 1e15)
    assert ok.sum() >= 10
    assert worst[ok].max() <= 1e-3


def test_fp32_per_arm_sums_to_total(gpu_lib):
    ev = synthetic.bbh_events(32, seed=17)
    net = synthetic.make_network(W.IMRPhenomD(), dets=(('ETS', 5.),), earth=True)
    Fa = net.FisherMatr(dict(ev), res=1000, return_all=True, precision='fp32')
    Ft = net.FisherMatr(dict(ev), res=1000, precision='fp32')
    S = Fa['ETS_0'] + Fa['ETS_1'] + Fa['ETS_2']
    assert entry_err(np.moveaxis(Ft, -1, 0), np.moveaxis(S, -1, 0)).max() < 1e-5


def hm_events(n, seed):
    """IMRPhenomHM catalogue distributions: m1 power law on [5, 150], q ~ U[0.1, 1], chi ~ U[-0.9, 0.9]."""
    return synthetic.bbh_events(n, seed=seed, mmax=150., qmin=0.1, chimax=0.9, dl=(0.5, 20.))


@pytest.mark.parametrize('earth', [True, False])
def test_phenomhm_network_fp32(gpu_lib, earth):
    """IMRPhenomHM split precision (FP64 mode phases, FP32 amplitudes, tangents and mode sums)."""
    ev = hm_events(256, seed=1003)
    net = synthetic.make_network(W.IMRPhenomHM(), dets=synthetic.NETWORK_ET_CE, earth=earth)
    F64 = np.moveaxis(net.FisherMatr(dict(ev), res=1000), -1, 0)
    F32 = np.moveaxis(net.FisherMatr(dict(ev), res=1000, precision='fp32'), -1, 0)
    e = entry_err(F32, F64)
    se, cond = sigma_err(F32, F64)
    worst = se.max(axis=1)
    ok = cond < 1e12
    print('PhenomHM fp32 entry err max %.2e median %.2e; sigma err median %.2e p95 %.2e max %.2e; frac<=1e-3 %.4f;'
          ' cond<1e12: %d events, max %.2e'
          % (e.max(), np.median(e.max(axis=(1, 2))), np.median(worst), np.percentile(worst, 95), worst.max(),
             np.mean(worst <= 1e-3), ok.sum(), worst[ok].max()))
    assert np.median(e.max(axis=(1, 2))) < 1e-4
    assert np.mean(worst <= 1e-3) >= 0.95


def test_phenomhm_mixed(gpu_lib):
    """IMRPhenomHM mixed form: sigma within 1e-3 of the FP64 kernel on every event with cond < 1e13."""
    ev = hm_events(256, seed=1004)
    net = synthetic.make_network(W.IMRPhenomHM(), dets=synthetic.NETWORK_ET_CE, earth=True)
    F64 = np.moveaxis(net.FisherMatr(dict(ev), res=1000), -1, 0)
    Fm = np.moveaxis(net.FisherMatr(dict(ev), res=1000, precision='mixed', refine_cond=1e11), -1, 0)
    se, cond = sigma_err(Fm, F64)
    worst = se.max(axis=1)
    ok = cond < 1e13
    print('PhenomHM mixed: sigma err median %.2e max (cond<1e13, %d events) %.2e'
          % (np.median(worst), ok.sum(), worst[ok].max()))
    assert worst[ok].max() <= 1e-3


@pytest.mark.parametrize('earth', [True, False])
def test_phenomhm_snr_fp32(gpu_lib, earth):
    """IMRPhenomHM FP32 SNR (mode phases in FP64 reduced modulo 2 pi, amplitudes, mode sums, pattern
    functions in FP32) against the FP64 SNR kernel on the ET + CE1Id + CE2NM events at R = 4000:
    network SNR within 2e-6, single arms within 1e-5 (their pattern functions can nearly vanish).
    Typical errors are ~1e-7 (standard deviation 1.2e-7 over these events); the largest, 1.2e-6, come
    from the lightest and most asymmetric systems of the catalogue (total mass 6-10 Msun, q ~ 0.1),
    against 2e-7 for IMRPhenomD on the same network. The FP64 SNR is the drop-in."""
    ev = hm_events(512, seed=1005)
    net = synthetic.make_network(W.IMRPhenomHM(), dets=synthetic.NETWORK_ET_CE, earth=earth)
    s64 = net.SNR(dict(ev), res=4000, return_all=True)
    s32 = net.SNR(dict(ev), res=4000, return_all=True, precision='fp32')
    worst_net = np.max(np.abs(s32['net'] - s64['net']) / s64['net'])
    worst_arm = max(np.max(np.abs(s32[k] - s64[k]) / s64[k]) for k in s64)
    print('PhenomHM fp32 SNR max rel err: network %.2e, single arms %.2e' % (worst_net, worst_arm))
    assert worst_net <= 2e-6
    assert worst_arm <= 1e-5


def test_phenomd_network_mixed(gpu_lib):
    """FP32 form plus FP64 for events above the condition-number threshold: sigma within 1e-3."""
    ev = synthetic.bbh_events(512, seed=1001)
    net = synthetic.make_network(W.IMRPhenomD(), earth=True)
    F64 = np.moveaxis(net.FisherMatr(dict(ev), res=2000), -1, 0)
    Fm = np.moveaxis(net.FisherMatr(dict(ev), res=2000, precision="mixed", refine_cond=3e11), -1, 0)
    se, cond = sigma_err(Fm, F64)
    worst = se.max(axis=1)
    exact = entry_err(Fm, F64).max(axis=(1, 2)) < 1e-11   # recomputed in FP64 (segmented: rounding-level)
    print('PhenomD mixed: FP64 events %.3f, cond of those >= %.2e; sigma err median %.2e max %.2e; frac<=1e-3 %.4f'
          % (exact.mean(), cond[exact].min() if exact.any() else np.nan, np.median(worst), worst.max(),
             np.mean(worst <= 1e-3)))
    # every event clearly above the threshold went to FP64 (the library estimates the condition
    # number by power and inverse iteration; 5 % slack around the threshold)
    assert np.all(cond[~exact] <= 3e11 * 1.05)
    assert np.all(cond[exact] >= 3e11 / 1.05)
    assert np.mean(worst <= 1e-3) >= 0.998


def test_mixed_all_refined_is_fp64(gpu_lib):
    """With a threshold below every condition number, the mixed form returns the FP64 matrices
    (gather, FP64 recomputation in frequency segments and scatter of every event), per arm as well;
    the segment sums differ from the per-event kernel only in summation order."""
    ev = synthetic.bbh_events(200, seed=5)
    net = synthetic.make_network(W.IMRPhenomD(), earth=True)
    F64 = net.FisherMatr(dict(ev), res=1000, return_all=True)
    Fm = net.FisherMatr(dict(ev), res=1000, return_all=True, precision='mixed', refine_cond=1.0)
    for k in F64:
        assert entry_err(np.moveaxis(Fm[k], -1, 0), np.moveaxis(F64[k], -1, 0)).max() < 1e-12, k


@pytest.mark.parametrize('model,dets,maker', [
    ('IMRPhenomD', synthetic.NETWORK_LHET, synthetic.bbh_events),
    ('TaylorF2_RestrictedPN', (('L1', 10.), ('H1', 10.), ('Virgo', 10.), ('ETS', 5.)), synthetic.bns_events)])
def test_mixed_all_refined_grouped_network(gpu_lib, model, dets, maker):
    """Network total only, so the detectors that share a grid run as one group (ETS beside them):
    with every event refined, the FP64 stage starts from the FP64 set-up records that the FP32 pass
    left in its scratch, and the result equals the FP64 kernel's up to summation order."""
    ev = maker(300, seed=9)
    net = synthetic.make_network(getattr(W, model)(), dets=dets, earth=True)
    F64 = np.moveaxis(net.FisherMatr(dict(ev), res=1000), -1, 0)
    Fm = np.moveaxis(net.FisherMatr(dict(ev), res=1000, precision='mixed', refine_cond=1.0), -1, 0)
    assert entry_err(Fm, F64).max() < 1e-12


def test_mixed_condition_estimate(gpu_lib):
    """The mixed form's condition-number estimate against the covariance kernel's (Jacobi) one."""
    ev = synthetic.bbh_events(400, seed=77)
    net = synthetic.make_network(W.IMRPhenomD(), earth=True)
    F = np.ascontiguousarray(np.moveaxis(net.FisherMatr(dict(ev), res=1000), -1, 0))
    _, _, cond = fisherTools.CovMatr(np.moveaxis(F, 0, -1), return_cond=True)
    for kappa in np.percentile(cond, [10, 50, 90]):
        # every event whose mixed result is FP64 had an estimated condition number above kappa; the
        # estimate (a few power and inverse iterations) never overestimates by more than ~5 % and
        # may underestimate by up to ~35 % when the two smallest eigenvalues are close
        Fm = np.moveaxis(net.FisherMatr(dict(ev), res=1000, precision='mixed', refine_cond=kappa), -1, 0)
        refined = entry_err(Fm, F).max(axis=(1, 2)) < 1e-11
        assert np.all(cond[refined] >= kappa / 1.1)
        assert np.all(cond[~refined] <= kappa * 1.6)


@pytest.mark.parametrize('model,dets,maker', [
    ('IMRPhenomD', synthetic.NETWORK_LHET, synthetic.bbh_events),
    ('TaylorF2_RestrictedPN', (('ETS', 5.), ('Virgo', 10.)), synthetic.bns_events)])
def test_snr_fp32(gpu_lib, model, dets, maker):
    """FP32 SNR kernel against the FP64 one: network SNR relative error <= 1e-6; single arms (whose
    pattern functions can nearly vanish, so their FP32 values lose relative accuracy) <= 1e-5."""
    ev = maker(512, seed=71)
    net = synthetic.make_network(getattr(W, model)(), dets=dets, earth=True)
    s64 = net.SNR(dict(ev), res=2000, return_all=True)
    s32 = net.SNR(dict(ev), res=2000, return_all=True, precision='fp32')
    worst_net = np.max(np.abs(s32['net'] - s64['net']) / s64['net'])
    worst_arm = max(np.max(np.abs(s32[k] - s64[k]) / s64[k]) for k in s64)
    print('%s fp32 SNR max rel err: network %.2e, single arms %.2e' % (model, worst_net, worst_arm))
    assert worst_net <= 1e-6
    assert worst_arm <= 1e-5


@pytest.mark.parametrize('model,dets,maker', [
    ('IMRPhenomD', synthetic.NETWORK_LHET, lambda n: synthetic.bbh_events(n, seed=5)),
    ('IMRPhenomHM', synthetic.NETWORK_ET_CE, lambda n: hm_events(n, seed=6)),
    ('TaylorF2_RestrictedPN', (('L1', 10.), ('Virgo', 10.), ('ETS', 10.)), lambda n: synthetic.bns_events(n, seed=7))])
def test_detector_groups(gpu_lib, model, dets, maker):
    """FP32 network total with the detectors that share the grid in one launch (the waveform once per
    point) against one launch per detector: the same Gram up to the fixed-point quantisation grid."""
    from gwfast_gb300 import _lib
    ev = maker(128)
    wf = getattr(W, model)()
    net = synthetic.make_network(wf, dets=dets, earth=True)
    ctx = _lib.context(0)
    res = 1000
    try:
        ctx.set_detector_groups(False)
        Fs = np.moveaxis(net.FisherMatr(dict(ev), res=res, precision='fp32'), -1, 0)
        ctx.set_detector_groups(True)
        Fg = np.moveaxis(net.FisherMatr(dict(ev), res=res, precision='fp32'), -1, 0)
    finally:
        ctx.set_detector_groups(True)
    F64 = np.moveaxis(net.FisherMatr(dict(ev), res=res), -1, 0)
    e = entry_err(Fg, Fs)
    sg, _ = sigma_err(Fg, F64)
    ss, _ = sigma_err(Fs, F64)
    print('%s groups vs per detector: entry err max %.2e; sigma err vs fp64 median %.2e (grouped) %.2e (per detector)'
          % (model, e.max(), np.median(sg.max(axis=1)), np.median(ss.max(axis=1))))
    assert e.max() < 1e-5
    assert np.median(sg.max(axis=1)) < 3 * np.median(ss.max(axis=1)) + 1e-6


def test_detector_groups_distinct_psds(gpu_lib):
    """A group of four detectors on one grid whose PSD tables differ: L1 and H1 share the aLIGO table
    (H1 reuses L1's per-point weight), Virgo has a reshaped one (another normalisation scale, so the
    group's common Gram scale differs per detector), KAGRA has L1's table again but follows Virgo
    (its own lookup). FP32 grouped launch against one launch per detector, and both against FP64."""
    from gwfast_gb300 import _lib
    from gwfast_gb300.network import DetNet
    from gwfast_gb300.signal import GWSignal
    ev = synthetic.bbh_events(128, seed=5)
    wf = W.IMRPhenomD()
    sigs = {}
    for name in ('L1', 'H1', 'Virgo', 'KAGRA'):
        spec = synthetic.detector_spec(name, 10.)
        f, S = spec['psd_path']
        if name == 'Virgo':
            spec['psd_path'] = (f, 3.0 * S * (1.0 + (f / 150.0) ** 2))
        sigs[name] = GWSignal(wf, useEarthMotion=True, verbose=False, **spec)
    net = DetNet(sigs, verbose=False)
    ctx = _lib.context(0)
    try:
        ctx.set_detector_groups(False)
        Fs = np.moveaxis(net.FisherMatr(dict(ev), res=1000, precision='fp32'), -1, 0)
        ctx.set_detector_groups(True)
        Fg = np.moveaxis(net.FisherMatr(dict(ev), res=1000, precision='fp32'), -1, 0)
    finally:
        ctx.set_detector_groups(True)
    F64 = np.moveaxis(net.FisherMatr(dict(ev), res=1000), -1, 0)
    e = entry_err(Fg, Fs)
    e64 = entry_err(Fg, F64)
    sg, _ = sigma_err(Fg, F64)
    ss, _ = sigma_err(Fs, F64)
    print('distinct PSDs in one group: grouped vs per detector entry err max %.2e, vs fp64 %.2e; sigma err median '
          '%.2e (grouped) %.2e (per detector)' % (e.max(), e64.max(), np.median(sg.max(axis=1)), np.median(ss.max(axis=1))))
    assert e.max() < 1e-5
    assert np.median(e64.max(axis=(1, 2))) < 1e-5
    assert np.median(sg.max(axis=1)) < 3 * np.median(ss.max(axis=1)) + 1e-6


@pytest.mark.parametrize('model,dets,maker', [
    ('IMRPhenomD', synthetic.NETWORK_LHET, synthetic.bbh_events),
    ('IMRPhenomD', (('ETS', 10.), ('L1', 10.), ('H1', 10.)), synthetic.bbh_events),
    ('IMRPhenomHM', (('L1', 10.), ('H1', 10.), ('Virgo', 10.)), synthetic.bbh_events),
    ('IMRPhenomHM', synthetic.NETWORK_ET_CE, synthetic.bbh_events),
    ('TaylorF2_RestrictedPN', (('L1', 10.), ('Virgo', 10.)), synthetic.bns_events)])
def test_fp64_detector_groups(gpu_lib, model, dets, maker):
    """FP64 network total with the detectors that share the grid in one launch (the waveform and its
    tangent once per point; a triangle among them contributes its two combined vectors) against one
    launch per detector: the same sums in another order."""
    from gwfast_gb300 import _lib
    ev = maker(64, seed=17)
    net = synthetic.make_network(getattr(W, model)(), dets=dets, earth=True)
    ctx = _lib.context(0)
    try:
        ctx.set_detector_groups(False)
        Fs = np.moveaxis(net.FisherMatr(dict(ev), res=600), -1, 0)
        ctx.set_detector_groups(True)
        Fg = np.moveaxis(net.FisherMatr(dict(ev), res=600), -1, 0)
    finally:
        ctx.set_detector_groups(True)
    e = entry_err(Fg, Fs).max()
    print('%s FP64 groups vs per detector: max normalised |dF| %.2e' % (model, e))
    assert e < 1e-12


@pytest.mark.parametrize('model,dets', [
    ('IMRPhenomD', (('L1', 10.), ('ETS', 5.), ('H1', 10.))),
    ('IMRPhenomD', (('ETS', 10.), ('L1', 10.), ('Virgo', 10.))),
    ('IMRPhenomHM', synthetic.NETWORK_ET_CE)])
@pytest.mark.parametrize('precision,tol', [('fp64', 1e-12), ('fp32', 1e-6)])
def test_snr_groups(gpu_lib, model, dets, precision, tol):
    """SNRs with the detectors that share the grid in one launch (the waveform value once per point)
    against one launch per detector, every arm and the network (FP64: the same sums in another order;
    FP32: the same Kahan sums, each detector's scale formed from detector 0's). The first network
    launches its L1 + H1 group before the triangle between them, so the per-arm slots are checked
    against the detectors' order."""
    from gwfast_gb300 import _lib
    ev = synthetic.bbh_events(64, seed=19)
    net = synthetic.make_network(getattr(W, model)(), dets=dets, earth=True)
    ctx = _lib.context(0)
    try:
        ctx.set_detector_groups(False)
        s1 = net.SNR(dict(ev), res=600, return_all=True, precision=precision)
        ctx.set_detector_groups(True)
        sg = net.SNR(dict(ev), res=600, return_all=True, precision=precision)
    finally:
        ctx.set_detector_groups(True)
    worst = max(np.max(np.abs(np.asarray(sg[k]) - np.asarray(s1[k])) / np.asarray(s1[k])) for k in s1)
    print('%s %s SNR groups vs per detector (%s): max rel diff %.2e' % (model, precision, ', '.join(s1), worst))
    assert worst < tol
