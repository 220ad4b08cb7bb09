"""Batch forecast pipeline (SNR -> threshold -> Fisher -> covariance -> errors, sky areas)."""
import numpy as np
import pytest

from gwfast_gb300 import fisherTools, pipeline, synthetic
from gwfast_gb300 import waveforms as W

pytestmark = pytest.mark.gpu


def test_compute_errs_forms_agree(gpu_lib):
    ev = synthetic.bbh_events(400, seed=81)
    ev['dL'] = ev['dL'] * 3.0          # push part of the catalogue below threshold
    net = synthetic.make_network(W.IMRPhenomD(), earth=True)
    r64 = pipeline.compute_errs(net, dict(ev), snr_th=12., res=2000, precision='fp64', snr_precision='fp64')
    rm = pipeline.compute_errs(net, dict(ev), snr_th=12., res=2000, precision='mixed', snr_precision='fp32')
    assert 0 < r64['detected'].sum() < len(r64['detected'])
    assert np.array_equal(r64['detected'], rm['detected'])
    assert np.max(np.abs(rm['snr'] - r64['snr']) / r64['snr']) < 1e-6
    ok = r64['cond'] < 1e13
    e = np.max(np.abs(rm['errors'] - r64['errors']) / r64['errors'], axis=0)
    print('detected %d of %d; mixed vs fp64 sigma err median %.2e max %.2e (cond < 1e13)'
          % (r64['detected'].sum(), len(r64['detected']), np.median(e[ok]), e[ok].max()))
    assert np.all(e[ok] <= 1e-3)
    a = r64['sky_area_90']
    assert np.all(np.isfinite(a[ok])) and np.all(a[ok] > 0)
    # the sky area is the one of the returned covariance
    ref = fisherTools.compute_localization_region(r64['cov'], r64['par_nums'], ev['theta'][r64['detected']])
    assert np.allclose(a, ref, equal_nan=True)


def test_compute_errs_fixed_params(gpu_lib):
    ev = synthetic.bbh_events(64, seed=82)
    net = synthetic.make_network(W.IMRPhenomD(), earth=True)
    full = pipeline.compute_errs(net, dict(ev), snr_th=0., res=1000, precision='fp64', snr_precision='fp64')
    fx = pipeline.compute_errs(net, dict(ev), snr_th=0., res=1000, precision='fp64', snr_precision='fp64',
                               params_fix=('psi', 'Phicoal'))
    assert fx['cov'].shape == (9, 9, 64)
    keep = [0, 1, 2, 3, 4, 5, 7, 9, 10]
    # reference: numpy's inverse of the reduced Fisher with its diagonal scaled out first (the raw 9x9
    # matrices reach condition numbers near 1e15, their equilibrated forms 1e11, and the unscaled
    # inverse then differs from either by ~1e-6 from rounding alone)
    F = np.moveaxis(full['fisher'][np.ix_(keep, keep)], -1, 0)
    d = 1.0 / np.sqrt(np.einsum('nii->ni', F))
    C = d[:, :, None] * np.linalg.inv(d[:, :, None] * F * d[:, None, :]) * d[:, None, :]
    ok = full['cond'] < 1e12
    rel = np.abs(np.sqrt(np.einsum('nii->in', C)) - fx['errors']) / fx['errors']
    assert np.max(rel[:, ok]) < 1e-6


def test_run_catalogue_batches_and_resume(gpu_lib, tmp_path, monkeypatch):
    """The driver loop: batches written under gwfast's file names, results equal to one compute_errs
    over the whole catalogue, and a resumed run recomputes only the batch whose files are missing."""
    ev = synthetic.bbh_events(300, seed=83)
    ev['dL'] = ev['dL'] * 1.5          # part of the catalogue below threshold
    net = synthetic.make_network(W.IMRPhenomD(), earth=True)
    kw = dict(snr_th=12., res=1000, precision='fp64', snr_precision='fp64')
    whole = pipeline.compute_errs(net, dict(ev), check_fisher=True, **kw)
    assert 0 < whole['detected'].sum() < 300
    tot = pipeline.run_catalogue(net, dict(ev), str(tmp_path), batch_size=128, **kw)
    names = sorted(p.name for p in tmp_path.iterdir())
    for a, b in ((0, 128), (128, 256), (256, 300)):
        assert 'snrs_%d_to_%d.txt' % (a, b) in names
        assert ('fishers_%d_to_%d.npy' % (a, b) in names) == bool(whole['detected'][a:b].any())
    assert np.allclose(tot['snrs'], whole['snr'], rtol=1e-12)
    assert np.array_equal(tot['idxs_det'].astype(int), np.where(whole['detected'])[0])
    assert np.allclose(tot['fishers'], whole['fisher'], rtol=1e-12, atol=0)
    assert np.allclose(tot['cond_numbers'], whole['cond_numbers'], rtol=1e-6)
    ok = whole['cond'] < 1e12
    assert np.allclose(tot['errors'][:, ok], whole['errors'][:, ok], rtol=1e-9)
    for p in tmp_path.iterdir():
        if p.name.endswith('_128_to_256.txt') or p.name.endswith('_128_to_256.npy'):
            p.unlink()
    calls = []
    orig = pipeline.compute_errs

    def counting(*a, **k):
        calls.append(len(a[1]['Mc']))
        return orig(*a, **k)
    monkeypatch.setattr(pipeline, 'compute_errs', counting)
    tot2 = pipeline.run_catalogue(net, dict(ev), str(tmp_path), batch_size=128, **kw)
    assert calls == [128]
    assert np.allclose(tot2['fishers'], tot['fishers'], rtol=1e-12, atol=0)
