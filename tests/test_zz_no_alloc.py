"""gwf_fisher_noalloc (the Fisher entry point that allocates no device memory) against gwf_fisher.

Callers whose device memory belongs to their own pool allocator, or whose loops cannot take the
device synchronisation of cudaMalloc/cudaFree, use this entry point: its scratch is one fixed
__device__ array in the library, shared by all calls. The GPU tests therefore make calls in a row
with different models, detectors and event sets (IMRPhenomD, TaylorF2 and IMRPhenomHM), a batch
larger than one pass of the scratch, and a two-detector network summed with accumulate=1: each
must match the context-based entry point on the same inputs.
"""
import ctypes

import numpy as np
import pytest

from gwfast_gb300 import _lib, synthetic, waveforms as W
from gwfast_gb300 import gwfastGlobals as glob
from gwfast_gb300.psd import aligo_table
from gwfast_gb300.signal import event_array

TOL = 1e-9   # |dF_ab| <= TOL sqrt(F_aa F_bb), the FP64 Fisher parity tolerance


def _det(name, fmin, earth):
    d = glob.detectors[name]
    return _lib.DetDesc(np.deg2rad(d['lat']), np.deg2rad(d['long']), np.deg2rad(d['xax']),
                        0 if d['shape'] == 'L' else 1, int(earth), float(fmin), -1.0)


def _noalloc(lib, det, f, S, wf, q, params, n, out, accumulate=0, stream=None):
    return lib.gwf_fisher_noalloc(ctypes.byref(det), _lib.ptr(f), _lib.ptr(S), len(f), ctypes.byref(wf),
                                  _lib.ptr(q[0]), _lib.ptr(q[1]), _lib.ptr(q[2]), q.shape[1], _lib.ptr(params),
                                  n, n, 2000, accumulate, _lib.ptr(out), stream)


def test_noalloc_rejects_oversized_tables():
    """Sizes beyond the stated maxima fail with a clear error before any device work."""
    lib = _lib.load()
    f, S = aligo_table(5., rows=20000)
    q = _lib._qnm_table()
    wf = W.IMRPhenomD().gpu_desc()
    rc = _noalloc(lib, _det('ETS', 5., True), f, S, wf, q, None, 0, None)
    assert rc == -1
    assert b'GWF_NOALLOC_MAX_PSD' in lib.gwf_last_error()


@pytest.mark.gpu
def test_noalloc_matches_fisher_calls_in_a_row():
    torch = pytest.importorskip('torch')
    assert torch.cuda.is_available()
    lib = _lib.load()
    ctx = _lib.Context(0)
    q = _lib._qnm_table()
    cases = [  # (model, detector, wall, Earth rotation, events, seed)
        (W.IMRPhenomD(), 'ETS', 5., True, 300, 11),
        (W.TaylorF2_RestrictedPN(), 'L1', 10., False, 200, 12),
        (W.IMRPhenomHM(), 'ETS', 5., True, 150, 14),
        (W.IMRPhenomD(), 'H1', 10., True, 257, 13),
    ]
    stream = torch.cuda.Stream()
    for model, name, wall, earth, n, seed in cases:
        f, S = aligo_table(wall, rows=8000)
        det = _det(name, wall, earth)
        d = glob.detectors[name]
        det_id = ctx.add_detector(det.lat_rad, det.long_rad, det.xax_rad, d['shape'], earth, wall, None, f, S)
        ev = synthetic.bbh_events(n, seed=seed)
        params = torch.from_numpy(event_array(ev)).cuda()
        ref = torch.empty((n, 11, 11), dtype=torch.float64, device='cuda')
        out = torch.full((n, 11, 11), float('nan'), dtype=torch.float64, device='cuda')
        wf = model.gpu_desc()
        with torch.cuda.stream(stream):
            ctx.fisher([det_id], wf, params, 2000, mem=_lib.MEM_DEVICE, out_net=ref, stream=stream.cuda_stream,
                       ld=n, n=n)
            rc = _noalloc(lib, det, f, S, wf, q, params, n, out, stream=stream.cuda_stream)
        assert rc == 0, lib.gwf_last_error()
        stream.synchronize()
        R, O = ref.cpu().numpy(), out.cpu().numpy()
        dg = np.sqrt(np.abs(np.einsum('nii->ni', R)))
        err = np.abs(O - R) / (dg[:, :, None] * dg[:, None, :])
        print('%s %s: max normalised |dF| %.2e' % (type(model).__name__, name, err.max()))
        assert np.all(np.isfinite(O))
        assert err.max() <= TOL


def _compare(ref, out):
    R, O = ref.cpu().numpy(), out.cpu().numpy()
    dg = np.sqrt(np.abs(np.einsum('nii->ni', R)))
    err = np.abs(O - R) / (dg[:, :, None] * dg[:, None, :])
    assert np.all(np.isfinite(O))
    return err.max()


@pytest.mark.gpu
def test_noalloc_multiple_passes_and_network_accumulate():
    """7000 IMRPhenomD events need two passes of the scratch (6869 events per pass): the second
    pass reads params + 6869 with the same leading dimension and writes out + 6869 matrices. Then a
    two-detector network summed by two calls (accumulate=0, then 1) against gwf_fisher's network
    total over the same detectors."""
    torch = pytest.importorskip('torch')
    assert torch.cuda.is_available()
    lib = _lib.load()
    ctx = _lib.Context(0)
    q = _lib._qnm_table()
    stream = torch.cuda.Stream()
    wf = W.IMRPhenomD().gpu_desc()
    f, S = aligo_table(10., rows=8000)
    dets, ids = [], []
    for name in ('L1', 'H1'):
        det = _det(name, 10., True)
        dets.append(det)
        ids.append(ctx.add_detector(det.lat_rad, det.long_rad, det.xax_rad, 'L', True, 10., None, f, S))
    n = 7000
    params = torch.from_numpy(event_array(synthetic.bbh_events(n, seed=21))).cuda()
    ref = torch.empty((n, 11, 11), dtype=torch.float64, device='cuda')
    out = torch.full((n, 11, 11), float('nan'), dtype=torch.float64, device='cuda')
    with torch.cuda.stream(stream):
        ctx.fisher([ids[0]], wf, params, 2000, mem=_lib.MEM_DEVICE, out_net=ref, stream=stream.cuda_stream, ld=n, n=n)
        rc = _noalloc(lib, dets[0], f, S, wf, q, params, n, out, stream=stream.cuda_stream)
    assert rc == 0, lib.gwf_last_error()
    stream.synchronize()
    e1 = _compare(ref, out)
    print('two passes, %d events: max normalised |dF| %.2e' % (n, e1))
    assert e1 <= TOL

    m = 600
    params = torch.from_numpy(event_array(synthetic.bbh_events(m, seed=22))).cuda()
    ref = torch.empty((m, 11, 11), dtype=torch.float64, device='cuda')
    out = torch.full((m, 11, 11), float('nan'), dtype=torch.float64, device='cuda')
    with torch.cuda.stream(stream):
        ctx.fisher(ids, wf, params, 2000, mem=_lib.MEM_DEVICE, out_net=ref, stream=stream.cuda_stream, ld=m, n=m)
        rc = _noalloc(lib, dets[0], f, S, wf, q, params, m, out, accumulate=0, stream=stream.cuda_stream)
        assert rc == 0, lib.gwf_last_error()
        rc = _noalloc(lib, dets[1], f, S, wf, q, params, m, out, accumulate=1, stream=stream.cuda_stream)
    assert rc == 0, lib.gwf_last_error()
    stream.synchronize()
    e2 = _compare(ref, out)
    print('L1 + H1 network by accumulation: max normalised |dF| %.2e' % e2)
    assert e2 <= TOL
