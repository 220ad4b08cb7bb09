"""Segmented persistent Fisher launches (work stealing over (event, frequency segment) items)
against the per-event launches, for uniform and per-event grid lengths, FP64 and FP32."""
import numpy as np
import pytest

from gwfast_gb300 import _lib, fisherTools, synthetic
from gwfast_gb300 import waveforms as W

pytestmark = pytest.mark.gpu


def norm_err(F, Fr):
    d = np.sqrt(np.abs(np.einsum('nii->ni', Fr)))
    return np.abs(F - Fr) / (d[:, :, None] * d[:, None, :])


def sigma_err(F, Fr, with_cond=False):
    c, _, _ = fisherTools.CovMatr(np.moveaxis(F, 0, -1), return_cond=True)
    cr, _, cond = fisherTools.CovMatr(np.moveaxis(Fr, 0, -1), return_cond=True)
    s, sr = np.sqrt(np.einsum('iin->ni', c)), np.sqrt(np.einsum('iin->ni', cr))
    e = (np.abs(s - sr) / sr).max(axis=1)
    return (e, cond) if with_cond else e


def run(net, ev, seg, **kw):
    ctx = _lib.context(0)
    ctx.set_segments(seg)
    try:
        return np.moveaxis(net.FisherMatr(dict(ev), **kw), -1, 0)
    finally:
        ctx.set_segments(0)


@pytest.mark.parametrize('seg', [128, 512, 2048])
def test_segments_fp64_uniform(gpu_lib, seg):
    ev = synthetic.bbh_events(300, seed=21)
    net = synthetic.make_network(W.IMRPhenomD(), earth=True)
    F0 = run(net, ev, 0, res=2000)
    F1 = run(net, ev, seg, res=2000)
    err = norm_err(F1, F0).max()
    print('seg %d fp64 max normalised diff %.2e' % (seg, err))
    assert err < 1e-12


def test_segments_fp64_per_event_res(gpu_lib):
    """Mixed BNS + BBH catalogue with per-event grid lengths (a few hundred to a few thousand)."""
    ev = synthetic.mixed_events(200, seed=31)
    res = synthetic.res_from_chirp_time(ev['Mc'], 2., lo=200, hi=4000)
    net = synthetic.make_network(W.IMRPhenomD(), dets=synthetic.NETWORK_LHET2, earth=True)
    F0 = run(net, ev, 0, res=int(res.max()), res_per_event=res)
    F1 = run(net, ev, 256, res=int(res.max()), res_per_event=res)
    err = norm_err(F1, F0).max()
    print('per-event res (%d..%d) fp64 max normalised diff %.2e' % (res.min(), res.max(), err))
    assert err < 1e-12
    # events of different lengths really differ from a uniform-length run
    F2 = run(net, ev, 0, res=int(res.max()))
    assert norm_err(F2, F0).max() > 1e-8


def test_segments_fp32_and_per_arm(gpu_lib):
    ev = synthetic.bbh_events(256, seed=41)
    net = synthetic.make_network(W.IMRPhenomD(), earth=True)
    F64 = run(net, ev, 0, res=2000)
    F32c = run(net, ev, 0, res=2000, precision='fp32')
    F32s = run(net, ev, 512, res=2000, precision='fp32')
    ec, es = sigma_err(F32c, F64), sigma_err(F32s, F64)
    print('fp32 sigma err vs fp64: per-event launch median %.2e max %.2e; segmented median %.2e max %.2e'
          % (np.median(ec), ec.max(), np.median(es), es.max()))
    assert np.median(es) < 1e-4 and np.mean(es <= 1e-3) >= 0.99
    assert norm_err(F32s, F32c).max() < 1e-5
    # per-arm output of the segmented path sums to its network total
    ctx = _lib.context(0)
    ctx.set_segments(512)
    try:
        Fa = net.FisherMatr(dict(ev), res=2000, return_all=True, precision='fp32')
    finally:
        ctx.set_segments(0)
    tot = sum(v for k, v in Fa.items() if k != 'net')
    assert norm_err(np.moveaxis(tot, -1, 0), F32s).max() < 1e-5


def test_segments_mixed_precision(gpu_lib):
    ev = synthetic.bbh_events(256, seed=51)
    net = synthetic.make_network(W.IMRPhenomD(), earth=True)
    F64 = run(net, ev, 0, res=2000)
    Fm = run(net, ev, 512, res=2000, precision='mixed', refine_cond=1e10)
    e, cond = sigma_err(Fm, F64, with_cond=True)
    # above ~1e13 the FP64 sigmas themselves move with the summation order (the FP64 recomputation
    # sums frequency segments, the reference FP64 run sums per event), so they are not compared
    ok = cond < 1e13
    print('mixed (segmented) sigma err median %.2e max %.2e over %d events with cond < 1e13 (%d above)'
          % (np.median(e[ok]), e[ok].max(), ok.sum(), (~ok).sum()))
    assert np.all(e[ok] <= 1e-3)


def test_autotune_segments(gpu_lib):
    ev = synthetic.mixed_events(64, seed=61)
    res = synthetic.res_from_chirp_time(ev['Mc'], 2., lo=200, hi=3000)
    net = synthetic.make_network(W.IMRPhenomD(), dets=synthetic.NETWORK_LHET2, earth=True)
    from gwfast_gb300.signal import event_array
    ctx = _lib.context(0)
    sigs = list(net.signals.values())
    p = event_array(ev)
    best = ctx.autotune_segments([s.det_id for s in sigs], W.IMRPhenomD().gpu_desc(), p, int(res.max()),
                                 res_ev=np.ascontiguousarray(res, dtype=np.int32))
    try:
        assert best in (0, 256, 512, 1024, 2048)
        F1 = np.moveaxis(net.FisherMatr(dict(ev), res=int(res.max()), res_per_event=res), -1, 0)
    finally:
        ctx.set_segments(0)
    F0 = np.moveaxis(net.FisherMatr(dict(ev), res=int(res.max()), res_per_event=res), -1, 0)
    print('autotuned segment length', best)
    assert norm_err(F1, F0).max() < 1e-12


@pytest.mark.parametrize('seg', [0, 512])
def test_graph_capture_and_replay(gpu_lib, seg):
    """Device-resident calls: the second identical call is captured into a CUDA graph, later ones
    replay it; new parameter values in the same buffers must show up in the replayed results."""
    torch = pytest.importorskip('torch')
    from gwfast_gb300.signal import event_array
    net = synthetic.make_network(W.IMRPhenomD(), earth=True)
    ids = [s.det_id for s in net.signals.values()]
    desc = W.IMRPhenomD().gpu_desc()
    n = 128
    ctx = _lib.context(0)
    st = torch.cuda.Stream()
    p_dev = torch.empty((11, n), dtype=torch.float64, device='cuda')
    out = torch.empty((n, 11, 11), dtype=torch.float64, device='cuda')
    ref = torch.empty((n, 11, 11), dtype=torch.float64, device='cuda')
    ctx.set_segments(seg)
    try:
        for call, seed in enumerate((101, 102, 103, 104)):
            p_dev.copy_(torch.from_numpy(event_array(synthetic.bbh_events(n, seed=seed))))
            for prec in ('fp64', 'fp32'):
                ctx.set_graphs(False)
                ctx.fisher(ids, desc, p_dev, 1000, mem=_lib.MEM_DEVICE, out_net=ref, stream=st.cuda_stream, ld=n, n=n,
                           precision=prec)
                ctx.set_graphs(True)
                for _ in range(3):   # plain run, capture, replay
                    ctx.fisher(ids, desc, p_dev, 1000, mem=_lib.MEM_DEVICE, out_net=out, stream=st.cuda_stream,
                               ld=n, n=n, precision=prec)
                st.synchronize()
                err = norm_err(out.cpu().numpy(), ref.cpu().numpy()).max()
                assert err < 1e-12, (call, prec, err)
    finally:
        ctx.set_graphs(False)
        ctx.set_segments(0)
