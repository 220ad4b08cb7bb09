#!/usr/bin/env python
"""Benchmark: network Fisher matrices per second on one GB300 (and SNR/s).

Workload (default): 10^4 BBH events, IMRPhenomD, network L1 + H1 (fmin 10 Hz) + ET
triangle at Sardinia (5 Hz wall), Earth rotation on, 2000 log-spaced frequency points
per event and detector, analytic aLIGO PSD fit.  One step = the network Fisher matrix
(11x11, summed over detectors and arms) of every event.

value: events/s of the chosen form with the event arrays resident in HBM, CUDA-event timed
       per step (L2 flushed by a 256 MB write before each step, outside the timed interval).
       The chosen form is 'mixed': the FP32 split-precision kernel for every event, the
       condition number of every network Fisher, and the FP64 kernel again for the events
       above 1e13 (gathered, recomputed, scattered back), all inside the step.  The plain FP64
       kernel and the FP32 form alone are timed the same way (`plain_fp64`, `fp32_only`), and
       the marginalised 1-sigma errors of both reduced forms are compared with the FP64 ones
       on the workload's events (`sigma_err`, `sigma_err_fp32_only`).
e2e:   the chosen form through the public API (DetNet.FisherMatr on a host events dict),
       wall-clock, host->device copy of the parameters and device->host copy of the Fisher
       matrices included.
Multi-GPU: one replica per GPU on its own seeded shard (events are independent; no
collective); value = all ranks' events / max-over-ranks time.

--impl reference: the CPU float64 oracle restatement of gwfast's algorithm (gwfast itself
needs jax[cpu], which is not installable here) on a bounded sample of the same workload, on
all host cores.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_EVENTS = 10000
RES = 2000
SNR_TH = 12.
METRIC = 'network Fisher matrices/s (IMRPhenomD, L1+H1+ETS, Earth rotation, R=2000)'
# DRAM bytes (read + write) per event of the L1 + H1 group launch, from one ncu capture of a
# 2048-event launch (6.575 MB read, 0.055 MB written)
GRP_DRAM_BYTES_PER_EVENT = (6.575104e6 + 5.4784e4) / 2048


def dist_info():
    return int(os.environ.get('RANK', 0)), int(os.environ.get('WORLD_SIZE', 1)), int(os.environ.get('LOCAL_RANK', 0))


def cpu_sample(n_events, res, threads, seed=1001):
    """Time the oracle (torch float64 on the CPU) on a sample of the workload's events."""
    import torch
    import oracle as O
    from gwfast_gb300 import synthetic
    torch.set_num_threads(threads)
    ev = synthetic.bbh_events(n_events, seed=seed)
    p = O.to_params(ev)
    dets = []
    for name, fmin in synthetic.NETWORK_LHET:
        spec = synthetic.detector_spec(name, fmin)
        f, S = spec['psd_path']
        dets.append(O.Detector(spec['det_lat'], spec['det_long'], spec['det_xax'], spec['detector_shape'],
                               fmin=fmin, psd_f=f, psd_S=S, earth=True))
    m = O.Model('PhenomD')
    t0 = time.perf_counter()
    O.network_fisher(dets, m, p, res)
    tf = time.perf_counter() - t0
    t0 = time.perf_counter()
    O.network_snr(dets, m, p, res)
    ts = time.perf_counter() - t0
    return n_events / tf, n_events / ts


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    n_sample = args.ref_events
    vals, svals = [], []
    for _ in range(args.warmup):
        cpu_sample(max(1, n_sample // 4), RES, threads)
    for k in range(args.steps):
        v, s = cpu_sample(n_sample, RES, threads, seed=1001 + k)
        vals.append(v)
        svals.append(s)
    v = statistics.median(vals)
    line = {
        'impl': 'reference', 'metric': METRIC, 'value': v, 'unit': 'Fisher/s', 'n_gpus': 0, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': 1e3 * n_sample / v, 'higher_is_better': True, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic',
        'config': {'workload': 'IMRPhenomD BBH, L1+H1+ETS, Earth rotation, R=2000 (sample of %d events per step)'
                   % n_sample, 'events_per_step': n_sample},
        'snr_per_s': statistics.median(svals),
        'cpu_baseline': {'value': v, 'unit': 'Fisher/s', 'cores': threads, 'kind': 'port',
                         'sample': '%d events per step, all 3 detectors, R=2000' % n_sample},
        'e2e': {'value': v, 'unit': 'Fisher/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
        'note': 'gwfast needs jax[cpu] (absent from the offline wheelhouse); the timed CPU path is the float64 '
                'oracle restatement of its algorithm (torch on the host cores)',
    }
    print(json.dumps(line))


class ClockSampler:
    def __init__(self, device):
        self.f = tempfile.NamedTemporaryFile('w+', suffix='.csv', delete=False)
        q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,'
             'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,'
             'clocks_event_reasons.sw_power_cap')
        try:
            self.p = subprocess.Popen(['nvidia-smi', '-i', str(device), '--query-gpu=' + q, '--format=csv,noheader,nounits',
                                       '-lms', '200'], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(',')]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace('.', '').isdigit()]
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith('active')})
        return {'sm_mhz': statistics.median(sm) if sm else None, 'sm_max_mhz': float(rows[0][2]) if rows else None,
                'reasons': reasons, 'samples': len(rows)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as fh:
            return json.load(fh)
    except OSError:
        return {}


def gemm_peak(torch, dev, dtype, n):
    """Dense GEMM throughput (cuBLAS through torch.matmul, TF32 off), best of 5, TFLOP/s."""
    torch.backends.cuda.matmul.allow_tf32 = False
    a = torch.randn(n, n, dtype=dtype, device=dev)
    b = torch.randn(n, n, dtype=dtype, device=dev)
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    return 2 * n ** 3 / best / 1e12


def _timed_stream(torch, stream, flush):
    """CUDA-event timer on `stream`: mean ms of k calls after `warm` untimed ones, L2 flushed before each."""
    def timed(fn, k, warm=0):
        for _ in range(warm):
            fn()
        tot = 0.0
        for _ in range(k):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            tot += e0.elapsed_time(e1)
        return tot / k
    return timed


def measure_mixed_catalogue(n_events, steps, warmup, refine_cond=1e13, fp64_sample=2000):
    """Batching workload: 50 % BNS + 50 % BBH, per-event grid lengths from the chirp time at 2 Hz
    (200 to 40000 points), L1 + H1 (10 Hz) + ET triangle (2 Hz wall), IMRPhenomD, Earth rotation.
    FP32 and mixed forms over all events, per-event launches against the autotuned persistent
    segmented launches (CUDA-graph replay for the device-resident FP32 form); the plain FP64 kernel
    (per-event launches) timed on the first fp64_sample events (i.i.d. events, so the per-event rate
    carries over). SNR/s of the FP32 and FP64 SNR kernels."""
    import torch
    from gwfast_gb300 import _build, _lib, synthetic
    from gwfast_gb300 import waveforms as W
    from gwfast_gb300.signal import event_array
    _build.build()
    dev = torch.device('cuda', 0)
    N = n_events
    ev = synthetic.mixed_events(N, seed=1002)
    res_ev = synthetic.res_from_chirp_time(ev['Mc'], 2.)
    rmax = int(res_ev.max())
    wf = W.IMRPhenomD()
    net = synthetic.make_network(wf, dets=synthetic.NETWORK_LHET2, earth=True)
    ids = [s.det_id for s in net.signals.values()]
    ctx = _lib.context(0)
    ctx.set_refine_cond(refine_cond)
    p_dev = torch.from_numpy(event_array(ev)).to(dev)
    r_dev = torch.from_numpy(np.ascontiguousarray(res_ev, dtype=np.int32)).to(dev)
    out = torch.empty((N, 11, 11), dtype=torch.float64, device=dev)
    snr_out = torch.empty((N,), dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    desc = wf.gpu_desc()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    timed = _timed_stream(torch, stream, flush)
    n64 = min(N, fp64_sample)

    def step(precision, n=N):
        ctx.fisher(ids, desc, p_dev, rmax, res_ev=r_dev, per_arm=False, mem=_lib.MEM_DEVICE, out_net=out,
                   stream=stream.cuda_stream, ld=N, n=n, precision=precision)

    forms = {}
    try:
        ctx.set_graphs(False)
        ctx.set_segments(0)
        forms['fp64_per_event'] = timed(lambda: step('fp64', n64), max(1, steps // 2), 1) * N / n64
        forms['fp32_per_event'] = timed(lambda: step('fp32'), steps, warmup)
        forms['mixed_per_event'] = timed(lambda: step('mixed'), steps, warmup)
        seg = ctx.autotune_segments(ids, desc, p_dev, rmax, res_ev=r_dev, precision='fp32', mem=_lib.MEM_DEVICE,
                                    ld=N, n=min(N, 4000))
        forms['fp32_segment_points'] = seg
        ctx.set_graphs(True)
        forms['fp32_segmented_graph'] = timed(lambda: step('fp32'), steps, warmup)
        ctx.set_graphs(False)
        forms['mixed_segmented'] = timed(lambda: step('mixed'), steps, warmup)
        ctx.set_segments(0)
        ms_snr = timed(lambda: ctx.snr(ids, desc, p_dev, rmax, res_ev=r_dev, mem=_lib.MEM_DEVICE, out_net=snr_out,
                                       stream=stream.cuda_stream, ld=N, n=N, precision='fp32'), steps, warmup)
        ms_snr64 = timed(lambda: ctx.snr(ids, desc, p_dev, rmax, res_ev=r_dev, mem=_lib.MEM_DEVICE, out_net=snr_out,
                                         stream=stream.cuda_stream, ld=N, n=n64), max(1, steps // 2), 1) * N / n64
    finally:
        ctx.set_graphs(False)
        ctx.set_segments(0)
    best = min(('mixed_per_event', 'mixed_segmented'), key=lambda k: forms[k])
    return {
        'metric': 'network Fisher matrices/s, mixed BNS+BBH catalogue (per-event grids 200-40000 points)',
        'value': N / (forms[best] / 1e3), 'unit': 'Fisher/s', 'chosen': best, 'ms_per_step': forms[best],
        'dtype': 'f32 per point, f64 for events with cond > %.0e' % refine_cond,
        'config': {'workload': 'IMRPhenomD, %d events (50%% BNS, 50%% BBH), L1+H1 (10 Hz) + ETS (2 Hz), Earth rotation, '
                               'per-event res from chirp time' % N, 'res_min': int(res_ev.min()), 'res_max': rmax,
                   'points_total': int(res_ev.sum()), 'l2': 'flushed (256 MB write) before every step',
                   'fp64_sampled_events': n64},
        'forms_ms_per_step': forms,
        'fisher_per_s': {k: N / (v / 1e3) for k, v in forms.items() if not k.endswith('points')},
        'speedup_vs_fp64_per_event': forms['fp64_per_event'] / forms[best],
        'snr_per_s': {'fp32': N / (ms_snr / 1e3), 'fp64': N / (ms_snr64 / 1e3)},
    }


def run_mixed_catalogue(args):
    line = measure_mixed_catalogue(args.events, args.steps, args.warmup, args.refine_cond)
    line.update({'n_gpus': 1, 'steps': args.steps, 'warmup': args.warmup, 'higher_is_better': True,
                 'scaling': 'weak', 'vs_baseline': None, 'data': 'synthetic (seeded mixed catalogue)'})
    print(json.dumps(line))


def measure_screen(n_events, train_events, train_epochs, steps, warmup, fp64_sample=50000, per_event_res=True):
    """Learned-screen workload: n_events of the mixed population with dL up to 30 Gpc, the headline
    network (L1 + H1 at 10 Hz, ET triangle at 5 Hz), IMRPhenomD, threshold SNR 12, per-event grid
    lengths from the chirp time at 2 Hz (200 to 40000 points). The screened path (MLP prediction,
    FP32 SNR for the events near threshold and a 1 % audit of the skipped ones, mixed-form Fisher of
    the detected ones) over all events, against the plain FP64 path (FP64 SNR of every event, FP64
    Fisher of the detected ones) timed on a random sample of fp64_sample events (the same population,
    so detected events per second carry over). The network is trained first on train_events exact
    SNRs of other events of the population (timed apart). Fisher/s = detected events / wall time,
    host dict in, host arrays out. The sigma error of the screened path's Fishers against the FP64
    kernel is checked on the detected events of the FP64 sample."""
    import torch
    from gwfast_gb300 import _build, fisherTools, pipeline, synthetic
    from gwfast_gb300 import waveforms as W
    from gwfast_gb300.screen import SNRScreen
    _build.build()
    torch.cuda.set_device(0)
    N = n_events
    net = synthetic.make_network(W.IMRPhenomD(), dets=synthetic.NETWORK_LHET, earth=True)
    train = synthetic.screen_population(train_events, seed=2004)
    ev = synthetic.screen_population(N, seed=1004)
    rmax = 40000 if per_event_res else 1000
    rtrain = synthetic.res_from_chirp_time(train['Mc'], 2.) if per_event_res else None
    rev = synthetic.res_from_chirp_time(ev['Mc'], 2.) if per_event_res else None
    t0 = time.perf_counter()
    screen = SNRScreen(net, hidden=256, layers=4, seed=1)
    loss = screen.fit(dict(train), res=rmax, res_per_event=rtrain, epochs=train_epochs, batch=4096, lr=2e-3)
    t_train = time.perf_counter() - t0
    kw = dict(snr_th=SNR_TH, res=rmax, sky_area=False)
    for _ in range(max(1, warmup)):
        pipeline.compute_errs(net, dict(ev), precision='mixed', screen=screen, res_per_event=rev, **kw)
    ts = []
    for _ in range(steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rs = pipeline.compute_errs(net, dict(ev), precision='mixed', screen=screen, res_per_event=rev, **kw)
        ts.append(time.perf_counter() - t0)
    rng = np.random.default_rng(7)
    samp = np.sort(rng.choice(N, size=min(N, fp64_sample), replace=False))
    evs = {k: np.asarray(v)[samp] for k, v in ev.items()}
    rs_samp = None if rev is None else rev[samp]
    pipeline.compute_errs(net, dict(evs), precision='fp64', snr_precision='fp64', res_per_event=rs_samp, **kw)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rp = pipeline.compute_errs(net, dict(evs), precision='fp64', snr_precision='fp64', res_per_event=rs_samp, **kw)
    t_p = time.perf_counter() - t0
    t_s = statistics.median(ts)
    det_s, det_p = rs['detected'], rp['detected']
    # sigma error of the screened path's Fisher matrices against the plain FP64 ones, on the events
    # detected by both in the FP64 sample
    pos_s = -np.ones(N, dtype=np.int64)
    pos_s[np.where(det_s)[0]] = np.arange(det_s.sum())
    both = det_p & det_s[samp]
    Fp = rp['fisher'][..., np.where(both[det_p])[0]]
    Fs = rs['fisher'][..., pos_s[samp[both]]]
    c64, _, cond = fisherTools.CovMatr(Fp, return_cond=True)
    cs, _, _ = fisherTools.CovMatr(Fs, return_cond=True)
    s64, ss = np.sqrt(np.abs(np.einsum('iin->ni', c64))), np.sqrt(np.abs(np.einsum('iin->ni', cs)))
    err = (np.abs(ss - s64) / s64).max(axis=1)
    ok = cond < 1e13
    rate_s = float(det_s.sum() / t_s)
    rate_p = float(det_p.sum() / t_p)
    return {
        'metric': 'forecast Fisher matrices/s with the learned SNR screen (detected events / wall time)',
        'value': rate_s, 'unit': 'Fisher/s', 'ms_per_step': 1e3 * t_s, 'steps': steps, 'warmup': warmup,
        'dtype': 'bf16 weights / f32 MLP; f32 SNR; f32 Fisher with f64 for cond > 1e13',
        'config': {'workload': '%d events, 50%% BNS / 50%% BBH, dL <= 30 Gpc, L1+H1+ETS, IMRPhenomD, %s, SNR > %g'
                               % (N, 'per-event res from chirp time at 2 Hz (200-40000)' if per_event_res else
                                  'R=1000', SNR_TH),
                   'mlp': '11 -> 4 x 256 SiLU -> 1, trained on %d exact SNRs, %d epochs' % (train_events, train_epochs),
                   'band_ln_snr': 0.3, 'audit_fraction': 0.01,
                   'points_total': int(rev.sum()) if rev is not None else N * 1000},
        'screen': rs['screen'], 'train_s': t_train, 'train_loss_ln_snr_mse': loss,
        'plain_fp64_path': {'value': rate_p, 'unit': 'Fisher/s', 's_sample': t_p, 'sample_events': int(len(samp)),
                            'detected_in_sample': int(det_p.sum()),
                            'what': 'FP64 SNR of every sampled event, FP64 Fisher of the detected ones'},
        'speedup_vs_plain_fp64_path': rate_s / rate_p,
        'detected': int(det_s.sum()),
        'recall_vs_exact_path_on_sample': float(np.mean(det_s[samp][det_p])) if det_p.any() else None,
        'false_detections_on_sample': int(np.sum(det_s[samp] & ~det_p)),
        'sigma_err_vs_fp64_on_sample': {'events_cond_lt_1e13': int(ok.sum()),
                                        'median': float(np.median(err[ok])) if ok.any() else None,
                                        'max': float(err[ok].max()) if ok.any() else None,
                                        'events_cond_ge_1e13': int((~ok).sum())},
    }


def run_screen(args):
    line = measure_screen(args.events if args.events != N_EVENTS else 1000000, args.train_events, args.train_epochs,
                          args.steps, args.warmup)
    line.update({'n_gpus': 1, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
                 'data': 'synthetic (seeded population, dL up to 30 Gpc)'})
    print(json.dumps(line))


def measure_hm(n_events, steps, warmup, refine_cond=1e13, fp64_sample=8192):
    """Higher-mode workload: IMRPhenomHM (modes 21, 22, 32, 33, 43, 44) aligned-spin BBH, m1 power law
    on [5, 150] Msun, q ~ U[0.1, 1], chi ~ U[-0.9, 0.9], dL ~ U[0.5, 20] Gpc; ET triangle + CE1Id +
    CE2NM (5 Hz walls), Earth rotation, R = 4000. Device-resident events; the FP32 split-precision
    form (FP64 mode phases) and the mixed form over all events, the FP64 kernel over the first
    fp64_sample (i.i.d. events, so the per-event rate carries over); sigma errors of both forms against
    the FP64 kernel on the first 4096 events; SNR/s of the FP64 and FP32 SNR kernels."""
    import torch
    from gwfast_gb300 import _build, _lib, fisherTools, synthetic
    from gwfast_gb300 import waveforms as W
    from gwfast_gb300.signal import event_array
    _build.build()
    dev = torch.device('cuda', 0)
    N = n_events
    R = 4000
    ev = synthetic.bbh_events(N, seed=1003, mmax=150., qmin=0.1, chimax=0.9, dl=(0.5, 20.))
    wf = W.IMRPhenomHM()
    net = synthetic.make_network(wf, dets=synthetic.NETWORK_ET_CE, earth=True)
    ids = [s.det_id for s in net.signals.values()]
    ctx = _lib.context(0)
    ctx.set_refine_cond(refine_cond)
    p_dev = torch.from_numpy(event_array(ev)).to(dev)
    out = torch.empty((N, 11, 11), dtype=torch.float64, device=dev)
    snr_out = torch.empty((N,), dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    desc = wf.gpu_desc()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    timed = _timed_stream(torch, stream, flush)

    def step(precision, n, o=out):
        ctx.fisher(ids, desc, p_dev, R, per_arm=False, mem=_lib.MEM_DEVICE, out_net=o, stream=stream.cuda_stream,
                   ld=N, n=n, precision=precision)

    n64 = min(N, fp64_sample)
    clk = ClockSampler(0)
    ms32 = timed(lambda: step('fp32', N), steps, warmup)
    msmix = timed(lambda: step('mixed', N), steps, warmup)
    ms64 = timed(lambda: step('fp64', n64), max(1, steps // 2), 1)
    ms_snr = timed(lambda: ctx.snr(ids, desc, p_dev, R, mem=_lib.MEM_DEVICE, out_net=snr_out,
                                   stream=stream.cuda_stream, ld=N, n=N), steps, warmup)
    ms_snr32 = timed(lambda: ctx.snr(ids, desc, p_dev, R, mem=_lib.MEM_DEVICE, out_net=snr_out,
                                     stream=stream.cuda_stream, ld=N, n=N, precision='fp32'), steps, warmup)
    clocks = clk.stop()
    ns = min(N, 4096)
    F = {}
    for prec in ('fp64', 'fp32', 'mixed'):
        o = torch.empty((ns, 11, 11), dtype=torch.float64, device=dev)
        step(prec, ns, o)
        torch.cuda.synchronize()
        F[prec] = o.cpu().numpy()

    def sigmas(Fx):
        c, _, cond = fisherTools.CovMatr(np.moveaxis(Fx, 0, -1), return_cond=True)
        return np.sqrt(np.abs(np.einsum('iin->ni', c))), cond

    s64, cond = sigmas(F['fp64'])
    stable = cond < 1e13
    errs = {}
    for prec in ('fp32', 'mixed'):
        sx, _ = sigmas(F[prec])
        w = (np.abs(sx - s64) / s64).max(axis=1)
        errs[prec] = {'median': float(np.median(w)), 'p99': float(np.percentile(w, 99)),
                      'max_cond_lt_1e13': float(w[stable].max()), 'events_cond_lt_1e13': int(stable.sum()),
                      'events': int(ns), 'frac_le_1e-3': float(np.mean(w <= 1e-3))}
    rate64 = n64 / (ms64 / 1e3)
    return {
        'metric': 'network Fisher matrices/s, IMRPhenomHM on ET + 2 CE (mixed form vs plain FP64 kernel)',
        'value': N / (msmix / 1e3), 'unit': 'Fisher/s', 'ms_per_step': msmix,
        'dtype': 'f64 mode phases, f32 amplitudes/tangents/mode sums, f64 for events with cond > %.0e' % refine_cond,
        'config': {'workload': 'IMRPhenomHM, %d BBH, ETS + CE1Id + CE2NM (5 Hz), Earth rotation, R=%d' % (N, R),
                   'l2': 'flushed (256 MB write) before every step', 'fp64_sampled_events': n64},
        'fisher_per_s': {'mixed': N / (msmix / 1e3), 'fp32': N / (ms32 / 1e3), 'fp64': rate64},
        'speedup_mixed_vs_fp64': (N / (msmix / 1e3)) / rate64,
        'snr_per_s': {'fp64': N / (ms_snr / 1e3), 'fp32': N / (ms_snr32 / 1e3)},
        'sigma_err_vs_fp64': errs,
        'clocks': clocks,
    }


def run_hm(args):
    line = measure_hm(args.events if args.events != N_EVENTS else 100000, args.steps, args.warmup, args.refine_cond)
    line.update({'n_gpus': 1, 'steps': args.steps, 'warmup': args.warmup, 'higher_is_better': True,
                 'scaling': 'weak', 'vs_baseline': None, 'data': 'synthetic (seeded BBH catalogue)'})
    print(json.dumps(line))


def run_mlp(args):
    """The screen's network alone: train the 11 -> 4 x 256 SiLU -> 1 MLP for --train-epochs epochs on
    --train-events events (batch 4096), then predict ln SNR for --events device-resident events (fused
    tensor-core inference), CUDA wall clock per call, median of --steps after --warmup."""
    import torch
    from gwfast_gb300 import _build, _lib, synthetic
    from gwfast_gb300.signal import event_array
    _build.build()
    torch.cuda.set_device(0)
    n = args.events if args.events != N_EVENTS else 1000000
    pt = event_array(synthetic.screen_population(args.train_events, seed=2004))
    target = np.log(np.random.default_rng(0).uniform(1.0, 100.0, pt.shape[1]))
    mlp = _lib.MLP(hidden=256, layers=4, seed=1)
    t0 = time.perf_counter()
    loss = mlp.train(pt, target, epochs=args.train_epochs, batch=4096, lr=1e-3)
    t_train = time.perf_counter() - t0
    lib = _lib.load()
    dp = torch.from_numpy(event_array(synthetic.screen_population(n, seed=1004))).cuda()
    out = torch.empty(n, dtype=torch.float64, device='cuda')

    def pred():
        _lib.check(lib.gwf_mlp_predict(mlp.h, _lib.ptr(dp), n, n, _lib.MEM_DEVICE, _lib.ptr(out)))

    for _ in range(args.warmup):
        pred()
    ts = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pred()
        ts.append(time.perf_counter() - t0)
    t = statistics.median(ts)
    print(json.dumps({'metric': 'MLP ln SNR predictions/s (11 -> 4 x 256 SiLU -> 1, BF16 weights, tensor cores)',
                      'value': n / t, 'unit': 'predictions/s', 'n_gpus': 1, 'steps': args.steps, 'warmup': args.warmup,
                      'ms_per_step': 1e3 * t, 'higher_is_better': True, 'events': n,
                      'train_s': t_train, 'train_epochs': args.train_epochs, 'train_events': args.train_events,
                      'train_loss': loss, 'data': 'synthetic (seeded population)'}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=5)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=('ours', 'reference'))
    ap.add_argument('--events', type=int, default=N_EVENTS)
    ap.add_argument('--ref-events', type=int, default=6)
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--only-device', action='store_true', help='only the device-resident Fisher steps (for ncu)')
    ap.add_argument('--precision', default='fp32', choices=('fp32', 'fp64', 'mixed'), help='form used with --only-device')
    ap.add_argument('--refine-cond', type=float, default=1e13, help='condition-number threshold of the mixed form')
    ap.add_argument('--no-autotune', action='store_true', help='per-event launches, no segment autotuning')
    ap.add_argument('--workload', default='lhet', choices=('lhet', 'mixed-catalogue', 'screen', 'hm', 'mlp'),
                    help='lhet: the headline workload; mixed-catalogue: the batching workload; screen: the learned '
                         'SNR screen on a 10^6-event population; hm: IMRPhenomHM on ET + CE; mlp: the screen network '
                         'alone, training and inference (separate lines)')
    ap.add_argument('--headline-only', action='store_true', help='leave out the other workloads\' keys')
    ap.add_argument('--train-events', type=int, default=200000)
    ap.add_argument('--train-epochs', type=int, default=40)
    args = ap.parse_args()
    if args.impl == 'reference':
        return run_reference(args)
    if args.workload == 'mixed-catalogue':
        return run_mixed_catalogue(args)
    if args.workload == 'screen':
        return run_screen(args)
    if args.workload == 'hm':
        return run_hm(args)
    if args.workload == 'mlp':
        return run_mlp(args)
    rank, world, local = dist_info()
    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl' if torch.cuda.is_available() else 'gloo')
    torch.cuda.set_device(local)
    dev = torch.device('cuda', local)
    from gwfast_gb300 import _build, _lib, fisherTools, synthetic
    from gwfast_gb300 import waveforms as W
    from gwfast_gb300.signal import event_array
    _build.build()
    N = args.events
    ev = synthetic.bbh_events(N, seed=1001 + rank)
    wf = W.IMRPhenomD()
    net = synthetic.make_network(wf, dets=synthetic.NETWORK_LHET, earth=True, device=local)
    sigs = list(net.signals.values())
    ids = [s.det_id for s in sigs]
    ctx = _lib.context(local)
    p_host = event_array(ev)
    p_dev = torch.from_numpy(p_host).to(dev)
    out = torch.empty((N, 11, 11), dtype=torch.float64, device=dev)
    out64 = torch.empty((N, 11, 11), dtype=torch.float64, device=dev)
    snr_out = torch.empty((N,), dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(dev)   # a real stream handle: NULL would mean the library's own stream
    torch.cuda.set_stream(stream)
    desc = wf.gpu_desc()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > 129 MB L2

    ctx.set_refine_cond(args.refine_cond)
    out32 = torch.empty((N, 11, 11), dtype=torch.float64, device=dev)
    # launch shape: per-event CTAs or persistent segments, chosen by the library's autotuner on a sample
    seg = 0
    if not args.no_autotune and not args.only_device:
        ns = min(N, 2000)
        seg = ctx.autotune_segments(ids, desc, p_dev, RES, precision='fp32', mem=_lib.MEM_DEVICE, ld=N, n=ns)

    def fisher_step(det_ids=ids, o=out, precision='mixed'):
        ctx.fisher(det_ids, desc, p_dev, RES, per_arm=False, mem=_lib.MEM_DEVICE, out_net=o, stream=stream.cuda_stream,
                   ld=N, n=N, precision=precision)

    def snr_step(precision='fp64'):
        ctx.snr(ids, desc, p_dev, RES, mem=_lib.MEM_DEVICE, out_net=snr_out, stream=stream.cuda_stream, ld=N, n=N,
                precision=precision)

    def timed(fn, k):
        tot = 0.0
        for _ in range(k):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            tot += e0.elapsed_time(e1)
        return tot / k

    if args.only_device:
        for _ in range(args.warmup + args.steps):
            fisher_step(precision=args.precision)
        torch.cuda.synchronize()
        print(json.dumps({'only_device': True, 'events': N, 'steps': args.steps, 'precision': args.precision}))
        return
    for _ in range(args.warmup):
        fisher_step()
        fisher_step(o=out32, precision='fp32')
        fisher_step(o=out64, precision='fp64')
        snr_step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clk = ClockSampler(local)
    ms = timed(fisher_step, args.steps)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = clk.stop()
    ms64 = timed(lambda: fisher_step(o=out64, precision='fp64'), args.steps)
    ms32 = timed(lambda: fisher_step(o=out32, precision='fp32'), args.steps)
    ms_snr = timed(snr_step, args.steps)
    snr_step('fp32')
    ms_snr32 = timed(lambda: snr_step('fp32'), args.steps)
    # each detector set's call alone (set-up launches + one Fisher launch): ETS (triangle kernel), L1
    ms_et = timed(lambda: fisher_step([ids[2]], o=out32, precision='fp32'), args.steps)
    ms_l1 = timed(lambda: fisher_step([ids[0]], o=out32, precision='fp32'), args.steps)
    # L1 + H1 share the grid: one group launch, the largest share of the step's GPU time
    ms_grp = timed(lambda: fisher_step(ids[:2], o=out32, precision='fp32'), args.steps)
    ms_et64 = timed(lambda: fisher_step([ids[2]], precision='fp64'), max(1, args.steps // 2))
    # kernel-only times: the library's CUDA events around its own launches (the set-up launches of a
    # chunk, each Fisher launch), on the stream each ran on; median over steps of the per-call sums
    ctx.set_kernel_timing(True)

    def sections(fn, k):
        per = {}
        for _ in range(k):
            flush.zero_()
            fn()
            tot = {}
            for name, t in ctx.kernel_times():
                tot[name] = tot.get(name, 0.0) + t
            for name, t in tot.items():
                per.setdefault(name, []).append(t)
        return {name: statistics.median(v) for name, v in per.items()}

    kt_grp = sections(lambda: fisher_step(ids[:2], o=out32, precision='fp32'), args.steps)
    kt_et = sections(lambda: fisher_step([ids[2]], o=out32, precision='fp32'), args.steps)
    kt_et64 = sections(lambda: fisher_step([ids[2]], precision='fp64'), max(1, args.steps // 2))
    kt_mixed = sections(fisher_step, args.steps)
    ctx.set_kernel_timing(False)
    if world > 1:
        t = torch.tensor([ms, ms64, ms32, ms_snr], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms, ms64, ms32, ms_snr = (float(x) for x in t)
    # accuracy of the reduced forms on this workload: marginalised 1-sigma errors against FP64
    fisher_step()
    fisher_step(o=out32, precision='fp32')
    fisher_step(o=out64, precision='fp64')
    torch.cuda.synchronize()
    Fm_all = out.cpu().numpy()
    F64_all = out64.cpu().numpy()
    dg = np.sqrt(np.abs(np.einsum('nii->ni', F64_all)))
    refined = float(np.mean((np.abs(Fm_all - F64_all) / (dg[:, :, None] * dg[:, None, :])).max(axis=(1, 2)) < 1e-11))
    nchk = min(N, 4000)
    c64, _, cond = fisherTools.CovMatr(np.moveaxis(F64_all[:nchk], 0, -1), return_cond=True, device=local)
    s64 = np.sqrt(np.einsum('iin->ni', c64))

    # above equilibrated cond ~1e13 the FP64 sigmas themselves change with the summation order
    # (two FP64 runs that sum in a different order disagree there), so those events are counted apart
    stable = cond < 1e13

    def sig_err(F):
        c, _, _ = fisherTools.CovMatr(np.moveaxis(F[:nchk], 0, -1), return_cond=True, device=local)
        e = np.nanmax(np.abs(np.sqrt(np.einsum('iin->ni', c)) - s64) / s64, axis=1)
        es = e[stable]
        return {'events': int(stable.sum()), 'median': float(np.nanmedian(es)), 'p99': float(np.nanpercentile(es, 99)),
                'max': float(np.nanmax(es)), 'frac_le_1e-3': float(np.mean(es <= 1e-3)),
                'events_cond_ge_1e13': int((~stable).sum()), 'frac_le_1e-3_all_events': float(np.mean(e <= 1e-3)),
                'what': 'max over 11 parameters of |sigma - sigma_fp64| / sigma_fp64 per event, events with '
                        'equilibrated cond < 1e13 (FP64 sigmas stable under summation order)'}

    serr_mixed = sig_err(Fm_all)
    serr_fp32 = sig_err(out32.cpu().numpy())
    # end to end through the public API with host buffers: DetNet.FisherMatr (mixed form) on every event
    for _ in range(max(1, args.warmup // 2)):
        net.FisherMatr(dict(ev), res=RES, precision='mixed', refine_cond=args.refine_cond)
    torch.cuda.synchronize()
    # three calls per step: each is ~10 ms of wall clock, so a few more keep one slow call from
    # dominating the mean
    e2e_iter = []
    n_e2e = 3 * args.steps
    t0 = time.perf_counter()
    for _ in range(n_e2e):
        ti = time.perf_counter()
        F_host = net.FisherMatr(dict(ev), res=RES, precision='mixed', refine_cond=args.refine_cond)
        e2e_iter.append(time.perf_counter() - ti)
    e2e_s = (time.perf_counter() - t0) / n_e2e
    # the forecast pipeline: SNR pass (FP32) on every event, threshold SNR > 12, network Fisher of the
    # detected events (mixed form), covariances; Fisher/s = detected events / wall time of SNR + Fisher
    from gwfast_gb300 import pipeline
    for _ in range(max(1, args.warmup // 2)):
        pipeline.compute_errs(net, dict(ev), snr_th=SNR_TH, res=RES, precision='mixed', refine_cond=args.refine_cond)
    torch.cuda.synchronize()
    pipe_t, cov_t, ndet = 0.0, 0.0, 0
    for _ in range(args.steps):
        tm = {}
        r = pipeline.compute_errs(net, dict(ev), snr_th=SNR_TH, res=RES, precision='mixed',
                                  refine_cond=args.refine_cond, timings=tm)
        pipe_t += tm['snr'] + tm['fisher']
        cov_t += tm['cov']
        ndet = int(r['detected'].sum())
    pipe_s = pipe_t / args.steps
    if rank != 0:
        torch.distributed.destroy_process_group()
        return
    ops = json.load(open(os.path.join(ROOT, 'profiles', 'opcounts.json')))['counts']['IMRPhenomD/earth']
    flop_arm_pt = ops['fisher_per_arm_point']
    flops_et = N * RES * 3 * flop_arm_pt
    flops_grp = N * RES * 2 * flop_arm_pt
    peak32 = gemm_peak(torch, dev, torch.float32, 8192)
    peak64 = gemm_peak(torch, dev, torch.float64, 4096)
    k_grp, k_et, k_et64 = kt_grp['group_f32'], kt_et['fisher_f32'], kt_et64['fisher_f64']
    ach = flops_et / (k_et / 1e3) / 1e12
    ach_grp = flops_grp / (k_grp / 1e3) / 1e12
    ach64 = flops_et / (k_et64 / 1e3) / 1e12
    kernel_note = ('CUDA events recorded by the library around this one launch on its stream (gwf_kernel_times), '
                   'median over steps; the L2 is flushed before each call')
    line = {
        'metric': METRIC, 'value': world * N / (ms / 1e3), 'unit': 'Fisher/s', 'n_gpus': world, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': ms, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'f32 per point (f64 per-event set-up, scaling, outputs, and f64 throughout for events with cond > %.0e)'
                 % args.refine_cond,
        'data': 'synthetic (seeded BBH catalogue, analytic aLIGO PSD fit)',
        'config': {'workload': 'IMRPhenomD BBH 1e4 events, L1+H1+ETS, Earth rotation, R=2000; mixed form (FP32 '
                               'split precision, FP64 for equilibrated cond > %.0e)' % args.refine_cond,
                   'events_per_gpu': N, 'res': RES, 'parallelism': 'replicas over event shards' if world > 1 else 'single',
                   'l2': 'flushed (256 MB write) before every step',
                   'segments': seg if seg else 'per-event launches (autotuned)' if not args.no_autotune else 'per-event launches'},
        'plain_fp64': {'value': world * N / (ms64 / 1e3), 'unit': 'Fisher/s', 'ms_per_step': ms64},
        'speedup_vs_plain_fp64': ms64 / ms,
        'fp32_only': {'value': world * N / (ms32 / 1e3), 'unit': 'Fisher/s', 'ms_per_step': ms32},
        'refined_fraction': refined,
        'sigma_err': serr_mixed,
        'sigma_err_fp32_only': serr_fp32,
        'snr_per_s': world * N / (ms_snr / 1e3),
        'snr_per_s_fp32': world * N / (ms_snr32 / 1e3),
        # first pass: 2 set-up + 2 FP32-record launches (L1, ETS), H1's projection launch, the L1+H1
        # group kernel, the ET kernel and the join of the two groups' totals; the condition estimate
        # and selection; with refined events: gather; L1 + H1 as one FP64 group (2 set-up record
        # copies, H1's projection patch, segment scan, segmented group kernel, reduction); ETS (record
        # copy, segment scan, segmented FP64 kernel, reduction); sum-scatter
        'gpu_launches': 8 + 2 + (12 if refined > 0 else 0),
        'e2e': {'value': world * N / e2e_s, 'unit': 'Fisher/s', 'h2d_bytes_per_step': int(p_host.nbytes),
                'd2h_bytes_per_step': int(F_host.nbytes),
                'ms_per_step_each': [round(1e3 * t, 3) for t in e2e_iter],
                'what': 'DetNet.FisherMatr(precision=mixed) on a host events dict, host (11, 11, N) out, wall clock'},
        'forecast_pipeline': {'value': world * ndet / pipe_s, 'unit': 'Fisher/s', 'detected': ndet, 'events': N,
                              'snr_plus_fisher_s': pipe_s, 'covariance_s': cov_t / args.steps,
                              'what': 'pipeline.compute_errs: DetNet.SNR (FP32) on every event, threshold SNR > %g, '
                                      'DetNet.FisherMatr (mixed) on the detected ones; Fisher/s = detected / wall '
                                      'time of SNR + Fisher (host dict in, host arrays out)' % SNR_TH,
                              'h2d_bytes': int(8 * 11 * (N + ndet)), 'd2h_bytes': int(8 * (5 * N + 121 * ndet))},
        'roofline': {'bound': 'fp32', 'kernel': 'fisher_group_kernel_f32<IMRPhenomD, earth, no triangle> (L1+H1)',
                     'achieved': ach_grp, 'peak': peak32, 'unit': 'TFLOP/s', 'frac': ach_grp / peak32,
                     'peak_source': 'cuBLAS SGEMM 8192^3 (TF32 off) measured in this run (MEASURED_PEAKS.json has '
                                    'no FP32 CUDA-core figure)',
                     'algorithmic_flop_per_launch': flops_grp, 'kernel_ms': k_grp, 'timing': kernel_note,
                     'traffic': GRP_DRAM_BYTES_PER_EVENT * N,
                     'traffic_source': 'ncu dram__bytes_read.sum + dram__bytes_write.sum of one 2048-event launch '
                                       '(profiles/fisher_group_f32_phenomd_l1h1.md), scaled by events',
                     'flop_model': 'profiles/opcounts.json IMRPhenomD/earth fisher_per_arm_point x 2 arms x R x N'},
        'roofline_triangle': {'bound': 'fp32', 'kernel': 'fisher_kernel_f32<IMRPhenomD, earth, triangle>',
                              'achieved': ach, 'peak': peak32, 'unit': 'TFLOP/s', 'frac': ach / peak32,
                              'algorithmic_flop_per_launch': flops_et, 'kernel_ms': k_et, 'timing': kernel_note,
                              'traffic': 3.49e6 * N / 1024,
                              'traffic_source': 'ncu dram__bytes_read.sum + dram__bytes_write.sum of a 1024-event '
                                                'launch (3.49 MB, profiles/fisher_f32_phenomd_ets.md), scaled by events',
                              'flop_model': 'profiles/opcounts.json IMRPhenomD/earth fisher_per_arm_point x 3 arms x R x N'},
        'roofline_fp64': {'bound': 'fp64', 'kernel': 'fisher_kernel<IMRPhenomD, earth, triangle>', 'achieved': ach64,
                          'peak': peak64, 'unit': 'TFLOP/s', 'frac': ach64 / peak64, 'kernel_ms': k_et64,
                          'timing': kernel_note, 'peak_source': 'cuBLAS DGEMM 4096^3 measured in this run'},
        'call_ms': {'L1': ms_l1, 'L1+H1': ms_grp, 'ETS': ms_et},
        'kernel_ms': {'L1+H1 FP32 call': kt_grp, 'ETS FP32 call': kt_et, 'ETS FP64 call': kt_et64,
                      'mixed step': kt_mixed,
                      'what': 'per call, summed by section: setup = FP64 set-up + FP32 record launches of each chunk; '
                              'in the mixed step the two detector groups run side by side, so sections overlap'},
        'clocks': clocks,
        'hbm_peak_gbs': measured_peaks().get('hbm_gbs'),
    }
    if world == 1 and not args.headline_only:
        # the other workloads as keys of the same line (each its own synthetic catalogue; plain FP64
        # arms on samples of the same catalogue, as stated in each)
        line['config4_screened_catalogue'] = measure_screen(1000000, args.train_events, args.train_epochs, 2, 1)
        line['config2_mixed_catalogue'] = measure_mixed_catalogue(100000, 2, 1, args.refine_cond)
        line['config3_phenomhm'] = measure_hm(100000, 2, 1, args.refine_cond)
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, _ = cpu_sample(args.ref_events, RES, threads)
        line['cpu_baseline'] = {'value': v, 'unit': 'Fisher/s', 'cores': threads, 'kind': 'port',
                                'sample': '%d events, L1+H1+ETS, R=2000, float64 oracle (torch CPU)' % args.ref_events}
    print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == '__main__':
    main()
