"""ctypes binding of libgwfast_gb300.so (the C ABI declared in include/gwfast_gb300.h).

The library is built in-tree by ``gwfast_gb300._build.build()``.  There is no CPU
fallback: if the library or a CUDA device is missing, every call raises.
"""
import ctypes
import os
import threading

import numpy as np

from . import _build

GWF_OK = 0
ERRORS = {-1: 'invalid argument', -2: 'CUDA error', -3: 'out of memory', -4: 'timeout', -5: 'unsupported'}
MODEL_IDS = {'TaylorF2_RestrictedPN': 0, 'IMRPhenomD': 1, 'IMRPhenomHM': 2, 'IMRPhenomD_NRTidalv2': 4,
             'IMRPhenomNSBH': 7}
MODEL_TF2_TIDAL = 3
MODEL_TF2_ECC = 5
MODEL_TF2_TIDAL_ECC = 6
TF2_PHIREF_VLSO, TF2_KERR_ISCO, TF2_QUADMON_TIDAL = 1, 2, 4   # gwf_wf_desc.flags
MEM_HOST, MEM_DEVICE = 0, 1
PRECISION = {'fp64': 0, 'fp32': 1, 'mixed': 2}


class GWFError(RuntimeError):
    pass


class DetDesc(ctypes.Structure):
    _fields_ = [('lat_rad', ctypes.c_double), ('long_rad', ctypes.c_double), ('xax_rad', ctypes.c_double),
                ('shape', ctypes.c_int), ('earth_rotation', ctypes.c_int), ('fmin', ctypes.c_double),
                ('fmax', ctypes.c_double)]


class WfDesc(ctypes.Structure):
    _fields_ = [('model', ctypes.c_int), ('spin_ho', ctypes.c_int), ('fcut_par', ctypes.c_double),
                ('flags', ctypes.c_int), ('reserved', ctypes.c_int), ('fref_ecc', ctypes.c_double)]


_P = ctypes.POINTER
_d = ctypes.c_double
_i64 = ctypes.c_int64
_vp = ctypes.c_void_p

SIGNATURES = {
    'gwf_version': ([], ctypes.c_int),
    'gwf_last_error': ([], ctypes.c_char_p),
    'gwf_ctx_create': ([ctypes.c_int, _P(_vp)], ctypes.c_int),
    'gwf_ctx_destroy': ([_vp], ctypes.c_int),
    'gwf_set_qnm_table': ([_vp, _vp, _vp, _vp, _i64], ctypes.c_int),
    'gwf_detector_add': ([_vp, _P(DetDesc), _vp, _vp, _i64, _P(ctypes.c_int)], ctypes.c_int),
    'gwf_snr': ([_vp, ctypes.c_int, _vp, _P(WfDesc), _vp, _i64, _i64, ctypes.c_int32, _vp, ctypes.c_int,
                 ctypes.c_int, ctypes.c_int, _vp, _vp, _vp], ctypes.c_int),
    'gwf_fisher': ([_vp, ctypes.c_int, _vp, _P(WfDesc), _vp, _i64, _i64, ctypes.c_int32, _vp, ctypes.c_int,
                    ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp], ctypes.c_int),
    'gwf_fisher_ex': ([_vp, ctypes.c_int, _vp, _P(WfDesc), _vp, _i64, _i64, ctypes.c_int32, _vp, ctypes.c_int,
                       ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp, _vp, _vp], ctypes.c_int),
    'gwf_strain_derivs': ([_vp, ctypes.c_int, _P(WfDesc), _vp, _i64, _i64, ctypes.c_int32, ctypes.c_int, ctypes.c_int,
                           _vp, _vp], ctypes.c_int),
    'gwf_strain': ([_vp, ctypes.c_int, _P(WfDesc), _vp, _i64, _i64, _vp, _i64, ctypes.c_int32, ctypes.c_int, _vp, _vp,
                    _vp, _vp], ctypes.c_int),
    'gwf_overlap': ([_vp, ctypes.c_int, _vp, _P(WfDesc), _vp, _i64, _P(WfDesc), _vp, _i64, _i64, ctypes.c_int32,
                     ctypes.c_int, _vp, _vp, _vp, _vp], ctypes.c_int),
    'gwf_cov': ([_vp, _vp, _i64, ctypes.c_int, _vp, _vp, _vp, _vp], ctypes.c_int),
    'gwf_xitide': ([_vp, _vp, _vp, _vp, _i64, _vp], ctypes.c_int),
    'gwf_cov_n': ([_vp, _vp, _i64, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp, _vp], ctypes.c_int),
    'gwf_set_refine_cond': ([_vp, _d], ctypes.c_int),
    'gwf_set_segments': ([_vp, ctypes.c_int], ctypes.c_int),
    'gwf_set_detector_groups': ([_vp, ctypes.c_int], ctypes.c_int),
    'gwf_set_kernel_timing': ([_vp, ctypes.c_int], ctypes.c_int),
    'gwf_kernel_times': ([_vp, ctypes.c_int, _vp, _vp, _P(ctypes.c_int)], ctypes.c_int),
    'gwf_set_graphs': ([_vp, ctypes.c_int], ctypes.c_int),
    'gwf_autotune_segments': ([_vp, ctypes.c_int, _vp, _P(WfDesc), _vp, _i64, _i64, ctypes.c_int32, _vp, ctypes.c_int,
                               ctypes.c_int, ctypes.c_int, _P(ctypes.c_int)], ctypes.c_int),
    'gwf_mlp_create': ([_vp, ctypes.c_int, ctypes.c_int, ctypes.c_uint64, _P(_vp)], ctypes.c_int),
    'gwf_mlp_destroy': ([_vp], ctypes.c_int),
    'gwf_mlp_num_weights': ([_vp, _P(_i64)], ctypes.c_int),
    'gwf_mlp_get_weights': ([_vp, _vp, _vp], ctypes.c_int),
    'gwf_mlp_set_weights': ([_vp, _vp, _vp], ctypes.c_int),
    'gwf_mlp_train': ([_vp, _vp, _i64, _i64, _vp, ctypes.c_int, ctypes.c_int, _d, ctypes.c_uint64, ctypes.c_int,
                       _P(_d)], ctypes.c_int),
    'gwf_mlp_gradients': ([_vp, _vp, _i64, _i64, _vp, ctypes.c_int, _P(_d), _vp], ctypes.c_int),
    'gwf_mlp_predict': ([_vp, _vp, _i64, _i64, ctypes.c_int, _vp], ctypes.c_int),
    'gwf_fisher_noalloc': ([_P(DetDesc), _vp, _vp, _i64, _P(WfDesc), _vp, _vp, _vp, _i64, _vp, _i64, _i64,
                            ctypes.c_int32, ctypes.c_int, _vp, _vp], ctypes.c_int),
}

_lock = threading.Lock()
_lib = None
_ctxs = {}


def library_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load (building first if needed) the CUDA library; raises if it cannot be loaded."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if not os.path.exists(path) and build_if_missing:
            _build.build()
        if not os.path.exists(path):
            raise GWFError('libgwfast_gb300.so is missing; run gwfast_gb300._build.build()')
        lib = ctypes.CDLL(path)
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _lib = lib
        return lib


def check(rc):
    if rc != GWF_OK:
        msg = load().gwf_last_error().decode(errors='replace')
        raise GWFError('%s: %s' % (ERRORS.get(rc, rc), msg))


def ptr(a):
    """Address of a numpy array, a torch tensor or an integer device pointer."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if hasattr(a, 'data_ptr'):
        return a.data_ptr()
    return int(a)


def _qnm_table():
    here = os.path.dirname(os.path.abspath(__file__))
    return np.ascontiguousarray(np.loadtxt(os.path.join(here, 'data', 'qnm_220.txt')).T)


class Context:
    """One library context (device, PSD tables, staging buffers)."""

    def __init__(self, device=0):
        lib = load()
        h = _vp()
        check(lib.gwf_ctx_create(int(device), ctypes.byref(h)))
        self.h = h
        self.device = device
        q = _qnm_table()
        check(lib.gwf_set_qnm_table(self.h, ptr(q[0]), ptr(q[1]), ptr(q[2]), q.shape[1]))
        self._keep = [q]

    def add_detector(self, lat_rad, long_rad, xax_rad, shape, earth, fmin, fmax, psd_f, psd_S):
        psd_f = np.ascontiguousarray(psd_f, dtype=np.float64)
        psd_S = np.ascontiguousarray(psd_S, dtype=np.float64)
        d = DetDesc(lat_rad, long_rad, xax_rad, 0 if shape == 'L' else 1, int(bool(earth)), float(fmin),
                    -1.0 if fmax is None else float(fmax))
        out = ctypes.c_int()
        check(load().gwf_detector_add(self.h, ctypes.byref(d), ptr(psd_f), ptr(psd_S), len(psd_f), ctypes.byref(out)))
        return out.value

    def snr(self, det_ids, wf, params, res, res_ev=None, spacing=0, mem=MEM_HOST, out_arm=None, out_net=None,
            stream=None, ld=None, n=None, precision='fp64'):
        ids = np.ascontiguousarray(det_ids, dtype=np.int32)
        n = params.shape[1] if n is None else n
        ld = (params.shape[1] if ld is None else ld)
        check(load().gwf_snr(self.h, len(ids), ptr(ids), ctypes.byref(wf), ptr(params), ld, n, int(res),
                             ptr(res_ev), spacing, PRECISION[precision], mem, ptr(out_arm), ptr(out_net), stream))

    def fisher(self, det_ids, wf, params, res, res_ev=None, spacing=0, per_arm=False, mem=MEM_HOST, out_arm=None,
               out_net=None, stream=None, ld=None, n=None, precision='fp64', out_sd_arm=None, out_sd_net=None):
        ids = np.ascontiguousarray(det_ids, dtype=np.int32)
        n = params.shape[1] if n is None else n
        ld = (params.shape[1] if ld is None else ld)
        if out_sd_arm is None and out_sd_net is None:
            check(load().gwf_fisher(self.h, len(ids), ptr(ids), ctypes.byref(wf), ptr(params), ld, n, int(res),
                                    ptr(res_ev), spacing, int(bool(per_arm)), PRECISION[precision], mem, ptr(out_arm),
                                    ptr(out_net), stream))
        else:
            check(load().gwf_fisher_ex(self.h, len(ids), ptr(ids), ctypes.byref(wf), ptr(params), ld, n, int(res),
                                       ptr(res_ev), spacing, int(bool(per_arm)), PRECISION[precision], mem,
                                       ptr(out_arm), ptr(out_net), ptr(out_sd_arm), ptr(out_sd_net), stream))

    def strain_derivs(self, det_id, wf, params, res, spacing=0, mem=MEM_HOST, out=None, stream=None, ld=None,
                      n=None):
        """d h / d theta on each event's grid: out complex128 [arms][11][N][res] (arms 1 or 3)."""
        n = params.shape[1] if n is None else n
        ld = params.shape[1] if ld is None else ld
        check(load().gwf_strain_derivs(self.h, int(det_id), ctypes.byref(wf), ptr(params), ld, n, int(res), spacing,
                                       mem, ptr(out), stream))

    def strain(self, det_id, wf, params, freqs, out_strain=None, out_amp=None, out_phase=None, mem=MEM_HOST,
               stream=None, ld=None, n=None):
        """Strain, amplitudes and phases at caller frequencies: freqs float64 (R,) shared by all events or
        (N, R) per event; out_strain / out_amp complex128 [arms][N][R] (amp: A+ + i Ax), out_phase
        float64 [2][N][R] (GWPhase, the strain's phase)."""
        n = params.shape[1] if n is None else n
        ld = params.shape[1] if ld is None else ld
        R = freqs.shape[-1]
        f_ld = freqs.shape[-1] if freqs.ndim == 2 else 0
        check(load().gwf_strain(self.h, int(det_id), ctypes.byref(wf), ptr(params), ld, n, ptr(freqs), f_ld, int(R), mem,
                                ptr(out_strain), ptr(out_amp), ptr(out_phase), stream))

    def overlap(self, det_ids, wf1, params1, wf2, params2, res, mem=MEM_HOST, out_ov=None, out_n1=None, out_n2=None,
                stream=None, n=None):
        """Per-detector 4 trapz(Re(h1 conj h2)/S), 4 trapz(|h1|^2/S), 4 trapz(|h2|^2/S), each [n_det][N]."""
        ids = np.ascontiguousarray(det_ids, dtype=np.int32)
        n = params1.shape[1] if n is None else n
        check(load().gwf_overlap(self.h, len(ids), ptr(ids), ctypes.byref(wf1), ptr(params1), params1.shape[1],
                                 ctypes.byref(wf2), ptr(params2), params2.shape[1], n, int(res), mem, ptr(out_ov),
                                 ptr(out_n1), ptr(out_n2), stream))

    def set_graphs(self, on):
        """Capture repeated device-resident Fisher calls in CUDA graphs and replay them."""
        check(load().gwf_set_graphs(self.h, int(bool(on))))

    def set_detector_groups(self, on):
        """Network totals: evaluate detectors that share the grid in one launch, the waveform once per
        point (TaylorF2, IMRPhenomD, IMRPhenomHM; every precision; default on)."""
        check(load().gwf_set_detector_groups(self.h, int(bool(on))))

    KT_NAMES = {1: 'setup', 2: 'group_f32', 3: 'fisher_f32', 4: 'fisher_f64', 5: 'segmented'}

    def set_kernel_timing(self, on):
        """Record CUDA events around the main launches of the following calls (see kernel_times)."""
        check(load().gwf_set_kernel_timing(self.h, int(bool(on))))

    def kernel_times(self):
        """[(section, ms)] of the last call: set-up launches, group/per-detector Fisher launches."""
        kind = np.zeros(64, dtype=np.int32)
        ms = np.zeros(64, dtype=np.float64)
        n = ctypes.c_int()
        check(load().gwf_kernel_times(self.h, 64, ptr(kind), ptr(ms), ctypes.byref(n)))
        return [(self.KT_NAMES.get(int(k), str(int(k))), float(t)) for k, t in zip(kind[:n.value], ms[:n.value])]

    def set_segments(self, points):
        """0: one CTA per event; > 0: persistent launches over frequency segments of this many points."""
        check(load().gwf_set_segments(self.h, int(points)))

    def autotune_segments(self, det_ids, wf, params, res, res_ev=None, spacing=0, precision='fp64', mem=MEM_HOST,
                          ld=None, n=None):
        """Time the candidate segment lengths on this workload, keep and return the fastest."""
        ids = np.ascontiguousarray(det_ids, dtype=np.int32)
        n = params.shape[1] if n is None else n
        ld = params.shape[1] if ld is None else ld
        best = ctypes.c_int()
        check(load().gwf_autotune_segments(self.h, len(ids), ptr(ids), ctypes.byref(wf), ptr(params), ld, n, int(res),
                                           ptr(res_ev), spacing, PRECISION[precision], mem, ctypes.byref(best)))
        return best.value

    def set_refine_cond(self, kappa):
        """Condition-number threshold above which the 'mixed' form recomputes an event in FP64."""
        check(load().gwf_set_refine_cond(self.h, float(kappa)))

    def cov(self, F, mem=MEM_HOST, cov=None, eps=None, cond=None, n=None, stream=None, n_params=11):
        n = F.shape[0] if n is None else n
        check(load().gwf_cov_n(self.h, ptr(F), n, int(n_params), mem, ptr(cov), ptr(eps), ptr(cond), stream))

    def xitide(self, comp, q, chi_bh):
        """IMRPhenomNSBH's interpolated xi_tide at the given (compactness, m1/m2, BH spin) points."""
        c, qq, x = (np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1)) for a in (comp, q, chi_bh))
        out = np.empty(c.shape[0])
        check(load().gwf_xitide(self.h, ptr(c), ptr(qq), ptr(x), c.shape[0], ptr(out)))
        return out


def context(device=0):
    """Process-wide context for ``device`` (created on first use)."""
    with _lock:
        c = _ctxs.get(device)
    if c is None:
        c = Context(device)
        with _lock:
            _ctxs[device] = c
    return c


class MLP:
    """The library's SNR-screen network (gwf_mlp_*): 11 features -> hidden SiLU layers -> ln SNR."""

    def __init__(self, hidden=256, layers=4, seed=0, device=0):
        lib = load()
        self._ctx = context(device)
        h = _vp()
        check(lib.gwf_mlp_create(self._ctx.h, int(hidden), int(layers), int(seed), ctypes.byref(h)))
        self.h = h
        self.hidden, self.layers = hidden, layers
        n = ctypes.c_int64()
        check(lib.gwf_mlp_num_weights(self.h, ctypes.byref(n)))
        self.n_weights = n.value

    def __del__(self):
        h = getattr(self, 'h', None)
        if h is not None and _lib is not None:
            _lib.gwf_mlp_destroy(h)
            self.h = None

    def get_weights(self):
        w = np.empty(self.n_weights, dtype=np.float32)
        check(load().gwf_mlp_get_weights(self.h, ptr(w), None))
        return w

    def get_norm(self):
        nm = np.empty(22, dtype=np.float32)
        check(load().gwf_mlp_get_weights(self.h, None, ptr(nm)))
        return nm

    def set_weights(self, w=None, norm=None):
        w = None if w is None else np.ascontiguousarray(w, dtype=np.float32)
        norm = None if norm is None else np.ascontiguousarray(norm, dtype=np.float32)
        check(load().gwf_mlp_set_weights(self.h, ptr(w), ptr(norm)))

    def train(self, params, target, epochs=30, batch=4096, lr=2e-3, seed=0):
        params = np.ascontiguousarray(params, dtype=np.float64)
        target = np.ascontiguousarray(target, dtype=np.float64)
        loss = ctypes.c_double()
        check(load().gwf_mlp_train(self.h, ptr(params), params.shape[1], params.shape[1], ptr(target), int(epochs),
                                   int(batch), float(lr), int(seed), MEM_HOST, ctypes.byref(loss)))
        return loss.value

    def gradients(self, params, target):
        params = np.ascontiguousarray(params, dtype=np.float64)
        target = np.ascontiguousarray(target, dtype=np.float64)
        g = np.empty(self.n_weights, dtype=np.float32)
        loss = ctypes.c_double()
        check(load().gwf_mlp_gradients(self.h, ptr(params), params.shape[1], params.shape[1], ptr(target), MEM_HOST,
                                       ctypes.byref(loss), ptr(g)))
        return loss.value, g

    def predict(self, params):
        params = np.ascontiguousarray(params, dtype=np.float64)
        out = np.empty(params.shape[1])
        check(load().gwf_mlp_predict(self.h, ptr(params), params.shape[1], params.shape[1], MEM_HOST, ptr(out)))
        return out
