// C-ABI layer: context, detector tables, staging and launches (see include/gwfast_gb300.h).
#include <cuda_runtime.h>
#include <sys/mman.h>
#include <unistd.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "gwf_launch.h"
#include "gwfast_gb300.h"

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define GWF_CK(x)                                                                               \
  do {                                                                                          \
    cudaError_t e_ = (x);                                                                       \
    if (e_ != cudaSuccess) return fail(GWF_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
  } while (0)

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  int ensure(size_t bytes) {
    if (bytes <= cap) return 0;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    if (cudaMalloc(&p, bytes) != cudaSuccess) return -1;
    cap = bytes;
    return 0;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
};

struct HostBuf {
  void* p = nullptr;
  size_t cap = 0;
  int ensure(size_t bytes) {
    if (bytes <= cap) return 0;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    if (cudaMallocHost(&p, bytes) != cudaSuccess) return -1;
    cap = bytes;
    return 0;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
  }
};

struct DetRec {
  gwf_det_desc desc;
  double* d_f = nullptr;
  double* d_S = nullptr;
  int* d_acc = nullptr;
  float4* d_seg = nullptr;
  int n = 0, nacc = 0;
  double l0 = 0.0, idl = 0.0, scale = 1.0;
  int psd_class = 0;   // id of the first detector added with an identical PSD table
  std::vector<double> h_f, h_S;
};

struct GraphEntry {
  cudaGraphExec_t exec;
  std::string bufs;   // buffer_sig at capture time
};

}  // namespace

namespace gwf {
// error text for gwf_last_error from the other translation units
void set_last_error(const char* msg) { g_err = msg; }
int ctx_device(const gwf_ctx* ctx);
}  // namespace gwf

struct gwf_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<DetRec> dets;
  double* d_qnm = nullptr;
  int nq = 0;
  DevBuf par, res, oarm, onet, fin, fout, feps, fcond, setup;
  DevBuf mix_idx, mix_cnt, mix_par, mix_res, mix_net, mix_arm;  // FP64 recomputation of GWF_PREC_MIXED
  // below 1e13 the FP32 form's marginalised errors are within 1e-4 of FP64 on every event of the
  // IMRPhenomD headline workload (max 7.0e-5 with either threshold 1e12 or 1e13)
  double refine_cond = 1e13;
  int seg_points = 0;      // Fisher launches: 0 = one CTA per event, > 0 = persistent, segments of this many points
  // segment length of the FP64 recomputation of GWF_PREC_MIXED: one point per thread (few events,
  // each thread's FP64 chain is the latency; 15 events of 10^4 at R = 2000: the recomputation took
  // 1.16 ms of stream time at 256 points per segment, 0.79 ms at 128 with the grid capped)
  int refine_seg = 128;
  DevBuf seg_off, seg_ctr, seg_part, seg_ovf, tune_out;
  // SNR-derivative outputs of the current gwf_fisher_ex call (host or device pointers, as mem says)
  double* call_sd_arm = nullptr;
  double* call_sd_net = nullptr;
  DevBuf osda, osdn, mix_sda, mix_sdn;
  int graphs = 0;                                  // capture device-resident Fisher calls in CUDA graphs
  std::map<std::string, GraphEntry> graph_cache;   // call identity -> instantiated graph
  std::string graph_pending;                       // identity of the last uncaptured call
  int64_t graph_rmax = 0;
  cudaEvent_t scratch_free = nullptr;  // recorded after the last launch that used the set-up scratch
  HostBuf hpar, hout;
  DevBuf wbuf, par2, fcutb, ovb;   // strain-tangent and overlap outputs
  DevBuf sfreq, samp, sph, srange;   // gwf_strain: caller frequencies, amplitude and phase staging, row ranges
  DevBuf core;                     // source-dependent model records, shared by the detectors of a call
  int groups = 1;                  // FP32 network totals: detectors sharing the grid in one launch
  DevBuf xit;                      // IMRPhenomNSBH xi_tide table, built on first use
  bool xit_ready = false;
  // GWF_PREC_MIXED recomputation: one stream per detector, so that the detectors' FP64 passes over
  // the few ill-conditioned events run side by side; per-detector scratch and segment buffers
  std::vector<cudaStream_t> aux;
  std::vector<cudaEvent_t> aux_done;
  cudaEvent_t fork = nullptr;
  DevBuf mix_scr, mix_soff, mix_sctr, mix_spart, mix_sovf;
  // detector groups of one call side by side (each on an aux stream after the first, which runs on
  // the call's stream and fills the source-record cache): per-group network totals, summed at the end
  cudaEvent_t core_ev = nullptr;
  DevBuf gnet;
  // gwf_set_kernel_timing: events around the main sections of the last call
  gwf::KernelTimer* ktimer = nullptr;
  bool ktiming = false;
};

namespace {

// Map every page of a host output buffer before a device-to-host copy into it. A buffer the caller
// has just allocated is not mapped yet; the copy would then take its page faults one by one inside
// the driver (~1 ms per MB measured on the GB300 host), while mapping them here first is several
// times cheaper: one madvise(MADV_POPULATE_WRITE) (Linux 5.14+), or else a touch per page that
// writes back the byte it read, so the contents are unchanged either way.
#ifndef MADV_POPULATE_WRITE
#define MADV_POPULATE_WRITE 23
#endif
void prefault_host(void* p, size_t bytes) {
  if (!p || !bytes) return;
  static const size_t page = [] { long s = sysconf(_SC_PAGESIZE); return s > 0 ? (size_t)s : (size_t)4096; }();
  const uintptr_t a = reinterpret_cast<uintptr_t>(p) & ~(uintptr_t)(page - 1);
  const size_t len = ((reinterpret_cast<uintptr_t>(p) + bytes - a) + page - 1) & ~(page - 1);
  if (madvise(reinterpret_cast<void*>(a), len, MADV_POPULATE_WRITE) == 0) return;
  volatile unsigned char* c = reinterpret_cast<volatile unsigned char*>(p);
  for (size_t i = 0; i < bytes; i += page) c[i] = c[i];
  c[bytes - 1] = c[bytes - 1];
}

// Fisher parameters of a waveform model: 11; 13 for the tidal models (LambdaTilde, deltaLambda); the
// eccentric TaylorF2 adds ecc (12, or 14 with the tidal terms)
int npar_of(int model) {
  return model == GWF_WF_TAYLORF2_ECC ? 12 : (model == GWF_WF_TAYLORF2_TIDAL_ECC ? 14 : (model >= GWF_WF_TAYLORF2_TIDAL ? 13 : 11));
}

// per-model entry points of the FP64 launch code (one translation unit per model)
size_t setup_stride_any(int model) {
  switch (model) {
    case 0: return gwf::setup_stride_m0();
    case 1: return gwf::setup_stride_m1();
    case 2: return gwf::setup_stride_m2();
    case 3: return gwf::setup_stride_m3();
    case 4: return gwf::setup_stride_m4();
    case 5: return gwf::setup_stride_m5();
    case 6: return gwf::setup_stride_m6();
    default: return gwf::setup_stride_m7();
  }
}
size_t core_bytes_any(int model) {
  switch (model) {
    case 0: return gwf::core_bytes_m0();
    case 1: return gwf::core_bytes_m1();
    case 2: return gwf::core_bytes_m2();
    case 3: return gwf::core_bytes_m3();
    case 4: return gwf::core_bytes_m4();
    case 5: return gwf::core_bytes_m5();
    case 6: return gwf::core_bytes_m6();
    default: return gwf::core_bytes_m7();
  }
}
cudaError_t launch_fisher_any(int model, const gwf::LaunchArgs& a) {
  switch (model) {
    case 0: return gwf::launch_fisher_m0(a);
    case 1: return gwf::launch_fisher_m1(a);
    case 2: return gwf::launch_fisher_m2(a);
    case 3: return gwf::launch_fisher_m3(a);
    case 4: return gwf::launch_fisher_m4(a);
    case 5: return gwf::launch_fisher_m5(a);
    case 6: return gwf::launch_fisher_m6(a);
    default: return gwf::launch_fisher_m7(a);
  }
}
cudaError_t launch_snr_any(int model, const gwf::LaunchArgs& a) {
  switch (model) {
    case 0: return gwf::launch_snr_m0(a);
    case 1: return gwf::launch_snr_m1(a);
    case 2: return gwf::launch_snr_m2(a);
    case 3: return gwf::launch_snr_m3(a);
    case 4: return gwf::launch_snr_m4(a);
    case 5: return gwf::launch_snr_m5(a);
    case 6: return gwf::launch_snr_m6(a);
    default: return gwf::launch_snr_m7(a);
  }
}

// the IMRPhenomNSBH xi_tide table (64 MiB), built on the device the first time it is needed, ordered
// on the stream of the call that needs it
int ensure_xitide(gwf_ctx* ctx, cudaStream_t st) {
  if (ctx->xit_ready) return GWF_OK;
  const size_t bytes = (size_t)gwf::kXiN * gwf::kXiN * gwf::kXiN * sizeof(double);
  if (ctx->xit.ensure(bytes)) return fail(GWF_ERR_OOM, "device allocation failed (xi_tide table)");
  cudaError_t e = gwf::launch_xitide_table((double*)ctx->xit.p, st);
  if (e != cudaSuccess) return fail(GWF_ERR_CUDA, std::string("xi_tide table: ") + cudaGetErrorString(e));
  ctx->xit_ready = true;
  return GWF_OK;
}

bool is_tf2_model(int model) {
  return model == GWF_WF_TAYLORF2 || model == GWF_WF_TAYLORF2_TIDAL || model == GWF_WF_TAYLORF2_ECC ||
         model == GWF_WF_TAYLORF2_TIDAL_ECC;
}

gwf::WfDesc wf_dev(const gwf_wf_desc* wf) {
  gwf::WfDesc w;
  w.model = wf->model;
  w.spin_ho = wf->spin_ho;
  w.fcut_par = wf->fcut_par;
  w.flags = wf->flags;
  w.pad_ = 0;
  w.fref_ecc = wf->fref_ecc;
  return w;
}

int check_ctx(gwf_ctx* ctx) {
  if (!ctx) return fail(GWF_ERR_INVALID_ARG, "null context");
  GWF_CK(cudaSetDevice(ctx->device));
  return GWF_OK;
}

int slots_of(const gwf_ctx* ctx, int n_det, const int* ids) {
  int s = 0;
  for (int i = 0; i < n_det; ++i) s += ctx->dets[ids[i]].desc.shape == GWF_SHAPE_T ? 3 : 1;
  return s;
}

gwf::DetDev dev_of(const DetRec& r) {
  gwf::DetDev d;
  d.lat = r.desc.lat_rad;
  d.lon = r.desc.long_rad;
  d.xax = r.desc.xax_rad;
  d.shape = r.desc.shape;
  d.sin_zeta = r.desc.shape == GWF_SHAPE_T ? std::sin(M_PI / 3.0) : 1.0;
  d.fmin = r.desc.fmin;
  d.fmax = r.desc.fmax;
  d.earth = r.desc.earth_rotation;
  d.psd_f = r.d_f;
  d.psd_S = r.d_S;
  d.npsd = r.n;
  d.acc = r.d_acc;
  d.nacc = r.nacc;
  d.acc_l0 = r.l0;
  d.acc_idl = r.idl;
  d.psd_seg = r.d_seg;
  d.psd_f32_lo = r.n > 0 ? (float)r.h_f.front() : 0.0f;
  d.psd_f32_hi = r.n > 0 ? (float)r.h_f.back() : 0.0f;
  d.psd_scale = r.scale;
  gwf::det_trig(d);
  return d;
}

int validate_common(gwf_ctx* ctx, int n_det, const int* det_ids, const gwf_wf_desc* wf, const double* params,
                    int64_t ld, int64_t N, int32_t res, const int32_t* res_ev, int spacing, int mem) {
  if (!det_ids || n_det < 1) return fail(GWF_ERR_INVALID_ARG, "need at least one detector");
  for (int i = 0; i < n_det; ++i)
    if (det_ids[i] < 0 || det_ids[i] >= (int)ctx->dets.size()) return fail(GWF_ERR_INVALID_ARG, "unknown detector id");
  if (!wf || wf->model < 0 || wf->model > GWF_WF_PHENOMNSBH) return fail(GWF_ERR_INVALID_ARG, "unknown waveform model");
  if (wf->flags & ~(GWF_TF2_PHIREF_VLSO | GWF_TF2_KERR_ISCO | GWF_TF2_QUADMON_TIDAL))
    return fail(GWF_ERR_INVALID_ARG, "unknown waveform flags");
  if (wf->flags && !is_tf2_model(wf->model))
    return fail(GWF_ERR_INVALID_ARG, "waveform flags apply to the TaylorF2 models only");
  if ((wf->flags & GWF_TF2_QUADMON_TIDAL) && wf->model != GWF_WF_TAYLORF2_TIDAL && wf->model != GWF_WF_TAYLORF2_TIDAL_ECC)
    return fail(GWF_ERR_INVALID_ARG, "GWF_TF2_QUADMON_TIDAL needs a tidal TaylorF2 model");
  if ((wf->model == GWF_WF_PHENOMD || wf->model == GWF_WF_PHENOMD_NRTIDALV2 || wf->model == GWF_WF_PHENOMNSBH) &&
      ctx->nq < 2)
    return fail(GWF_ERR_INVALID_ARG, "IMRPhenomD needs the QNM table (gwf_set_qnm_table)");
  if (!(wf->fcut_par > 0.0)) return fail(GWF_ERR_INVALID_ARG, "fcut_par must be positive");
  if (N < 0 || (N > 0 && !params)) return fail(GWF_ERR_INVALID_ARG, "bad event array");
  if (ld < N) return fail(GWF_ERR_INVALID_ARG, "ld must be >= n_events");
  if (!res_ev && res < 1) return fail(GWF_ERR_INVALID_ARG, "res must be >= 1");
  if (spacing != GWF_SPACING_GEOM && spacing != GWF_SPACING_LIN) return fail(GWF_ERR_INVALID_ARG, "bad spacing");
  if (mem != GWF_MEM_HOST && mem != GWF_MEM_DEVICE) return fail(GWF_ERR_INVALID_ARG, "bad memory mode");
  if (N > (int64_t)1 << 40) return fail(GWF_ERR_INVALID_ARG, "too many events");
  return GWF_OK;
}

int stage_inputs_to(gwf_ctx* ctx, DevBuf& par, const double* params, int64_t ld, int64_t N, const int32_t* res_ev,
                    int mem, cudaStream_t st, const double** dp, int64_t* dld, const int** dres, int npar = gwf::NP);

// stage host inputs into device buffers; returns device pointers
int stage_inputs(gwf_ctx* ctx, const double* params, int64_t ld, int64_t N, const int32_t* res_ev, int mem,
                 cudaStream_t st, const double** dp, int64_t* dld, const int** dres, int npar = gwf::NP) {
  return stage_inputs_to(ctx, ctx->par, params, ld, N, res_ev, mem, st, dp, dld, dres, npar);
}

int stage_inputs_to(gwf_ctx* ctx, DevBuf& par, const double* params, int64_t ld, int64_t N, const int32_t* res_ev,
                    int mem, cudaStream_t st, const double** dp, int64_t* dld, const int** dres, int npar) {
  if (mem == GWF_MEM_DEVICE) {
    *dp = params;
    *dld = ld;
    *dres = res_ev;
    return GWF_OK;
  }
  const size_t pb = (size_t)npar * (size_t)N * sizeof(double);
  if (par.ensure(pb ? pb : 8)) return fail(GWF_ERR_OOM, "device allocation failed (params)");
  if (N > 0) {
    if (ld == N) GWF_CK(cudaMemcpyAsync(par.p, params, pb, cudaMemcpyHostToDevice, st));
    else GWF_CK(cudaMemcpy2DAsync(par.p, N * sizeof(double), params, ld * sizeof(double), N * sizeof(double),
                                  npar, cudaMemcpyHostToDevice, st));
  }
  *dp = (const double*)par.p;
  *dld = N;
  *dres = nullptr;
  if (res_ev) {
    if (ctx->res.ensure((size_t)N * sizeof(int) + 4)) return fail(GWF_ERR_OOM, "device allocation failed (res)");
    GWF_CK(cudaMemcpyAsync(ctx->res.p, res_ev, (size_t)N * sizeof(int), cudaMemcpyHostToDevice, st));
    *dres = (const int*)ctx->res.p;
  }
  return GWF_OK;
}

// largest per-event resolution of a call (bounds the number of segments per event)
int max_res(int32_t res, const int32_t* res_ev, int64_t N, int mem, int64_t* out) {
  if (!res_ev) { *out = res; return GWF_OK; }
  int64_t m = 1;
  if (mem == GWF_MEM_HOST) {
    for (int64_t i = 0; i < N; ++i) m = res_ev[i] > m ? res_ev[i] : m;
  } else {
    std::vector<int32_t> h((size_t)N);
    GWF_CK(cudaMemcpy(h.data(), res_ev, (size_t)N * sizeof(int32_t), cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < N; ++i) m = h[i] > m ? h[i] : m;
  }
  *out = m;
  return GWF_OK;
}

// buffers of the segmented launches for chunks of up to `chunk` events with at most rmax points
int seg_setup(gwf_ctx* ctx, gwf::LaunchArgs& a, int seg, int64_t chunk, int64_t rmax, cudaStream_t st) {
  const long long per_ev = (long long)((rmax + seg - 1) / seg);
  const long long cap = (long long)chunk * (per_ev > 0 ? per_ev : 1);
  if (ctx->seg_off.ensure((size_t)(gwf::kChunk + 1) * sizeof(long long)) ||
      ctx->seg_ctr.ensure(sizeof(unsigned long long)) || ctx->seg_ovf.ensure(sizeof(int)) ||
      ctx->seg_part.ensure((size_t)cap * 3 * gwf::NEX * sizeof(double)))
    return fail(GWF_ERR_OOM, "device allocation failed (segments)");
  GWF_CK(cudaMemsetAsync(ctx->seg_ovf.p, 0, sizeof(int), st));
  a.seg = seg;
  a.seg_off = (long long*)ctx->seg_off.p;
  a.seg_ctr = (unsigned long long*)ctx->seg_ctr.p;
  a.seg_part = (double*)ctx->seg_part.p;
  a.seg_cap = cap;
  a.seg_ovf = (int*)ctx->seg_ovf.p;
  return GWF_OK;
}

int ensure_aux(gwf_ctx* ctx, int n) {
  if (!ctx->fork) GWF_CK(cudaEventCreateWithFlags(&ctx->fork, cudaEventDisableTiming));
  while ((int)ctx->aux.size() < n) {
    cudaStream_t s;
    cudaEvent_t e;
    GWF_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
      cudaStreamDestroy(s);
      return fail(GWF_ERR_CUDA, "event creation failed");
    }
    ctx->aux.push_back(s);
    ctx->aux_done.push_back(e);
  }
  return GWF_OK;
}

// GWF_PREC_MIXED, second stage: condition numbers of the FP32 network Fishers, then the FP64
// Fisher of the events above the threshold, computed as a compact batch (the detectors side by side
// on their own streams) and scattered back
// recs[i]: where the first pass left detector i's FP64 set-up records for the whole batch, or null;
// patch[i]: those are another detector's records (same grid and model), to be given detector i's
// projection header
int refine(gwf_ctx* ctx, int n_det, const int* det_ids, gwf::LaunchArgs a, const double* dp, int64_t dld,
           const int* dres, int64_t N, int slots, double* darm, double* dnet, double* dsda, double* dsdn,
           bool core_filled, const std::vector<const unsigned char*>& recs, const std::vector<int>& patch,
           cudaStream_t st) {
  const size_t per = (size_t)gwf::NP * gwf::NP;
  if (ctx->fcond.ensure((size_t)N * sizeof(double)) || ctx->mix_idx.ensure((size_t)N * sizeof(long long)) ||
      ctx->mix_cnt.ensure(sizeof(unsigned long long)))
    return fail(GWF_ERR_OOM, "device allocation failed (mixed precision)");
  long long* idx = (long long*)ctx->mix_idx.p;
  cudaError_t e = gwf::launch_cond(dnet, N, (double*)ctx->fcond.p, st);
  if (e == cudaSuccess)
    e = gwf::launch_select((const double*)ctx->fcond.p, N, ctx->refine_cond, idx, (unsigned long long*)ctx->mix_cnt.p, st);
  unsigned long long M = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&M, ctx->mix_cnt.p, sizeof(M), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail(GWF_ERR_CUDA, std::string("mixed precision: ") + cudaGetErrorString(e));
  if (M == 0) return GWF_OK;
  if (ctx->mix_par.ensure(M * gwf::NP * sizeof(double)) || ctx->mix_net.ensure((size_t)n_det * M * per * sizeof(double)) ||
      (dres && ctx->mix_res.ensure(M * sizeof(int))) || (darm && ctx->mix_arm.ensure((size_t)slots * M * per * sizeof(double))))
    return fail(GWF_ERR_OOM, "device allocation failed (mixed precision)");
  double* cpar = (double*)ctx->mix_par.p;
  double* cnet = (double*)ctx->mix_net.p;
  double* carm = darm ? (double*)ctx->mix_arm.p : nullptr;
  int* cres = dres ? (int*)ctx->mix_res.p : nullptr;
  if ((dsda && ctx->mix_sda.ensure((size_t)slots * M * gwf::NP * sizeof(double))) ||
      (dsdn && ctx->mix_sdn.ensure((size_t)n_det * M * gwf::NP * sizeof(double))))
    return fail(GWF_ERR_OOM, "device allocation failed (mixed precision)");
  double* csda = dsda ? (double*)ctx->mix_sda.p : nullptr;
  double* csdn = dsdn ? (double*)ctx->mix_sdn.p : nullptr;
  e = gwf::launch_gather(dp, dld, dres, idx, (long long)M, cpar, cres, st);
  if (e != cudaSuccess) return fail(GWF_ERR_CUDA, cudaGetErrorString(e));
  a.ev.p = cpar;
  a.ev.ld = (long long)M;
  a.ev.N = (long long)M;
  a.ev.res_ev = cres;
  a.precision = GWF_PREC_FP64;
  // the source records of these events are in the cache when the first pass filled it
  a.core = core_filled ? (unsigned char*)ctx->core.p : nullptr;
  a.core_mode = core_filled ? 2 : 0;
  a.core_idx = core_filled ? idx : nullptr;
  // few events: split each into frequency segments so that they fill the GPU
  int64_t rmax = a.ev.res;
  if (dres) {
    int rc = max_res(a.ev.res, dres, N, GWF_MEM_DEVICE, &rmax);
    if (rc) return rc;
  }
  // per-detector scratch and segment buffers
  const int64_t chunk = (int64_t)M < gwf::kChunk ? (int64_t)M : gwf::kChunk;
  const int seg = ctx->refine_seg;
  const long long per_ev = (long long)((rmax + seg - 1) / seg);
  const long long cap = (long long)chunk * (per_ev > 0 ? per_ev : 1);
  const size_t stride = setup_stride_any(a.wf.model);
  if (ctx->mix_scr.ensure((size_t)n_det * chunk * stride) ||
      ctx->mix_soff.ensure((size_t)n_det * (gwf::kChunk + 1) * sizeof(long long)) ||
      ctx->mix_sctr.ensure((size_t)n_det * sizeof(unsigned long long)) ||
      ctx->mix_spart.ensure((size_t)n_det * cap * 3 * gwf::NEX * sizeof(double)) ||
      ctx->mix_sovf.ensure((size_t)n_det * sizeof(int)))
    return fail(GWF_ERR_OOM, "device allocation failed (mixed precision)");
  int rc = ensure_aux(ctx, n_det);
  if (rc) return rc;
  GWF_CK(cudaMemsetAsync(ctx->mix_sovf.p, 0, (size_t)n_det * sizeof(int), st));
  // network totals only: the detectors that share the grid run as one FP64 group launch (the waveform
  // once per point), on the first member's stream, its network total in that member's slice
  std::vector<std::vector<int>> rg;
  const bool rgroup = ctx->groups && !carm && !csda && !csdn && a.wf.model <= GWF_WF_PHENOMHM;
  for (int i = 0; i < n_det; ++i) {
    const gwf_det_desc& di = ctx->dets[det_ids[i]].desc;
    bool placed = false;
    for (auto& g : rg) {
      const gwf_det_desc& d0 = ctx->dets[det_ids[g[0]]].desc;
      if (rgroup && (int)g.size() < gwf::kMaxGroup && d0.fmin == di.fmin && d0.fmax == di.fmax &&
          d0.earth_rotation == di.earth_rotation) {
        g.push_back(i);
        placed = true;
        break;
      }
    }
    if (!placed) rg.push_back({i});
  }
  GWF_CK(cudaEventRecord(ctx->fork, st));
  int slot = 0;
  for (auto& grp : rg) {
    const int i = grp[0];
    const DetRec& r = ctx->dets[det_ids[i]];
    gwf::LaunchArgs ai = a;
    ai.stream = ctx->aux[i];
    GWF_CK(cudaStreamWaitEvent(ai.stream, ctx->fork, 0));
    ai.det = dev_of(r);
    if (recs[i]) {   // copy the records of these events instead of recomputing them
      ai.rec_src = recs[i];
      ai.rec_patch_proj = patch[i];
      ai.core_idx = idx;
    }
    ai.scratch = (unsigned char*)ctx->mix_scr.p + (size_t)i * chunk * stride;
    ai.cap_events = chunk;
    ai.seg = seg;
    ai.seg_off = (long long*)ctx->mix_soff.p + (size_t)i * (gwf::kChunk + 1);
    ai.seg_ctr = (unsigned long long*)ctx->mix_sctr.p + i;
    ai.seg_part = (double*)ctx->mix_spart.p + (size_t)i * cap * 3 * gwf::NEX;
    ai.seg_cap = cap;
    ai.seg_ovf = (int*)ctx->mix_sovf.p + i;
    ai.out_arm = carm ? carm + (size_t)slot * M * per : nullptr;
    ai.out_det = cnet + (size_t)i * M * per;
    ai.out_sd_arm = csda ? csda + (size_t)slot * M * gwf::NP : nullptr;
    ai.out_sd_det = csdn ? csdn + (size_t)i * M * gwf::NP : nullptr;
    ai.accum = 0;
    if (grp.size() > 1) {
      gwf::Group64 G;
      G.nd = (int)grp.size();
      for (int d = 0; d < G.nd; ++d) {
        const int m = grp[d];
        G.det[d] = dev_of(ctx->dets[det_ids[m]]);
        G.same_psd[d] = d > 0 && ctx->dets[det_ids[m]].psd_class == ctx->dets[det_ids[grp[d - 1]]].psd_class;
        G.scratch[d] = (unsigned char*)ctx->mix_scr.p + (size_t)m * chunk * stride;
        G.rec_src[d] = recs[m];
        G.patch[d] = patch[m];
        if (recs[m]) ai.core_idx = idx;
        if (d > 0) GWF_CK(cudaMemsetAsync(cnet + (size_t)m * M * per, 0, (size_t)M * per * sizeof(double), ai.stream));
      }
      e = ai.wf.model == 0 ? gwf::launch_group64_m0(ai, G)
                           : (ai.wf.model == 1 ? gwf::launch_group64_m1(ai, G) : gwf::launch_group64_m2(ai, G));
    } else {
      e = launch_fisher_any(ai.wf.model, ai);
    }
    if (e != cudaSuccess) return fail(GWF_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    GWF_CK(cudaEventRecord(ctx->aux_done[i], ai.stream));
    for (int m : grp) slot += ctx->dets[det_ids[m]].desc.shape == GWF_SHAPE_T ? 3 : 1;
  }
  for (auto& grp : rg) GWF_CK(cudaStreamWaitEvent(st, ctx->aux_done[grp[0]], 0));
  e = gwf::launch_sum_scatter(cnet, n_det, (long long)M * per, idx, (long long)M, (int)per, dnet, st);
  for (int s = 0; carm && s < slots && e == cudaSuccess; ++s)
    e = gwf::launch_scatter(carm + (size_t)s * M * per, idx, (long long)M, (int)per, darm + (size_t)s * N * per, st);
  if (csdn && e == cudaSuccess)
    e = gwf::launch_sum_scatter(csdn, n_det, (long long)M * gwf::NP, idx, (long long)M, gwf::NP, dsdn, st);
  for (int s = 0; csda && s < slots && e == cudaSuccess; ++s)
    e = gwf::launch_scatter(csda + (size_t)s * M * gwf::NP, idx, (long long)M, gwf::NP,
                            dsda + (size_t)s * N * gwf::NP, st);
  if (e != cudaSuccess) return fail(GWF_ERR_CUDA, cudaGetErrorString(e));
  return GWF_OK;
}

int run_body(gwf_ctx* ctx, bool fisher, int n_det, const int* det_ids, const gwf_wf_desc* wf, const double* params,
             int64_t ld, int64_t N, int32_t res, const int32_t* res_ev, int spacing, int per_arm, int precision,
             int mem, double* out_arm, double* out_net, cudaStream_t st, bool capturing);

// a call's identity for the graph cache: every argument, pointers included
std::string graph_key(int n_det, const int* det_ids, const gwf_wf_desc* wf, const double* params, int64_t ld,
                      int64_t N, int32_t res, const int32_t* res_ev, int spacing, int per_arm, int precision,
                      const double* out_arm, const double* out_net, cudaStream_t st, const double* sd_arm,
                      const double* sd_net) {
  std::string k;
  auto add = [&](const void* p, size_t n) { k.append(reinterpret_cast<const char*>(p), n); };
  add(&n_det, sizeof n_det);
  add(det_ids, sizeof(int) * (size_t)n_det);
  add(wf, sizeof(*wf));
  add(&params, sizeof params); add(&ld, sizeof ld); add(&N, sizeof N); add(&res, sizeof res); add(&res_ev, sizeof res_ev);
  add(&spacing, sizeof spacing); add(&per_arm, sizeof per_arm); add(&precision, sizeof precision);
  add(&out_arm, sizeof out_arm); add(&out_net, sizeof out_net); add(&st, sizeof st);
  add(&sd_arm, sizeof sd_arm); add(&sd_net, sizeof sd_net);
  return k;
}

// the context buffers a captured graph refers to
std::string buffer_sig(const gwf_ctx* ctx) {
  const void* p[] = {ctx->setup.p, ctx->seg_off.p, ctx->seg_ctr.p, ctx->seg_part.p, ctx->seg_ovf.p, ctx->core.p};
  std::string k(reinterpret_cast<const char*>(p), sizeof p);
  k.append(reinterpret_cast<const char*>(&ctx->seg_points), sizeof ctx->seg_points);
  return k;
}

int run(gwf_ctx* ctx, bool fisher, int n_det, const int* det_ids, const gwf_wf_desc* wf, const double* params,
        int64_t ld, int64_t N, int32_t res, const int32_t* res_ev, int spacing, int per_arm, int precision, int mem,
        double* out_arm, double* out_net, void* stream) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  rc = validate_common(ctx, n_det, det_ids, wf, params, ld, N, res, res_ev, spacing, mem);
  if (rc) return rc;
  if (!out_arm && !out_net) return fail(GWF_ERR_INVALID_ARG, "no output requested");
  if (precision != GWF_PREC_FP64 && precision != GWF_PREC_FP32 && precision != GWF_PREC_MIXED)
    return fail(GWF_ERR_INVALID_ARG, "bad precision");
  if (precision != GWF_PREC_FP64 && wf->model >= GWF_WF_TAYLORF2_TIDAL)
    return fail(GWF_ERR_UNSUPPORTED, "the tidal models are implemented in FP64");
  if (precision == GWF_PREC_MIXED && !fisher) return fail(GWF_ERR_INVALID_ARG, "the mixed form is a Fisher form");
  if (fisher && !per_arm) out_arm = nullptr;
  if (fisher && per_arm && !out_arm) return fail(GWF_ERR_INVALID_ARG, "per_arm needs out_arm");
  if (!fisher && (ctx->call_sd_arm || ctx->call_sd_net)) return fail(GWF_ERR_INVALID_ARG, "SNR derivatives come with the Fisher");
  if (N == 0) return GWF_OK;
  for (int j = 0; j < N && res_ev && mem == GWF_MEM_HOST; ++j)
    if (res_ev[j] < 1) return fail(GWF_ERR_INVALID_ARG, "res_per_event must be >= 1");
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  // CUDA graphs: device-resident Fisher calls without a host round trip are captured on their
  // second identical call and replayed afterwards
  if (ctx->graphs && fisher && mem == GWF_MEM_DEVICE && precision != GWF_PREC_MIXED) {
    std::string key = graph_key(n_det, det_ids, wf, params, ld, N, res, res_ev, spacing, per_arm, precision,
                                out_arm, out_net, st, ctx->call_sd_arm, ctx->call_sd_net);
    const std::string bufs = buffer_sig(ctx);
    auto it = ctx->graph_cache.find(key);
    if (it != ctx->graph_cache.end() && it->second.bufs == bufs) {
      GWF_CK(cudaStreamWaitEvent(st, ctx->scratch_free, 0));
      GWF_CK(cudaGraphLaunch(it->second.exec, st));
      GWF_CK(cudaEventRecord(ctx->scratch_free, st));
      return GWF_OK;
    }
    if (it != ctx->graph_cache.end()) {   // buffers were reallocated since the capture
      cudaGraphExecDestroy(it->second.exec);
      ctx->graph_cache.erase(it);
    }
    if (key == ctx->graph_pending) {
      GWF_CK(cudaStreamWaitEvent(st, ctx->scratch_free, 0));
      cudaGraph_t graph = nullptr;
      GWF_CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
      rc = run_body(ctx, fisher, n_det, det_ids, wf, params, ld, N, res, res_ev, spacing, per_arm, precision, mem,
                    out_arm, out_net, st, true);
      const cudaError_t ce = cudaStreamEndCapture(st, &graph);
      if (rc) { if (graph) cudaGraphDestroy(graph); return rc; }
      if (ce != cudaSuccess) return fail(GWF_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
      cudaGraphExec_t exec = nullptr;
      const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
      cudaGraphDestroy(graph);
      if (ie != cudaSuccess) return fail(GWF_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
      if (ctx->graph_cache.size() >= 16) {
        cudaGraphExecDestroy(ctx->graph_cache.begin()->second.exec);
        ctx->graph_cache.erase(ctx->graph_cache.begin());
      }
      ctx->graph_cache[key] = GraphEntry{exec, buffer_sig(ctx)};
      ctx->graph_pending.clear();
      GWF_CK(cudaGraphLaunch(exec, st));
      GWF_CK(cudaEventRecord(ctx->scratch_free, st));
      return GWF_OK;
    }
    ctx->graph_pending = key;
  }
  return run_body(ctx, fisher, n_det, det_ids, wf, params, ld, N, res, res_ev, spacing, per_arm, precision, mem,
                  out_arm, out_net, st, false);
}

// the launches of one call; capturing: inside a stream capture (no host round trips, no
// ordering events: the caller orders the graph launch)
int run_body(gwf_ctx* ctx, bool fisher, int n_det, const int* det_ids, const gwf_wf_desc* wf, const double* params,
             int64_t ld, int64_t N, int32_t res, const int32_t* res_ev, int spacing, int per_arm, int precision,
             int mem, double* out_arm, double* out_net, cudaStream_t st, bool capturing) {
  int rc = GWF_OK;
  const double* dp;
  int64_t dld;
  const int* dres;
  const int npar = npar_of(wf->model);
  rc = stage_inputs(ctx, params, ld, N, res_ev, mem, st, &dp, &dld, &dres, npar);
  if (rc) return rc;
  const int slots = slots_of(ctx, n_det, det_ids);
  const size_t per = fisher ? (size_t)npar * npar : 1;
  double* darm = nullptr;
  double* dnet = nullptr;
  if (mem == GWF_MEM_DEVICE) {
    darm = out_arm;
    dnet = out_net;
  } else {
    if (out_arm) {
      if (ctx->oarm.ensure((size_t)slots * N * per * sizeof(double))) return fail(GWF_ERR_OOM, "device allocation failed (out)");
      darm = (double*)ctx->oarm.p;
    }
    if (out_net) {
      if (ctx->onet.ensure((size_t)N * per * sizeof(double))) return fail(GWF_ERR_OOM, "device allocation failed (out)");
      dnet = (double*)ctx->onet.p;
    }
  }
  // SNR-derivative outputs (Fisher calls through gwf_fisher_ex)
  double* sd_arm = fisher ? ctx->call_sd_arm : nullptr;
  double* sd_net = fisher ? ctx->call_sd_net : nullptr;
  double* dsda = nullptr;
  double* dsdn = nullptr;
  if (mem == GWF_MEM_DEVICE) {
    dsda = sd_arm;
    dsdn = sd_net;
  } else {
    if (sd_arm) {
      if (ctx->osda.ensure((size_t)slots * N * npar * sizeof(double))) return fail(GWF_ERR_OOM, "device allocation failed (out)");
      dsda = (double*)ctx->osda.p;
    }
    if (sd_net) {
      if (ctx->osdn.ensure((size_t)N * npar * sizeof(double))) return fail(GWF_ERR_OOM, "device allocation failed (out)");
      dsdn = (double*)ctx->osdn.p;
    }
  }
  // the mixed form needs the network total to decide which events get FP64
  if (precision == GWF_PREC_MIXED && !dnet) {
    if (ctx->onet.ensure((size_t)N * per * sizeof(double))) return fail(GWF_ERR_OOM, "device allocation failed (out)");
    dnet = (double*)ctx->onet.p;
  }
  const size_t stride = setup_stride_any(wf->model);
  const size_t chunk = (size_t)(N < gwf::kChunk ? N : gwf::kChunk);
  // FP32 network totals: detectors with the same grid (fmin, fmax, Earth rotation) form groups
  // that one launch evaluates together (the waveform once per point for the whole group)
  std::vector<std::vector<int>> groups;
  // (the 11-parameter models: Fisher network totals and SNRs, every precision)
  const bool fp64_groups = precision == GWF_PREC_FP64;
  const bool grouping = ctx->groups && !dsda && !dsdn && ctx->seg_points == 0 && wf->model <= GWF_WF_PHENOMHM &&
                        (!fisher || !darm);
  // per-arm output slot of each detector, in the order of det_ids (groups may launch in another order)
  std::vector<int> slot_of(n_det, 0);
  for (int i = 1; i < n_det; ++i)
    slot_of[i] = slot_of[i - 1] + (ctx->dets[det_ids[i - 1]].desc.shape == GWF_SHAPE_T ? 3 : 1);
  for (int i = 0; i < n_det; ++i) {
    const gwf_det_desc& di = ctx->dets[det_ids[i]].desc;
    bool placed = false;
    for (auto& g : groups) {
      const gwf_det_desc& d0 = ctx->dets[det_ids[g[0]]].desc;
      if (grouping && (int)g.size() < gwf::kMaxGroup && d0.fmin == di.fmin && d0.fmax == di.fmax &&
          d0.earth_rotation == di.earth_rotation) {
        g.push_back(i);
        placed = true;
        break;
      }
    }
    if (!placed) groups.push_back({i});
  }
  size_t gmax = 1;
  for (auto& g : groups) gmax = g.size() > gmax ? g.size() : gmax;
  // the groups run side by side when each has its own scratch and output: network totals and
  // per-arm slots without SNR derivatives, not in a graph capture, no segmented launches
  const int ngr = (int)groups.size();
  const bool side = ngr > 1 && !capturing && !dsda && !dsdn && !(fisher && ctx->seg_points > 0) && dnet;
  if (ctx->setup.ensure((side ? ngr : 1) * gmax * chunk * stride))
    return fail(GWF_ERR_OOM, "device allocation failed (set-up scratch)");
  if (side) {
    if (ctx->gnet.ensure((size_t)(ngr - 1) * N * per * sizeof(double))) return fail(GWF_ERR_OOM, "device allocation failed (out)");
    rc = ensure_aux(ctx, ngr);
    if (!rc && !ctx->core_ev && cudaEventCreateWithFlags(&ctx->core_ev, cudaEventDisableTiming) != cudaSuccess)
      rc = fail(GWF_ERR_CUDA, "event creation failed");
    if (rc) return rc;
  }
  // a network shares the source-dependent part of the per-event set-up between its detectors
  const size_t core_b = core_bytes_any(wf->model);
  const bool share = n_det > 1 && ctx->core.ensure((size_t)N * core_b) == 0;
  // the scratch is shared by every call on this context: order this call after the previous one
  if (!capturing) GWF_CK(cudaStreamWaitEvent(st, ctx->scratch_free, 0));
  gwf::LaunchArgs a;
  a.scratch = (unsigned char*)ctx->setup.p;
  a.cap_events = (long long)chunk;
  if (ctx->ktiming && ctx->ktimer && !capturing) {
    ctx->ktimer->n = 0;
    ctx->ktimer->open = false;
    a.timer = ctx->ktimer;
  }
  if (fisher && ctx->seg_points > 0 && wf->model < GWF_WF_TAYLORF2_TIDAL) {
    int64_t rmax = 0;
    if (capturing && res_ev) rmax = ctx->graph_rmax;   // from the uncaptured run of the same call
    else rc = max_res(res, res_ev, N, mem, &rmax);
    ctx->graph_rmax = rmax;
    if (!rc) rc = seg_setup(ctx, a, ctx->seg_points, (int64_t)chunk, rmax, st);
    if (rc) return rc;
  }
  a.ev.p = dp;
  a.ev.ld = dld;
  a.ev.N = N;
  a.ev.n0 = 0;
  a.ev.res = res;
  a.ev.res_ev = dres;
  a.ev.spacing = spacing;
  a.wf = wf_dev(wf);
  if (wf->model == GWF_WF_PHENOMNSBH) {
    const int xrc = ensure_xitide(ctx, st);
    if (xrc) return xrc;
    a.wf.xitide = (const double*)ctx->xit.p;
  }
  a.qnm = ctx->d_qnm;
  a.nq = ctx->nq;
  a.per_arm = per_arm || dsda;   // per-arm SNR derivatives need the per-arm Gram sets
  a.precision = precision == GWF_PREC_FP64 ? GWF_PREC_FP64 : GWF_PREC_FP32;
  a.stream = st;
  bool first = true;
  if (side) GWF_CK(cudaEventRecord(ctx->fork, st));
  // the mixed form's second stage reuses the FP64 set-up records of this pass when they all stay in
  // the scratch until then: one chunk, and every group in its own scratch area
  std::vector<const unsigned char*> recs(n_det, nullptr);
  std::vector<int> patch(n_det, 0);
  const bool keep_recs = precision == GWF_PREC_MIXED && fisher && N <= gwf::kChunk && (side || ngr == 1);
  int gi = 0;
  for (auto& grp : groups) {
    a.core = share ? (unsigned char*)ctx->core.p : nullptr;
    a.core_mode = share ? (first ? 1 : 2) : 0;
    a.accum = !first;
    a.out_det = dnet;
    if (side) {
      a.accum = 0;
      a.core_done = first && share ? ctx->core_ev : nullptr;
      a.scratch = (unsigned char*)ctx->setup.p + (size_t)gi * gmax * chunk * stride;
      if (!first) {
        a.stream = ctx->aux[gi];
        a.out_det = (double*)ctx->gnet.p + (size_t)(gi - 1) * N * per;
        GWF_CK(cudaStreamWaitEvent(a.stream, ctx->fork, 0));
        if (share) GWF_CK(cudaStreamWaitEvent(a.stream, ctx->core_ev, 0));
      }
    }
    first = false;
    ++gi;
    cudaError_t err;
    if (grp.size() > 1 && fp64_groups) {   // FP64 network total of the group
      gwf::Group64 G;
      G.nd = (int)grp.size();
      for (int d = 0; d < G.nd; ++d) {
        G.det[d] = dev_of(ctx->dets[det_ids[grp[d]]]);
        G.same_psd[d] = d > 0 && ctx->dets[det_ids[grp[d]]].psd_class == ctx->dets[det_ids[grp[d - 1]]].psd_class;
        G.scratch[d] = a.scratch + (size_t)d * chunk * stride;
      }
      a.det = G.det[0];
      a.out_arm = nullptr;
      a.out_sd_arm = nullptr;
      a.out_sd_det = nullptr;
      if (fisher) {
        err = wf->model == 0 ? gwf::launch_group64_m0(a, G)
                             : (wf->model == 1 ? gwf::launch_group64_m1(a, G) : gwf::launch_group64_m2(a, G));
      } else {
        for (int d = 0; d < G.nd; ++d) G.out_arm[d] = darm ? darm + (size_t)slot_of[grp[d]] * N : nullptr;
        err = wf->model == 0 ? gwf::launch_snr_group64_m0(a, G)
                             : (wf->model == 1 ? gwf::launch_snr_group64_m1(a, G) : gwf::launch_snr_group64_m2(a, G));
      }
      if (err != cudaSuccess) return fail(GWF_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(err));
      if (side && gi > 1) GWF_CK(cudaEventRecord(ctx->aux_done[gi - 1], a.stream));
      continue;
    }
    if (grp.size() > 1 && !fisher) {   // FP32 SNR of the group
      gwf::Group64 G;
      G.nd = (int)grp.size();
      for (int d = 0; d < G.nd; ++d) {
        G.det[d] = dev_of(ctx->dets[det_ids[grp[d]]]);
        G.same_psd[d] = d > 0 && ctx->dets[det_ids[grp[d]]].psd_class == ctx->dets[det_ids[grp[d - 1]]].psd_class;
        G.out_arm[d] = darm ? darm + (size_t)slot_of[grp[d]] * N : nullptr;
      }
      a.det = G.det[0];
      a.out_arm = nullptr;
      err = wf->model == 0 ? gwf::launch_snr_group_f32_m0(a, G)
                           : (wf->model == 1 ? gwf::launch_snr_group_f32_m1(a, G) : gwf::launch_snr_group_f32_m2(a, G));
      if (err != cudaSuccess) return fail(GWF_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(err));
      if (side && gi > 1) GWF_CK(cudaEventRecord(ctx->aux_done[gi - 1], a.stream));
      continue;
    }
    if (grp.size() > 1) {   // (grouping implies here: FP32 Fisher, network total only)
      gwf::GroupDev g;
      g.nd = (int)grp.size();
      for (int d = 0; d < g.nd; ++d) {
        g.det[d] = dev_of(ctx->dets[det_ids[grp[d]]]);
        g.wr[d] = (float)std::sqrt(g.det[0].psd_scale / g.det[d].psd_scale);
        g.same_psd[d] = d > 0 && ctx->dets[det_ids[grp[d]]].psd_class == ctx->dets[det_ids[grp[d - 1]]].psd_class;
      }
      g.slice = 0;
      // the group's other detectors get only their projection in the first pass (their FP64 records
      // would equal detector 0's but for the projection header): the FP64 stage copies detector 0's
      // records for them and recomputes that header
      for (int d = 0; keep_recs && d < g.nd; ++d) {
        recs[grp[d]] = a.scratch;
        patch[grp[d]] = d > 0;
      }
      a.det = g.det[0];
      a.out_arm = nullptr;
      a.out_sd_arm = nullptr;
      a.out_sd_det = nullptr;
      err = wf->model == 0 ? gwf::launch_group_m0(a, g) : (wf->model == 1 ? gwf::launch_group_m1(a, g) : gwf::launch_group_m2(a, g));
      if (err != cudaSuccess) return fail(GWF_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(err));
      if (side && gi > 1) GWF_CK(cudaEventRecord(ctx->aux_done[gi - 1], a.stream));
      continue;
    }
    const DetRec& r = ctx->dets[det_ids[grp[0]]];
    if (keep_recs) recs[grp[0]] = a.scratch;
    a.det = dev_of(r);
    a.out_arm = darm ? darm + (size_t)slot_of[grp[0]] * N * per : nullptr;
    a.out_sd_arm = dsda ? dsda + (size_t)slot_of[grp[0]] * N * npar : nullptr;
    a.out_sd_det = dsdn;
    err = fisher ? launch_fisher_any(wf->model, a) : launch_snr_any(wf->model, a);
    if (err != cudaSuccess) return fail(GWF_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(err));
    if (side && gi > 1) GWF_CK(cudaEventRecord(ctx->aux_done[gi - 1], a.stream));
  }
  if (side) {   // join the groups and add their network totals
    for (int g = 1; g < ngr; ++g) GWF_CK(cudaStreamWaitEvent(st, ctx->aux_done[g], 0));
    a.stream = st;
    a.scratch = (unsigned char*)ctx->setup.p;
    a.core_done = nullptr;
    GWF_CK(gwf::launch_add_slices((const double*)ctx->gnet.p, ngr - 1, (long long)N * per, (long long)N * per, dnet, st));
  }
  if (precision == GWF_PREC_MIXED) {
    rc = refine(ctx, n_det, det_ids, a, dp, dld, dres, N, slots, darm, dnet, dsda, dsdn, share, recs, patch, st);
    if (rc) return rc;
  }
  if (!capturing) GWF_CK(cudaEventRecord(ctx->scratch_free, st));
  if (mem == GWF_MEM_HOST) {
    prefault_host(out_arm, out_arm ? (size_t)slots * N * per * sizeof(double) : 0);
    prefault_host(out_net, out_net ? (size_t)N * per * sizeof(double) : 0);
    if (out_arm) GWF_CK(cudaMemcpyAsync(out_arm, darm, (size_t)slots * N * per * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (out_net) GWF_CK(cudaMemcpyAsync(out_net, dnet, (size_t)N * per * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (sd_arm) GWF_CK(cudaMemcpyAsync(sd_arm, dsda, (size_t)slots * N * npar * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (sd_net) GWF_CK(cudaMemcpyAsync(sd_net, dsdn, (size_t)N * npar * sizeof(double), cudaMemcpyDeviceToHost, st));
    int ovf = 0;
    std::vector<int> movf(precision == GWF_PREC_MIXED && ctx->mix_sovf.p ? n_det : 0, 0);
    if (fisher && a.seg > 0 && ctx->seg_ovf.p)
      GWF_CK(cudaMemcpyAsync(&ovf, ctx->seg_ovf.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    if (fisher && !movf.empty())
      GWF_CK(cudaMemcpyAsync(movf.data(), ctx->mix_sovf.p, movf.size() * sizeof(int), cudaMemcpyDeviceToHost, st));
    GWF_CK(cudaStreamSynchronize(st));
    for (int v : movf) ovf |= v;
    if (ovf) return fail(GWF_ERR_CUDA, "segment buffer overflow (internal error)");
  }
  return GWF_OK;
}

// WFOverlap grid: upper frequency max(fcut_1, fcut_2) per event; with a detector fmax, gwfast
// takes fmax where that maximum exceeds it and the first waveform's cut elsewhere
// (gwfast/signal.py:1861-1867, reproduced as written)
// lowest and highest of each event's frequencies (row n of f, or the one row shared by every event
// when f_ld = 0): the models' reference frequency and the upper end that IMRPhenomNSBH reads
__global__ void row_range_kernel(const double* f, long long f_ld, int R, long long N, double* lo, double* hi) {
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const double* r = f + (f_ld > 0 ? n * f_ld : 0);
  double a = r[0], b = r[0];
  for (int k = 1; k < R; ++k) {
    a = fmin(a, r[k]);
    b = fmax(b, r[k]);
  }
  lo[n] = a;
  hi[n] = b;
}

__global__ void fcut_pair_kernel(const double* p1, long long ld1, gwf::WfDesc w1, const double* p2, long long ld2,
                                 gwf::WfDesc w2, double fmax, long long N, double* out) {
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  // IMRPhenomD_NRTidalv2 ends at 1.2 times its merger frequency (its deformabilities in rows 11, 12)
  const double f1 = w1.model == GWF_WF_PHENOMD_NRTIDALV2
                        ? gwf::nrt_fcut(p1[n], p1[ld1 + n], p1[11 * ld1 + n], p1[12 * ld1 + n])
                        : gwf::model_fcut(w1, p1[n], p1[ld1 + n], p1[9 * ld1 + n], p1[10 * ld1 + n]);
  const double f2 = w2.model == GWF_WF_PHENOMD_NRTIDALV2
                        ? gwf::nrt_fcut(p2[n], p2[ld2 + n], p2[11 * ld2 + n], p2[12 * ld2 + n])
                        : gwf::model_fcut(w2, p2[n], p2[ld2 + n], p2[9 * ld2 + n], p2[10 * ld2 + n]);
  double fu = f1 > f2 ? f1 : f2;
  if (fmax > 0.0) fu = fu > fmax ? fmax : f1;
  out[n] = fu;
}

size_t stride_of(int model) { return setup_stride_any(model); }

// the phase constant the strain outputs add for TaylorF2 with phiref_vlso (gwfast/waveforms.py:796-802)
double wave_dphi(const gwf_wf_desc* wf) { return (is_tf2_model(wf->model) && (wf->flags & GWF_TF2_PHIREF_VLSO)) ? -M_PI : 0.0; }

cudaError_t launch_wave(const gwf::LaunchArgs& a, const gwf::WaveOut& o) {
  switch (a.wf.model) {
    case 0: return gwf::launch_wave_m0(a, o);
    case 1: return gwf::launch_wave_m1(a, o);
    case 2: return gwf::launch_wave_m2(a, o);
    case 3: return gwf::launch_wave_m3(a, o);
    case 4: return gwf::launch_wave_m4(a, o);
    case 5: return gwf::launch_wave_m5(a, o);
    case 6: return gwf::launch_wave_m6(a, o);
    default: return gwf::launch_wave_m7(a, o);
  }
}

// events per output launch so that a staging buffer of per_event bytes each stays near 1 GiB
int64_t wave_chunk(size_t per_event) {
  int64_t c = (int64_t)(((size_t)1 << 30) / (per_event ? per_event : 1));
  if (c < 1) c = 1;
  return c < gwf::kChunk ? c : gwf::kChunk;
}

}  // namespace

int gwf::ctx_device(const gwf_ctx* ctx) { return ctx->device; }

extern "C" {

int gwf_version(void) { return 1; }

const char* gwf_last_error(void) { return g_err.c_str(); }

int gwf_ctx_create(int device, gwf_ctx** out) {
  if (!out) return fail(GWF_ERR_INVALID_ARG, "null output pointer");
  int ndev = 0;
  GWF_CK(cudaGetDeviceCount(&ndev));
  if (device < 0 || device >= ndev) return fail(GWF_ERR_INVALID_ARG, "no such CUDA device");
  GWF_CK(cudaSetDevice(device));
  gwf_ctx* c = new gwf_ctx();
  c->device = device;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->scratch_free, cudaEventDisableTiming) != cudaSuccess) {
    delete c;
    return fail(GWF_ERR_CUDA, "stream creation failed");
  }
  *out = c;
  return GWF_OK;
}

int gwf_ctx_destroy(gwf_ctx* ctx) {
  if (!ctx) return GWF_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (auto& r : ctx->dets) {
    cudaFree(r.d_f);
    cudaFree(r.d_S);
    cudaFree(r.d_acc);
    cudaFree(r.d_seg);
  }
  cudaFree(ctx->d_qnm);
  ctx->par.release(); ctx->res.release(); ctx->oarm.release(); ctx->onet.release();
  ctx->fin.release(); ctx->fout.release(); ctx->feps.release(); ctx->fcond.release(); ctx->setup.release();
  ctx->mix_idx.release(); ctx->mix_cnt.release(); ctx->mix_par.release(); ctx->mix_res.release();
  ctx->mix_net.release(); ctx->mix_arm.release();
  ctx->seg_off.release(); ctx->seg_ctr.release(); ctx->seg_part.release(); ctx->seg_ovf.release();
  ctx->tune_out.release();
  ctx->osda.release(); ctx->osdn.release(); ctx->mix_sda.release(); ctx->mix_sdn.release();
  ctx->wbuf.release(); ctx->par2.release(); ctx->fcutb.release(); ctx->ovb.release();
  ctx->sfreq.release(); ctx->samp.release(); ctx->sph.release(); ctx->srange.release();
  ctx->core.release();
  ctx->xit.release();
  ctx->mix_scr.release(); ctx->mix_soff.release(); ctx->mix_sctr.release(); ctx->mix_spart.release();
  ctx->mix_sovf.release();
  for (auto s : ctx->aux) cudaStreamDestroy(s);
  for (auto e : ctx->aux_done) cudaEventDestroy(e);
  if (ctx->fork) cudaEventDestroy(ctx->fork);
  if (ctx->core_ev) cudaEventDestroy(ctx->core_ev);
  ctx->gnet.release();
  for (auto& g : ctx->graph_cache) cudaGraphExecDestroy(g.second.exec);
  ctx->graph_cache.clear();
  ctx->hpar.release(); ctx->hout.release();
  if (ctx->ktimer) {
    for (auto e : ctx->ktimer->ev) cudaEventDestroy(e);
    delete ctx->ktimer;
  }
  cudaEventDestroy(ctx->scratch_free);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return GWF_OK;
}

int gwf_xitide(gwf_ctx* ctx, const double* comp, const double* q, const double* chi_bh, int64_t n, double* out) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (n < 0 || (n > 0 && (!comp || !q || !chi_bh || !out))) return fail(GWF_ERR_INVALID_ARG, "bad arguments");
  cudaStream_t st = ctx->stream;
  rc = ensure_xitide(ctx, st);
  if (rc || n == 0) return rc;
  if (ctx->fin.ensure((size_t)n * 4 * sizeof(double))) return fail(GWF_ERR_OOM, "device allocation failed");
  double* d = (double*)ctx->fin.p;
  GWF_CK(cudaMemcpyAsync(d, comp, n * sizeof(double), cudaMemcpyHostToDevice, st));
  GWF_CK(cudaMemcpyAsync(d + n, q, n * sizeof(double), cudaMemcpyHostToDevice, st));
  GWF_CK(cudaMemcpyAsync(d + 2 * n, chi_bh, n * sizeof(double), cudaMemcpyHostToDevice, st));
  GWF_CK(gwf::launch_xitide_eval((const double*)ctx->xit.p, d, d + n, d + 2 * n, n, d + 3 * n, st));
  GWF_CK(cudaMemcpyAsync(out, d + 3 * n, n * sizeof(double), cudaMemcpyDeviceToHost, st));
  GWF_CK(cudaStreamSynchronize(st));
  return GWF_OK;
}

int gwf_set_qnm_table(gwf_ctx* ctx, const double* spin, const double* fring, const double* fdamp, int64_t n) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (!spin || !fring || !fdamp || n < 2 || n > (1 << 24)) return fail(GWF_ERR_INVALID_ARG, "bad QNM table");
  for (int64_t i = 1; i < n; ++i)
    if (!(spin[i] > spin[i - 1])) return fail(GWF_ERR_INVALID_ARG, "QNM spin grid must be strictly increasing");
  std::vector<double> h(3 * n);
  std::memcpy(h.data(), spin, n * sizeof(double));
  std::memcpy(h.data() + n, fring, n * sizeof(double));
  std::memcpy(h.data() + 2 * n, fdamp, n * sizeof(double));
  cudaFree(ctx->d_qnm);
  ctx->d_qnm = nullptr;
  GWF_CK(cudaMalloc(&ctx->d_qnm, 3 * n * sizeof(double)));
  GWF_CK(cudaMemcpy(ctx->d_qnm, h.data(), 3 * n * sizeof(double), cudaMemcpyHostToDevice));
  ctx->nq = (int)n;
  return GWF_OK;
}

int gwf_detector_add(gwf_ctx* ctx, const gwf_det_desc* desc, const double* psd_f, const double* psd_S, int64_t n,
                     int* det_id) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (!desc || !psd_f || !psd_S || !det_id) return fail(GWF_ERR_INVALID_ARG, "null argument");
  if (desc->shape != GWF_SHAPE_L && desc->shape != GWF_SHAPE_T) return fail(GWF_ERR_INVALID_ARG, "Enter valid detector configuration");
  if (n < 2 || n > (1 << 28)) return fail(GWF_ERR_INVALID_ARG, "PSD table needs at least two rows");
  if (!(desc->fmin > 0.0)) return fail(GWF_ERR_INVALID_ARG, "fmin must be positive");
  for (int64_t i = 0; i < n; ++i) {
    if (!(psd_f[i] > 0.0)) return fail(GWF_ERR_INVALID_ARG, "PSD frequencies must be positive");
    if (i && !(psd_f[i] > psd_f[i - 1])) return fail(GWF_ERR_INVALID_ARG, "PSD frequencies must be strictly increasing");
  }
  DetRec r;
  r.desc = *desc;
  r.n = (int)n;
  r.nacc = 4096;
  r.l0 = std::log(psd_f[0]);
  const double l1 = std::log(psd_f[n - 1]);
  r.idl = r.nacc / (l1 - r.l0);
  std::vector<int> acc(r.nacc);
  int64_t j = 0;
  for (int b = 0; b < r.nacc; ++b) {
    const double fb = std::exp(r.l0 + b / r.idl);
    while (j + 1 < n - 1 && psd_f[j + 1] <= fb) ++j;
    acc[b] = (int)j;
  }
  GWF_CK(cudaMalloc(&r.d_f, n * sizeof(double)));
  GWF_CK(cudaMalloc(&r.d_S, n * sizeof(double)));
  GWF_CK(cudaMalloc(&r.d_acc, r.nacc * sizeof(int)));
  GWF_CK(cudaMemcpy(r.d_f, psd_f, n * sizeof(double), cudaMemcpyHostToDevice));
  GWF_CK(cudaMemcpy(r.d_S, psd_S, n * sizeof(double), cudaMemcpyHostToDevice));
  GWF_CK(cudaMemcpy(r.d_acc, acc.data(), r.nacc * sizeof(int), cudaMemcpyHostToDevice));
  // FP32 segments: frequencies, and the PSD divided by its smallest positive value
  double smin = INFINITY;
  for (int64_t i = 0; i < n; ++i)
    if (psd_S[i] > 0.0 && psd_S[i] < smin) smin = psd_S[i];
  r.scale = std::isfinite(smin) ? smin : 1.0;
  std::vector<float> f32(n), s32(n);
  for (int64_t i = 0; i < n; ++i) {
    f32[i] = (float)psd_f[i];
    s32[i] = (float)(psd_S[i] / r.scale);
  }
  std::vector<float4> seg(n - 1);
  for (int64_t i = 0; i + 1 < n; ++i) {
    const double y0 = psd_S[i] / r.scale, y1 = psd_S[i + 1] / r.scale;
    seg[i] = make_float4(f32[i], f32[i + 1], s32[i], (float)((y1 - y0) / (psd_f[i + 1] - psd_f[i])));
  }
  GWF_CK(cudaMalloc(&r.d_seg, (n - 1) * sizeof(float4)));
  GWF_CK(cudaMemcpy(r.d_seg, seg.data(), (n - 1) * sizeof(float4), cudaMemcpyHostToDevice));
  r.h_f.assign(psd_f, psd_f + n);
  r.h_S.assign(psd_S, psd_S + n);
  r.psd_class = (int)ctx->dets.size();
  for (const DetRec& o : ctx->dets)
    if (o.h_f == r.h_f && o.h_S == r.h_S) { r.psd_class = o.psd_class; break; }
  ctx->dets.push_back(r);
  *det_id = (int)ctx->dets.size() - 1;
  return GWF_OK;
}

int gwf_snr(gwf_ctx* ctx, int n_det, const int* det_ids, const gwf_wf_desc* wf, const double* params, int64_t ld,
            int64_t n_events, int32_t res, const int32_t* res_per_event, int spacing, int precision, int mem,
            double* out_arm, double* out_net, void* stream) {
  return run(ctx, false, n_det, det_ids, wf, params, ld, n_events, res, res_per_event, spacing, 0, precision, mem,
             out_arm, out_net, stream);
}

int gwf_fisher(gwf_ctx* ctx, int n_det, const int* det_ids, const gwf_wf_desc* wf, const double* params, int64_t ld,
               int64_t n_events, int32_t res, const int32_t* res_per_event, int spacing, int per_arm, int precision,
               int mem, double* out_arm, double* out_net, void* stream) {
  return run(ctx, true, n_det, det_ids, wf, params, ld, n_events, res, res_per_event, spacing, per_arm, precision, mem,
             out_arm, out_net, stream);
}

int gwf_set_refine_cond(gwf_ctx* ctx, double kappa) {
  if (!ctx) return fail(GWF_ERR_INVALID_ARG, "null context");
  if (!(kappa > 0.0)) return fail(GWF_ERR_INVALID_ARG, "refinement threshold must be positive");
  ctx->refine_cond = kappa;
  return GWF_OK;
}

int gwf_set_graphs(gwf_ctx* ctx, int on) {
  if (!ctx) return fail(GWF_ERR_INVALID_ARG, "null context");
  GWF_CK(cudaSetDevice(ctx->device));
  ctx->graphs = on ? 1 : 0;
  if (!on) {
    for (auto& g : ctx->graph_cache) cudaGraphExecDestroy(g.second.exec);
    ctx->graph_cache.clear();
    ctx->graph_pending.clear();
  }
  return GWF_OK;
}

int gwf_set_kernel_timing(gwf_ctx* ctx, int on) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (on && !ctx->ktimer) {
    auto* t = new gwf::KernelTimer();
    for (int i = 0; i < 2 * gwf::KernelTimer::kMax; ++i) {
      if (cudaEventCreate(&t->ev[i]) != cudaSuccess) {
        for (int j = 0; j < i; ++j) cudaEventDestroy(t->ev[j]);
        delete t;
        return fail(GWF_ERR_CUDA, "event creation failed");
      }
    }
    ctx->ktimer = t;
  }
  ctx->ktiming = on != 0;
  return GWF_OK;
}

int gwf_kernel_times(gwf_ctx* ctx, int max_entries, int* kind, double* ms, int* n_entries) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (!n_entries || max_entries < 0 || (max_entries > 0 && (!kind || !ms)))
    return fail(GWF_ERR_INVALID_ARG, "bad output arrays");
  gwf::KernelTimer* t = ctx->ktimer;
  const int n = t ? t->n : 0;
  *n_entries = n;
  for (int i = 0; i < n && i < max_entries; ++i) {
    GWF_CK(cudaEventSynchronize(t->ev[2 * i + 1]));
    float v = 0.0f;
    GWF_CK(cudaEventElapsedTime(&v, t->ev[2 * i], t->ev[2 * i + 1]));
    kind[i] = t->kind[i];
    ms[i] = v;
  }
  return GWF_OK;
}

int gwf_set_detector_groups(gwf_ctx* ctx, int on) {
  if (!ctx) return fail(GWF_ERR_INVALID_ARG, "null context");
  ctx->groups = on ? 1 : 0;
  return GWF_OK;
}

int gwf_set_segments(gwf_ctx* ctx, int points) {
  if (!ctx) return fail(GWF_ERR_INVALID_ARG, "null context");
  if (points < 0 || points % gwf::kThreads) return fail(GWF_ERR_INVALID_ARG, "segment length must be 0 or a multiple of 128");
  ctx->seg_points = points;
  return GWF_OK;
}

int gwf_autotune_segments(gwf_ctx* ctx, int n_det, const int* det_ids, const gwf_wf_desc* wf, const double* params,
                          int64_t ld, int64_t n_events, int32_t res, const int32_t* res_per_event, int spacing,
                          int precision, int mem, int* best) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  rc = validate_common(ctx, n_det, det_ids, wf, params, ld, n_events, res, res_per_event, spacing, mem);
  if (rc) return rc;
  if (n_events < 1) return fail(GWF_ERR_INVALID_ARG, "autotuning needs events");
  cudaStream_t st = ctx->stream;
  const double* dp;
  int64_t dld;
  const int* dres;
  const int npar = npar_of(wf->model);
  rc = stage_inputs(ctx, params, ld, n_events, res_per_event, mem, st, &dp, &dld, &dres, npar);
  if (rc) return rc;
  // keep staged inputs: later runs reuse ctx->par / ctx->res, so copy them aside
  DevBuf tp, tr;
  if (mem == GWF_MEM_HOST) {
    if (tp.ensure((size_t)npar * n_events * sizeof(double)) || (dres && tr.ensure((size_t)n_events * sizeof(int))))
      return fail(GWF_ERR_OOM, "device allocation failed (autotune)");
    GWF_CK(cudaMemcpyAsync(tp.p, dp, (size_t)npar * n_events * sizeof(double), cudaMemcpyDeviceToDevice, st));
    if (dres) GWF_CK(cudaMemcpyAsync(tr.p, dres, (size_t)n_events * sizeof(int), cudaMemcpyDeviceToDevice, st));
    dp = (const double*)tp.p;
    dres = dres ? (const int*)tr.p : nullptr;
    dld = n_events;
  }
  if (ctx->tune_out.ensure((size_t)n_events * npar * npar * sizeof(double)))
    return fail(GWF_ERR_OOM, "device allocation failed (autotune)");
  const int cands[] = {0, 256, 512, 1024, 2048};
  const int saved = ctx->seg_points;
  cudaEvent_t e0, e1;
  GWF_CK(cudaEventCreate(&e0));
  GWF_CK(cudaEventCreate(&e1));
  float best_ms = 1e30f;
  int best_seg = saved;
  for (int c : cands) {
    ctx->seg_points = c;
    float tot = 0.0f;
    for (int rep = 0; rep < 3 && rc == GWF_OK; ++rep) {   // first run warms up
      cudaEventRecord(e0, st);
      rc = run(ctx, true, n_det, det_ids, wf, dp, dld, n_events, res, dres, spacing, 0, precision, GWF_MEM_DEVICE,
               nullptr, (double*)ctx->tune_out.p, st);
      cudaEventRecord(e1, st);
      cudaEventSynchronize(e1);
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep) tot += ms;
    }
    if (rc) break;
    if (tot < best_ms) { best_ms = tot; best_seg = c; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  tp.release();
  tr.release();
  ctx->seg_points = rc ? saved : best_seg;
  if (best) *best = ctx->seg_points;
  return rc;
}

int gwf_fisher_ex(gwf_ctx* ctx, int n_det, const int* det_ids, const gwf_wf_desc* wf, const double* params, int64_t ld,
                  int64_t n_events, int32_t res, const int32_t* res_per_event, int spacing, int per_arm, int precision,
                  int mem, double* out_arm, double* out_net, double* out_snr_der_arm, double* out_snr_der_net,
                  void* stream) {
  if (!ctx) return fail(GWF_ERR_INVALID_ARG, "null context");
  ctx->call_sd_arm = out_snr_der_arm;
  ctx->call_sd_net = out_snr_der_net;
  if (!out_arm && !out_net && (out_snr_der_arm || out_snr_der_net)) {   // derivatives only: a throw-away total
    const int npar = wf ? npar_of(wf->model) : gwf::NP;
    if (ctx->tune_out.ensure((size_t)(n_events > 0 ? n_events : 1) * npar * npar * sizeof(double))) {
      ctx->call_sd_arm = ctx->call_sd_net = nullptr;
      return fail(GWF_ERR_OOM, "device allocation failed");
    }
  }
  const bool tmp_net = !out_arm && !out_net && (out_snr_der_arm || out_snr_der_net);
  double* host_tmp = nullptr;
  std::vector<double> htmp;
  if (tmp_net && mem == GWF_MEM_HOST) {
    htmp.resize((size_t)(n_events > 0 ? n_events : 1) * (wf ? npar_of(wf->model) : gwf::NP) * (wf ? npar_of(wf->model) : gwf::NP));
    host_tmp = htmp.data();
  }
  const int rc = run(ctx, true, n_det, det_ids, wf, params, ld, n_events, res, res_per_event, spacing, per_arm,
                     precision, mem, out_arm, tmp_net ? (mem == GWF_MEM_HOST ? host_tmp : (double*)ctx->tune_out.p)
                                                      : out_net, stream);
  ctx->call_sd_arm = ctx->call_sd_net = nullptr;
  return rc;
}

int gwf_strain(gwf_ctx* ctx, int det_id, const gwf_wf_desc* wf, const double* params, int64_t ld, int64_t n_events,
               const double* freqs, int64_t f_ld, int32_t n_freq, int mem, double* out_strain, double* out_amp,
               double* out_phase, void* stream) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  rc = validate_common(ctx, 1, &det_id, wf, params, ld, n_events, 2, nullptr, 0, mem);
  if (rc) return rc;
  if (!out_strain && !out_amp && !out_phase) return fail(GWF_ERR_INVALID_ARG, "no output requested");
  if (!freqs || n_freq < 1) return fail(GWF_ERR_INVALID_ARG, "need at least one frequency");
  if (f_ld != 0 && f_ld < n_freq) return fail(GWF_ERR_INVALID_ARG, "f_ld must be 0 or >= n_freq");
  if (out_phase && wf->model == GWF_WF_PHENOMHM)
    return fail(GWF_ERR_UNSUPPORTED, "GWPhase of IMRPhenomHM: its phase is one per mode");
  const int64_t N = n_events;
  if (N == 0) return GWF_OK;
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  const int npar = npar_of(wf->model);
  const double* dp;
  int64_t dld;
  const int* dres;
  rc = stage_inputs(ctx, params, ld, N, nullptr, mem, st, &dp, &dld, &dres, npar);
  if (rc) return rc;
  if (wf->model == GWF_WF_PHENOMNSBH && (rc = ensure_xitide(ctx, st))) return rc;
  const size_t nf = f_ld ? (size_t)N * (size_t)f_ld : (size_t)n_freq;
  const double* dfreq = freqs;
  if (mem == GWF_MEM_HOST) {
    for (size_t i = 0; i < nf; ++i)
      if (!(freqs[i] > 0.0) && (f_ld == 0 || (int64_t)(i % (size_t)f_ld) < n_freq))
        return fail(GWF_ERR_INVALID_ARG, "frequencies must be positive");
    if (ctx->sfreq.ensure(nf * sizeof(double))) return fail(GWF_ERR_OOM, "device allocation failed (frequencies)");
    GWF_CK(cudaMemcpyAsync(ctx->sfreq.p, freqs, nf * sizeof(double), cudaMemcpyHostToDevice, st));
    dfreq = (const double*)ctx->sfreq.p;
  }
  // per event: the lowest frequency sets the models' reference (as gwfast takes fRef = min of the
  // grid it is given), the highest stands for the grid end
  if (ctx->srange.ensure((size_t)2 * N * sizeof(double))) return fail(GWF_ERR_OOM, "device allocation failed (ranges)");
  double* flo = (double*)ctx->srange.p;
  row_range_kernel<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(dfreq, f_ld, n_freq, N, flo, flo + N);
  GWF_CK(cudaGetLastError());
  const DetRec& r = ctx->dets[det_id];
  const int NA = r.desc.shape == GWF_SHAPE_T ? 3 : 1;
  const size_t row_c = (size_t)n_freq * 2 * sizeof(double);   // one event's row of complex values
  const size_t row_d = (size_t)n_freq * sizeof(double);
  const size_t per_ev = (out_strain ? NA * row_c : 0) + (out_amp ? NA * row_c : 0) + (out_phase ? 2 * row_d : 0);
  const int64_t chunk = mem == GWF_MEM_DEVICE ? (N < gwf::kChunk ? N : gwf::kChunk) : wave_chunk(per_ev);
  const int64_t cap = chunk < N ? chunk : N;
  if (ctx->setup.ensure((size_t)cap * stride_of(wf->model))) return fail(GWF_ERR_OOM, "device allocation failed (set-up scratch)");
  if (mem == GWF_MEM_HOST && ((out_strain && ctx->wbuf.ensure((size_t)cap * NA * row_c)) ||
                              (out_amp && ctx->samp.ensure((size_t)cap * NA * row_c)) ||
                              (out_phase && ctx->sph.ensure((size_t)cap * 2 * row_d))))
    return fail(GWF_ERR_OOM, "device allocation failed (strain)");
  GWF_CK(cudaStreamWaitEvent(st, ctx->scratch_free, 0));
  gwf::LaunchArgs a;
  a.ev.p = dp;
  a.ev.ld = dld;
  a.ev.N = N;
  a.ev.n0 = 0;
  a.ev.res = 2;   // (the set-up needs a grid; the points are the caller's)
  a.ev.res_ev = nullptr;
  a.ev.spacing = 0;
  a.ev.fmin_ev = flo;
  a.ev.fcut_ev = flo + N;
  a.det = dev_of(r);
  a.wf = wf_dev(wf);
  if (wf->model == GWF_WF_PHENOMNSBH) a.wf.xitide = (const double*)ctx->xit.p;
  a.qnm = ctx->d_qnm;
  a.nq = ctx->nq;
  a.out_arm = a.out_det = nullptr;
  a.accum = 0;
  a.per_arm = 0;
  a.precision = GWF_PREC_FP64;
  a.scratch = (unsigned char*)ctx->setup.p;
  a.cap_events = cap;
  a.stream = st;
  if (mem == GWF_MEM_HOST) {
    if (out_strain) prefault_host(out_strain, (size_t)NA * N * row_c);
    if (out_amp) prefault_host(out_amp, (size_t)NA * N * row_c);
    if (out_phase) prefault_host(out_phase, (size_t)2 * N * row_d);
  }
  for (int64_t n0 = 0; n0 < N; n0 += chunk) {
    const int64_t cnt = (N - n0) < chunk ? (N - n0) : chunk;
    gwf::WaveOut o{};
    o.mode = gwf::WAVE_STRAIN;
    o.dphi = wave_dphi(wf);
    o.n0 = n0;
    o.cnt = cnt;
    o.R_out = n_freq;
    o.f_ld = f_ld;
    const bool dev = mem == GWF_MEM_DEVICE;
    o.out_n = dev ? N : cnt;
    o.out_base = dev ? 0 : n0;
    o.f_in = dev || f_ld == 0 ? dfreq : dfreq + (size_t)n0 * f_ld;
    o.out = out_strain ? reinterpret_cast<gwf::cd*>(dev ? (void*)out_strain : ctx->wbuf.p) : nullptr;
    o.amp = out_amp ? reinterpret_cast<gwf::cd*>(dev ? (void*)out_amp : ctx->samp.p) : nullptr;
    o.phase = out_phase ? (dev ? out_phase : (double*)ctx->sph.p) : nullptr;
    cudaError_t e = launch_wave(a, o);
    if (e != cudaSuccess) return fail(GWF_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    if (!dev) {   // rows [n0, n0 + cnt) of each (arm) block
      if (out_strain)
        GWF_CK(cudaMemcpy2DAsync(out_strain + (size_t)n0 * n_freq * 2, (size_t)N * row_c, ctx->wbuf.p, (size_t)cnt * row_c,
                                 (size_t)cnt * row_c, (size_t)NA, cudaMemcpyDeviceToHost, st));
      if (out_amp)
        GWF_CK(cudaMemcpy2DAsync(out_amp + (size_t)n0 * n_freq * 2, (size_t)N * row_c, ctx->samp.p, (size_t)cnt * row_c,
                                 (size_t)cnt * row_c, (size_t)NA, cudaMemcpyDeviceToHost, st));
      if (out_phase)
        GWF_CK(cudaMemcpy2DAsync(out_phase + (size_t)n0 * n_freq, (size_t)N * row_d, ctx->sph.p, (size_t)cnt * row_d,
                                 (size_t)cnt * row_d, 2, cudaMemcpyDeviceToHost, st));
    }
  }
  GWF_CK(cudaEventRecord(ctx->scratch_free, st));
  if (mem == GWF_MEM_HOST) GWF_CK(cudaStreamSynchronize(st));
  return GWF_OK;
}

int gwf_strain_derivs(gwf_ctx* ctx, int det_id, const gwf_wf_desc* wf, const double* params, int64_t ld,
                      int64_t n_events, int32_t res, int spacing, int mem, double* out, void* stream) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  rc = validate_common(ctx, 1, &det_id, wf, params, ld, n_events, res, nullptr, spacing, mem);
  if (rc) return rc;
  if (!out) return fail(GWF_ERR_INVALID_ARG, "no output requested");
  const int64_t N = n_events;
  if (N == 0) return GWF_OK;
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  const int npar = npar_of(wf->model);
  const double* dp;
  int64_t dld;
  const int* dres;
  rc = stage_inputs(ctx, params, ld, N, nullptr, mem, st, &dp, &dld, &dres, npar);
  if (rc) return rc;
  if (wf->model == GWF_WF_PHENOMNSBH && (rc = ensure_xitide(ctx, st))) return rc;
  const DetRec& r = ctx->dets[det_id];
  const int NA = r.desc.shape == GWF_SHAPE_T ? 3 : 1;
  const size_t per_ev = (size_t)NA * npar * (size_t)res * 2 * sizeof(double);
  const int64_t chunk = mem == GWF_MEM_DEVICE ? (N < gwf::kChunk ? N : gwf::kChunk) : wave_chunk(per_ev);
  const int64_t cap = chunk < N ? chunk : N;
  if (ctx->setup.ensure((size_t)cap * stride_of(wf->model))) return fail(GWF_ERR_OOM, "device allocation failed (set-up scratch)");
  if (mem == GWF_MEM_HOST && ctx->wbuf.ensure((size_t)cap * per_ev)) return fail(GWF_ERR_OOM, "device allocation failed (derivatives)");
  GWF_CK(cudaStreamWaitEvent(st, ctx->scratch_free, 0));
  gwf::LaunchArgs a;
  a.ev.p = dp;
  a.ev.ld = dld;
  a.ev.N = N;
  a.ev.n0 = 0;
  a.ev.res = res;
  a.ev.res_ev = nullptr;
  a.ev.spacing = spacing;
  a.det = dev_of(r);
  a.wf = wf_dev(wf);
  if (wf->model == GWF_WF_PHENOMNSBH) a.wf.xitide = (const double*)ctx->xit.p;
  a.qnm = ctx->d_qnm;
  a.nq = ctx->nq;
  a.out_arm = a.out_det = nullptr;
  a.accum = 0;
  a.per_arm = 0;
  a.precision = GWF_PREC_FP64;
  a.scratch = (unsigned char*)ctx->setup.p;
  a.cap_events = cap;
  a.stream = st;
  for (int64_t n0 = 0; n0 < N; n0 += chunk) {
    const int64_t cnt = (N - n0) < chunk ? (N - n0) : chunk;
    gwf::WaveOut o{};
    o.mode = gwf::WAVE_DERIVS;
    o.dphi = wave_dphi(wf);
    o.n0 = n0;
    o.cnt = cnt;
    o.R_out = res;
    if (mem == GWF_MEM_DEVICE) {
      o.out = reinterpret_cast<gwf::cd*>(out);
      o.out_n = N;
      o.out_base = 0;
    } else {
      o.out = reinterpret_cast<gwf::cd*>(ctx->wbuf.p);
      o.out_n = cnt;
      o.out_base = n0;
    }
    cudaError_t e = launch_wave(a, o);
    if (e != cudaSuccess) return fail(GWF_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    if (mem == GWF_MEM_HOST) {   // rows [n0, n0 + cnt) of each (arm, parameter) block
      const size_t row = (size_t)res * 2 * sizeof(double);
      if (n0 == 0) prefault_host(out, (size_t)NA * npar * N * row);
      GWF_CK(cudaMemcpy2DAsync(out + (size_t)n0 * res * 2, (size_t)N * row, ctx->wbuf.p, (size_t)cnt * row,
                               (size_t)cnt * row, (size_t)NA * npar, cudaMemcpyDeviceToHost, st));
    }
  }
  GWF_CK(cudaEventRecord(ctx->scratch_free, st));
  if (mem == GWF_MEM_HOST) GWF_CK(cudaStreamSynchronize(st));
  return GWF_OK;
}

int gwf_overlap(gwf_ctx* ctx, int n_det, const int* det_ids, const gwf_wf_desc* wf1, const double* params1,
                int64_t ld1, const gwf_wf_desc* wf2, const double* params2, int64_t ld2, int64_t n_events, int32_t res,
                int mem, double* out_ov, double* out_n1, double* out_n2, void* stream) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  rc = validate_common(ctx, n_det, det_ids, wf1, params1, ld1, n_events, res, nullptr, GWF_SPACING_GEOM, mem);
  if (!rc) rc = validate_common(ctx, n_det, det_ids, wf2, params2, ld2, n_events, res, nullptr, GWF_SPACING_GEOM, mem);
  if (rc) return rc;
  if (!out_ov || !out_n1 || !out_n2) return fail(GWF_ERR_INVALID_ARG, "overlap needs all three outputs");
  const int64_t N = n_events;
  if (N == 0) return GWF_OK;
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  const double *dp1, *dp2;
  int64_t dld1, dld2;
  const int* dres;
  rc = stage_inputs(ctx, params1, ld1, N, nullptr, mem, st, &dp1, &dld1, &dres, npar_of(wf1->model));
  if (!rc) rc = stage_inputs_to(ctx, ctx->par2, params2, ld2, N, nullptr, mem, st, &dp2, &dld2, &dres, npar_of(wf2->model));
  if (rc) return rc;
  if ((wf1->model == GWF_WF_PHENOMNSBH || wf2->model == GWF_WF_PHENOMNSBH) && (rc = ensure_xitide(ctx, st))) return rc;
  const size_t per_ev = (size_t)2 * res * 2 * sizeof(double);   // at most two computed arms
  const int64_t chunk = wave_chunk(per_ev);
  const int64_t cap = chunk < N ? chunk : N;
  const size_t stride = std::max(stride_of(wf1->model), stride_of(wf2->model));
  if (ctx->setup.ensure((size_t)cap * stride) || ctx->wbuf.ensure((size_t)cap * per_ev) ||
      ctx->fcutb.ensure((size_t)N * sizeof(double)) ||
      (mem == GWF_MEM_HOST && ctx->ovb.ensure((size_t)3 * n_det * N * sizeof(double))))
    return fail(GWF_ERR_OOM, "device allocation failed (overlap)");
  double* dov = mem == GWF_MEM_DEVICE ? out_ov : (double*)ctx->ovb.p;
  double* dn1 = mem == GWF_MEM_DEVICE ? out_n1 : dov + (size_t)n_det * N;
  double* dn2 = mem == GWF_MEM_DEVICE ? out_n2 : dov + (size_t)2 * n_det * N;
  GWF_CK(cudaStreamWaitEvent(st, ctx->scratch_free, 0));
  gwf::LaunchArgs a;
  a.ev.N = N;
  a.ev.n0 = 0;
  a.ev.res = res;
  a.ev.res_ev = nullptr;
  a.ev.spacing = GWF_SPACING_GEOM;
  a.ev.fcut_ev = (const double*)ctx->fcutb.p;
  a.qnm = ctx->d_qnm;
  a.nq = ctx->nq;
  a.out_arm = a.out_det = nullptr;
  a.accum = 0;
  a.per_arm = 0;
  a.precision = GWF_PREC_FP64;
  a.scratch = (unsigned char*)ctx->setup.p;
  a.cap_events = cap;
  a.stream = st;
  for (int i = 0; i < n_det; ++i) {
    const DetRec& r = ctx->dets[det_ids[i]];
    a.det = dev_of(r);
    fcut_pair_kernel<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(dp1, dld1, wf_dev(wf1), dp2, dld2, wf_dev(wf2),
                                                                 r.desc.fmax, N, (double*)ctx->fcutb.p);
    GWF_CK(cudaGetLastError());
    for (int64_t n0 = 0; n0 < N; n0 += chunk) {
      const int64_t cnt = (N - n0) < chunk ? (N - n0) : chunk;
      gwf::WaveOut o{};
      o.n0 = n0;
      o.cnt = cnt;
      o.out = reinterpret_cast<gwf::cd*>(ctx->wbuf.p);
      o.out_n = cnt;
      o.out_base = n0;
      o.R_out = res;
      o.ov = dov + (size_t)i * N;
      o.n1 = dn1 + (size_t)i * N;
      o.n2 = dn2 + (size_t)i * N;
      o.mode = gwf::WAVE_STORE;
      o.dphi = wave_dphi(wf1);
      a.ev.p = dp1;
      a.ev.ld = dld1;
      a.wf = wf_dev(wf1);
      a.wf.xitide = (const double*)ctx->xit.p;
      cudaError_t e = launch_wave(a, o);
      o.mode = gwf::WAVE_OVERLAP;
      o.dphi = wave_dphi(wf2);
      a.ev.p = dp2;
      a.ev.ld = dld2;
      a.wf = wf_dev(wf2);
      a.wf.xitide = (const double*)ctx->xit.p;
      if (e == cudaSuccess) e = launch_wave(a, o);
      if (e != cudaSuccess) return fail(GWF_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    }
  }
  GWF_CK(cudaEventRecord(ctx->scratch_free, st));
  if (mem == GWF_MEM_HOST) {
    const size_t b = (size_t)n_det * N * sizeof(double);
    GWF_CK(cudaMemcpyAsync(out_ov, dov, b, cudaMemcpyDeviceToHost, st));
    GWF_CK(cudaMemcpyAsync(out_n1, dn1, b, cudaMemcpyDeviceToHost, st));
    GWF_CK(cudaMemcpyAsync(out_n2, dn2, b, cudaMemcpyDeviceToHost, st));
    GWF_CK(cudaStreamSynchronize(st));
  }
  return GWF_OK;
}

int gwf_cov_n(gwf_ctx* ctx, const double* F, int64_t N, int n_params, int mem, double* cov, double* eps, double* cond,
              void* stream) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (n_params != 11 && n_params != 13 && n_params != 14)
    return fail(GWF_ERR_INVALID_ARG, "n_params must be 11, 13 or 14");
  if (N < 0 || (N > 0 && (!F || !cov))) return fail(GWF_ERR_INVALID_ARG, "bad covariance arguments");
  if (mem != GWF_MEM_HOST && mem != GWF_MEM_DEVICE) return fail(GWF_ERR_INVALID_ARG, "bad memory mode");
  if (N == 0) return GWF_OK;
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  const size_t mb = (size_t)N * n_params * n_params * sizeof(double);
  if (mem == GWF_MEM_DEVICE) {
    cudaError_t e = gwf::launch_cov(F, N, cov, eps, cond, st, n_params);
    if (e != cudaSuccess) return fail(GWF_ERR_CUDA, cudaGetErrorString(e));
    return GWF_OK;
  }
  if (ctx->fin.ensure(mb) || ctx->fout.ensure(mb) || ctx->feps.ensure(N * sizeof(double)) ||
      ctx->fcond.ensure(N * sizeof(double)))
    return fail(GWF_ERR_OOM, "device allocation failed (cov)");
  GWF_CK(cudaMemcpyAsync(ctx->fin.p, F, mb, cudaMemcpyHostToDevice, st));
  cudaError_t e = gwf::launch_cov((const double*)ctx->fin.p, N, (double*)ctx->fout.p, (double*)ctx->feps.p,
                                  (double*)ctx->fcond.p, st, n_params);
  if (e != cudaSuccess) return fail(GWF_ERR_CUDA, cudaGetErrorString(e));
  GWF_CK(cudaMemcpyAsync(cov, ctx->fout.p, mb, cudaMemcpyDeviceToHost, st));
  if (eps) GWF_CK(cudaMemcpyAsync(eps, ctx->feps.p, N * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (cond) GWF_CK(cudaMemcpyAsync(cond, ctx->fcond.p, N * sizeof(double), cudaMemcpyDeviceToHost, st));
  GWF_CK(cudaStreamSynchronize(st));
  return GWF_OK;
}

int gwf_cov(gwf_ctx* ctx, const double* F, int64_t N, int mem, double* cov, double* eps, double* cond, void* stream) {
  return gwf_cov_n(ctx, F, N, 11, mem, cov, eps, cond, stream);
}

}  // extern "C"
