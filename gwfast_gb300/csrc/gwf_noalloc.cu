// Fisher entry point that allocates no device memory (gwf_fisher_noalloc, include/gwfast_gb300.h).
//
// Who needs it: callers that cannot call cudaMalloc. Typical cases are programs whose device
// memory is owned by their own pool allocator (a framework that reserves most of the GPU at
// start-up and hands out sub-blocks, so a library's own cudaMalloc either fails or fragments
// the pool), and real-time loops that cannot afford cudaMalloc/cudaFree, which synchronise
// the device. Such callers own the inputs and outputs; the entry point needs only scratch
// space, and that lives in one fixed-size array in this file.
//
// The scratch is a file-scope __device__ array: every GPU that loads the library holds it
// (kScratchBytes) until the process exits. In host code its name is only a host-side stand-in,
// so its device address is looked up with cudaGetSymbolAddress. The lookup is done by the first
// call made in a CUDA context (with that context's device current) and cached under the
// context's unique ID, so a context created later on the same device (after cudaDeviceReset, or a
// caller's own context) gets its own lookup instead of a stale address; that first call in a
// context should come before any stream capture in it. All calls share the array and it keeps the
// last call's contents. Each call rewrites every byte it reads (PSD and QNM tables, PSD index,
// per-event set-up records) before its kernels read them, so nothing has to start at zero. Calls
// whose GPU work overlaps (different streams without ordering) race on the array.
#include <cuda.h>   // CUcontext and the driver function types only (no link against libcuda)
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "gwf_launch.h"
#include "gwfast_gb300.h"

namespace gwf {
void set_last_error(const char* msg);  // gwf_api.cu
}

namespace {

constexpr size_t kScratchBytes = (size_t)GWF_NOALLOC_SCRATCH_MIB << 20;
constexpr int kAccBins = 4096;
// section offsets inside the scratch (each 256-byte aligned)
constexpr size_t kOffPsdF = 0;
constexpr size_t kOffPsdS = kOffPsdF + (size_t)GWF_NOALLOC_MAX_PSD * sizeof(double);
constexpr size_t kOffAcc = kOffPsdS + (size_t)GWF_NOALLOC_MAX_PSD * sizeof(double);
constexpr size_t kOffQnm = kOffAcc + (size_t)kAccBins * sizeof(int);
constexpr size_t kOffRec = kOffQnm + 3 * (size_t)GWF_NOALLOC_MAX_QNM * sizeof(double);
static_assert(kOffRec % 256 == 0, "scratch sections must stay 256-byte aligned");
static_assert(kOffRec < kScratchBytes, "scratch too small for its tables");

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace {

std::mutex g_mu;

int fail(int code, const char* msg) {
  gwf::set_last_error(msg);
  return code;
}

// unique ID of the current CUDA context (0 when none is current yet); the driver functions come
// through the runtime's entry-point query, so the library needs no link against libcuda
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_get_current = nullptr;
CtxGetIdFn g_get_id = nullptr;

int current_ctx_id(unsigned long long* id) {
  *id = 0;
  if (!g_get_current || !g_get_id) {
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 4000, cudaEnableDefault, &q1) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
      return fail(GWF_ERR_CUDA, "gwf_fisher_noalloc: cuCtxGetCurrent/cuCtxGetId not available from the driver");
    g_get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
    g_get_id = reinterpret_cast<CtxGetIdFn>(f2);
  }
  CUcontext c = nullptr;
  if (g_get_current(&c) != CUDA_SUCCESS) return fail(GWF_ERR_CUDA, "gwf_fisher_noalloc: cuCtxGetCurrent failed");
  if (c && g_get_id(c, id) != CUDA_SUCCESS) return fail(GWF_ERR_CUDA, "gwf_fisher_noalloc: cuCtxGetId failed");
  return GWF_OK;
}

// scratch addresses already looked up, keyed by context ID (oldest entry replaced when full)
constexpr int kCacheSlots = 64;
unsigned long long g_ctx_id[kCacheSlots] = {};
unsigned char* g_ptr[kCacheSlots] = {};
int g_next_slot = 0;

// device address of the scratch in the current context, looked up on the first call in it
int scratch_ptr(unsigned char** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0)
    return fail(GWF_ERR_CUDA, "gwf_fisher_noalloc: no usable current CUDA device");
  std::lock_guard<std::mutex> lock(g_mu);
  unsigned long long id = 0;
  int rc = current_ctx_id(&id);
  if (rc) return rc;
  if (id)
    for (int i = 0; i < kCacheSlots; ++i)
      if (g_ctx_id[i] == id) {
        *out = g_ptr[i];
        return GWF_OK;
      }
  // first call in this context (the lookup also makes the device's primary context current when
  // the runtime has not done so yet)
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p) {
    gwf::set_last_error(cudaGetErrorString(e));
    return GWF_ERR_CUDA;
  }
  if (!id) {
    rc = current_ctx_id(&id);
    if (rc) return rc;
  }
  if (id) {
    g_ctx_id[g_next_slot] = id;
    g_ptr[g_next_slot] = static_cast<unsigned char*>(p);
    g_next_slot = (g_next_slot + 1) % kCacheSlots;
  }
  *out = static_cast<unsigned char*>(p);
  return GWF_OK;
}

// PSD index: for each of nacc log-frequency bins, the last table row at or below the bin's lower
// edge (a starting point for the lookup, which corrects it in either direction), by binary search
__global__ void psd_index_kernel(const double* psd_f, int n, double l0, double idl, int* acc, int nacc) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nacc) return;
  const double fb = exp(l0 + b / idl);
  int lo = 0, hi = n - 2;   // answer in [0, n - 2]
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (psd_f[mid] <= fb) lo = mid;
    else hi = mid - 1;
  }
  acc[b] = lo;
}

}  // namespace

extern "C" int gwf_fisher_noalloc(const gwf_det_desc* det, const double* psd_f, const double* psd_S, int64_t n_psd,
                                  const gwf_wf_desc* wf, const double* qnm_spin, const double* qnm_fring,
                                  const double* qnm_fdamp, int64_t n_qnm, const double* params, int64_t ld,
                                  int64_t n_events, int32_t res, int accumulate, double* out, void* stream) {
  if (!det || !psd_f || !psd_S || !wf) return fail(GWF_ERR_INVALID_ARG, "gwf_fisher_noalloc: null argument");
  if (det->shape != GWF_SHAPE_L && det->shape != GWF_SHAPE_T)
    return fail(GWF_ERR_INVALID_ARG, "Enter valid detector configuration");
  if (!(det->fmin > 0.0)) return fail(GWF_ERR_INVALID_ARG, "fmin must be positive");
  if (n_psd < 2) return fail(GWF_ERR_INVALID_ARG, "PSD table needs at least two rows");
  if (n_psd > GWF_NOALLOC_MAX_PSD)
    return fail(GWF_ERR_INVALID_ARG, "gwf_fisher_noalloc: PSD table longer than GWF_NOALLOC_MAX_PSD (16384) rows");
  for (int64_t i = 0; i < n_psd; ++i) {
    if (!(psd_f[i] > 0.0)) return fail(GWF_ERR_INVALID_ARG, "PSD frequencies must be positive");
    if (i && !(psd_f[i] > psd_f[i - 1])) return fail(GWF_ERR_INVALID_ARG, "PSD frequencies must be strictly increasing");
  }
  if (wf->model < 0 || wf->model > 2) return fail(GWF_ERR_INVALID_ARG, "unknown waveform model");
  if (wf->flags & ~(GWF_TF2_PHIREF_VLSO | GWF_TF2_KERR_ISCO)) return fail(GWF_ERR_INVALID_ARG, "unknown waveform flags");
  if (wf->flags && wf->model != GWF_WF_TAYLORF2)
    return fail(GWF_ERR_INVALID_ARG, "waveform flags apply to the TaylorF2 models only");
  if (!(wf->fcut_par > 0.0)) return fail(GWF_ERR_INVALID_ARG, "fcut_par must be positive");
  if (wf->model == GWF_WF_PHENOMD) {
    if (!qnm_spin || !qnm_fring || !qnm_fdamp || n_qnm < 2)
      return fail(GWF_ERR_INVALID_ARG, "IMRPhenomD needs the QNM table");
    if (n_qnm > GWF_NOALLOC_MAX_QNM)
      return fail(GWF_ERR_INVALID_ARG, "gwf_fisher_noalloc: QNM table longer than GWF_NOALLOC_MAX_QNM (2048) rows");
    for (int64_t i = 1; i < n_qnm; ++i)
      if (!(qnm_spin[i] > qnm_spin[i - 1])) return fail(GWF_ERR_INVALID_ARG, "QNM spin grid must be strictly increasing");
  }
  if (n_events < 0 || (n_events > 0 && (!params || !out))) return fail(GWF_ERR_INVALID_ARG, "bad event or output array");
  if (ld < n_events) return fail(GWF_ERR_INVALID_ARG, "ld must be >= n_events");
  if (res < 1) return fail(GWF_ERR_INVALID_ARG, "res must be >= 1");
  if (n_events == 0) return GWF_OK;

  unsigned char* base = nullptr;
  int rc = scratch_ptr(&base);
  if (rc) return rc;
  const cudaStream_t st = (cudaStream_t)stream;

  // PSD table and the QNM table are copied into the scratch; the PSD index is built there on the
  // device from the copied table (no library-owned host buffer is copied)
  const double l0 = std::log(psd_f[0]);
  const double idl = kAccBins / (std::log(psd_f[n_psd - 1]) - l0);
  cudaError_t e = cudaMemcpyAsync(base + kOffPsdF, psd_f, n_psd * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(base + kOffPsdS, psd_S, n_psd * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    psd_index_kernel<<<(kAccBins + 255) / 256, 256, 0, st>>>(reinterpret_cast<const double*>(base + kOffPsdF),
                                                            (int)n_psd, l0, idl, reinterpret_cast<int*>(base + kOffAcc),
                                                            kAccBins);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && wf->model == GWF_WF_PHENOMD) {
    double* q = reinterpret_cast<double*>(base + kOffQnm);
    e = cudaMemcpyAsync(q, qnm_spin, n_qnm * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(q + n_qnm, qnm_fring, n_qnm * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(q + 2 * n_qnm, qnm_fdamp, n_qnm * sizeof(double), cudaMemcpyHostToDevice, st);
  }
  // (copies from pageable host memory return once the source has been read; copies from
  // page-locked memory read it when the stream reaches them)
  if (e != cudaSuccess) return fail(GWF_ERR_CUDA, cudaGetErrorString(e));

  gwf::LaunchArgs a;
  a.det.lat = det->lat_rad;
  a.det.lon = det->long_rad;
  a.det.xax = det->xax_rad;
  a.det.shape = det->shape;
  a.det.sin_zeta = det->shape == GWF_SHAPE_T ? std::sin(M_PI / 3.0) : 1.0;
  a.det.fmin = det->fmin;
  a.det.fmax = det->fmax;
  a.det.earth = det->earth_rotation;
  a.det.psd_f = reinterpret_cast<const double*>(base + kOffPsdF);
  a.det.psd_S = reinterpret_cast<const double*>(base + kOffPsdS);
  a.det.npsd = (int)n_psd;
  a.det.acc = reinterpret_cast<const int*>(base + kOffAcc);
  a.det.nacc = kAccBins;
  a.det.acc_l0 = l0;
  a.det.acc_idl = idl;
  a.det.psd_seg = nullptr;
  a.det.psd_f32_lo = a.det.psd_f32_hi = 0.0f;
  a.det.psd_scale = 1.0;
  gwf::det_trig(a.det);
  a.wf.model = wf->model;
  a.wf.spin_ho = wf->spin_ho;
  a.wf.fcut_par = wf->fcut_par;
  a.wf.flags = wf->flags;
  a.wf.pad_ = 0;
  a.wf.fref_ecc = wf->fref_ecc;
  a.qnm = reinterpret_cast<const double*>(base + kOffQnm);
  a.nq = wf->model == GWF_WF_PHENOMD ? (int)n_qnm : 0;
  a.out_arm = nullptr;
  a.accum = accumulate ? 1 : 0;
  a.per_arm = 0;
  a.precision = GWF_PREC_FP64;
  a.scratch = base + kOffRec;
  a.stream = st;
  const size_t stride = wf->model == 0 ? gwf::setup_stride_m0() : (wf->model == 1 ? gwf::setup_stride_m1() : gwf::setup_stride_m2());
  long long per_pass = (long long)((kScratchBytes - kOffRec) / stride);
  if (per_pass > gwf::kChunk) per_pass = gwf::kChunk;
  a.cap_events = per_pass;
  // events are processed in passes that fit the set-up records into the scratch
  for (long long s0 = 0; s0 < n_events; s0 += per_pass) {
    const long long cnt = (n_events - s0) < per_pass ? (n_events - s0) : per_pass;
    a.ev.p = params + s0;
    a.ev.ld = ld;
    a.ev.N = cnt;
    a.ev.n0 = 0;
    a.ev.res = res;
    a.ev.res_ev = nullptr;
    a.ev.spacing = GWF_SPACING_GEOM;
    a.out_det = out + (size_t)s0 * gwf::NP * gwf::NP;
    e = wf->model == 0 ? gwf::launch_fisher_m0(a) : (wf->model == 1 ? gwf::launch_fisher_m1(a) : gwf::launch_fisher_m2(a));
    if (e != cudaSuccess) return fail(GWF_ERR_CUDA, cudaGetErrorString(e));
  }
  return GWF_OK;
}
