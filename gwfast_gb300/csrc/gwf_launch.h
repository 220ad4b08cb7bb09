// Launch descriptors shared by the per-model translation units and the C-ABI layer.
#pragma once
#include <cuda_runtime.h>
#include "gwfast_gb300.h"
#include "gwf_kernels_f32.cuh"
#include "gwf_wave_out.cuh"

namespace gwf {

// events per set-up/main launch pair (bounds the set-up scratch: chunk x record stride)
constexpr long long kChunk = 16384;

// SMs of the current device (cached per device ordinal)
inline int device_sms() {
  static int cache[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) dev = 0;
  if (dev < 64 && cache[dev] > 0) return cache[dev];
  int n = 0;
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  n = n > 0 ? n : 1;
  if (dev < 64) cache[dev] = n;
  return n;
}

// Launch shape of the per-event kernels (ev_thread): full warps once a batch of cnt events gives
// every SM kEvWarpsPerSM warps, fewer events per warp below that (at least kEvMinLanes). The FP64
// pipe charges a warp instruction the same however few lanes are active, so spreading further
// costs more than it hides: for 10^4 IMRPhenomD events the first set-up took 0.437 ms in full warps
// (2 per SM), 0.416 ms at 4 warps per SM, 0.61 ms at 8 and 1.43 ms at 32.
constexpr int kEvWarpsPerSM = 4;
constexpr int kEvMinLanes = 4;
// the FP32 record kernel (setup_f32_kernel) does little FP64 work per event (its conversions run on
// the integer pipe; FP64 pipe 23 % busy) and moves ~3 KB per event; more warps per SM still do not
// pay: the L1 + H1 set-up section (10^4 events) took 0.326 ms at 4 warps per SM, 0.330 at 8 and
// 0.341 at 16
constexpr int kRecWarpsPerSM = 4;
inline int ev_lanes(long long cnt, int warps_per_sm = kEvWarpsPerSM) {
  const long long warps = (long long)warps_per_sm * device_sms();
  long long epw = (cnt + warps - 1) / warps;
  epw = epw < kEvMinLanes ? kEvMinLanes : (epw > 32 ? 32 : epw);
  return (int)epw;
}
inline unsigned ev_blocks(long long cnt, int epw) {
  const long long warps = (cnt + epw - 1) / epw;
  return (unsigned)((warps + kEvBlock / 32 - 1) / (kEvBlock / 32));
}

// Optional CUDA-event timing of the main launches of one call (gwf_set_kernel_timing): a start and
// a stop event around each timed section on the stream it runs on. Nothing is recorded inside a
// stream capture or once kMax sections are taken.
struct KernelTimer {
  static constexpr int kMax = 64;
  cudaEvent_t ev[2 * kMax] = {};
  int kind[kMax] = {};
  int n = 0;
  bool open = false;
  static bool capturing(cudaStream_t st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    return cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone;
  }
  cudaError_t begin(cudaStream_t st, int k) {
    if (open || n >= kMax || capturing(st)) return cudaSuccess;
    kind[n] = k;
    open = true;
    return cudaEventRecord(ev[2 * n], st);
  }
  cudaError_t end(cudaStream_t st) {
    if (!open) return cudaSuccess;
    open = false;
    return cudaEventRecord(ev[2 * n++ + 1], st);
  }
};

struct LaunchArgs {
  EvBatch ev;
  DetDev det;
  WfDesc wf;
  const double* qnm;
  int nq;
  double* out_arm;
  double* out_det;
  double* out_sd_arm = nullptr;   // Re<dh/dtheta | h> per arm slot [slots][N][11] (SNR derivatives), or null
  double* out_sd_det = nullptr;   // the same summed over the detector's arms [N][11] (+= when accum)
  int accum;
  int per_arm;
  int precision;  // 0 = FP64, 1 = FP32 split precision (22-mode models); the launchers see no other value
  unsigned char* scratch;  // cap_events x setup_stride(model) bytes: FP64 records, then FP32 records
  long long cap_events;    // events the scratch holds (locates the FP32 records)
  cudaStream_t stream;
  // segmented persistent launches (seg > 0: points per segment, a multiple of kThreads)
  int seg = 0;
  long long* seg_off = nullptr;            // kChunk + 1
  unsigned long long* seg_ctr = nullptr;   // item counter
  double* seg_part = nullptr;              // seg_cap x 3 x 77 partial Grams
  long long seg_cap = 0;
  int* seg_ovf = nullptr;                  // set if the items exceed seg_cap
  // cache of the source-dependent model records across the detectors of one call (see setup_kernel)
  unsigned char* core = nullptr;           // N x core_bytes(model)
  int core_mode = 0;                       // 0: none, 1: compute and store, 2: load
  const long long* core_idx = nullptr;     // cache row of each event of a gathered batch
  cudaEvent_t core_done = nullptr;         // recorded after each set-up that stores into the cache
  // FP64 set-up records of this detector for the whole batch, left by an earlier pass of the same
  // call (event n at rec_src + n * rec_stride): a gathered batch (core_idx) copies its rows from
  // there instead of running the set-up again
  const unsigned char* rec_src = nullptr;
  // rec_src holds another detector's records (a detector group shares grid and model): the copied
  // rows get this detector's projection header
  int rec_patch_proj = 0;
  KernelTimer* timer = nullptr;            // gwf_set_kernel_timing: events around the main launches
};

cudaError_t launch_fisher_m0(const LaunchArgs& a);
cudaError_t launch_fisher_m1(const LaunchArgs& a);
cudaError_t launch_fisher_m2(const LaunchArgs& a);
cudaError_t launch_snr_m0(const LaunchArgs& a);
cudaError_t launch_snr_m1(const LaunchArgs& a);
cudaError_t launch_snr_m2(const LaunchArgs& a);
cudaError_t launch_fisher_m3(const LaunchArgs& a);   // tidal TaylorF2: FP64, 13 parameters
cudaError_t launch_snr_m3(const LaunchArgs& a);
size_t setup_stride_m3();
size_t core_bytes_m3();
cudaError_t launch_fisher_m4(const LaunchArgs& a);   // IMRPhenomD_NRTidalv2: FP64, 13 parameters
cudaError_t launch_snr_m4(const LaunchArgs& a);
size_t setup_stride_m4();
size_t core_bytes_m4();
cudaError_t launch_fisher_m5(const LaunchArgs& a);   // eccentric TaylorF2: FP64, 12 parameters
cudaError_t launch_snr_m5(const LaunchArgs& a);
size_t setup_stride_m5();
size_t core_bytes_m5();
cudaError_t launch_fisher_m6(const LaunchArgs& a);   // tidal eccentric TaylorF2: FP64, 14 parameters
cudaError_t launch_snr_m6(const LaunchArgs& a);
size_t setup_stride_m6();
size_t core_bytes_m6();
cudaError_t launch_fisher_m7(const LaunchArgs& a);   // IMRPhenomNSBH: FP64, 13 parameters
cudaError_t launch_snr_m7(const LaunchArgs& a);
size_t setup_stride_m7();
size_t core_bytes_m7();
// IMRPhenomNSBH xi_tide table (200^3 doubles) and its interpolation at given points
cudaError_t launch_xitide_table(double* tab, cudaStream_t st);
cudaError_t launch_xitide_eval(const double* tab, const double* C, const double* q, const double* chi, long long n,
                               double* out, cudaStream_t st);
// strain tangent / strain / overlap outputs (gwf_wave_out.cuh): set-up and output launch for
// events [o.n0, o.n0 + o.cnt) of a.ev; a.scratch holds at least o.cnt records
cudaError_t launch_wave_m0(const LaunchArgs& a, const WaveOut& o);
cudaError_t launch_wave_m1(const LaunchArgs& a, const WaveOut& o);
cudaError_t launch_wave_m2(const LaunchArgs& a, const WaveOut& o);
cudaError_t launch_wave_m3(const LaunchArgs& a, const WaveOut& o);
cudaError_t launch_wave_m4(const LaunchArgs& a, const WaveOut& o);
cudaError_t launch_wave_m5(const LaunchArgs& a, const WaveOut& o);
cudaError_t launch_wave_m6(const LaunchArgs& a, const WaveOut& o);
cudaError_t launch_wave_m7(const LaunchArgs& a, const WaveOut& o);
// FP32 network total of a group of detectors sharing the grid (gwf_kernels_f32.cuh); a.det is the
// group's first detector, a.scratch holds g.nd slices of a.cap_events set-up records
cudaError_t launch_group_m0(const LaunchArgs& a, const GroupDev& g);
cudaError_t launch_group_m1(const LaunchArgs& a, const GroupDev& g);
cudaError_t launch_group_m2(const LaunchArgs& a, const GroupDev& g);
// FP64 network total of a group of detectors sharing the grid (11-parameter models): per
// detector its set-up record slice (a.cap_events records) and, for a gathered batch (a.core_idx),
// where its records are copied from; a.seg > 0: segmented launch with a's segment buffers
struct Group64 {
  int nd = 0;
  DetDev det[kMaxGroup];
  int same_psd[kMaxGroup] = {};
  unsigned char* scratch[kMaxGroup] = {};
  const unsigned char* rec_src[kMaxGroup] = {};   // null: the set-up runs (detector 0) or only the header
  int patch[kMaxGroup] = {};                       // rec_src is another detector's: recompute the header
  double* out_arm[kMaxGroup] = {};                 // SNR: each detector's per-arm slots (or null)
};
cudaError_t launch_group64_m0(const LaunchArgs& a, const Group64& g);
cudaError_t launch_group64_m1(const LaunchArgs& a, const Group64& g);
cudaError_t launch_group64_m2(const LaunchArgs& a, const Group64& g);
// FP64 SNR of such a group (network total into a.out_det, per-arm slots into g.out_arm)
cudaError_t launch_snr_group64_m0(const LaunchArgs& a, const Group64& g);
cudaError_t launch_snr_group64_m1(const LaunchArgs& a, const Group64& g);
cudaError_t launch_snr_group64_m2(const LaunchArgs& a, const Group64& g);
// FP32 SNR of a group (a.scratch holds g.nd slices of a.cap_events set-up records; g.scratch unused)
cudaError_t launch_snr_group_f32_m0(const LaunchArgs& a, const Group64& g);
cudaError_t launch_snr_group_f32_m1(const LaunchArgs& a, const Group64& g);
cudaError_t launch_snr_group_f32_m2(const LaunchArgs& a, const Group64& g);
size_t setup_stride_m0();
size_t core_bytes_m0();
size_t core_bytes_m1();
size_t core_bytes_m2();
size_t setup_stride_m1();
size_t setup_stride_m2();
cudaError_t launch_cov(const double* F, long long N, double* cov, double* eps, double* cond, cudaStream_t st,
                       int np = NP);
// mixed precision (gwf_mixed.cu)
cudaError_t launch_cond(const double* F, long long N, double* cond, cudaStream_t st);
cudaError_t launch_select(const double* cond, long long N, double thresh, long long* idx, unsigned long long* count,
                          cudaStream_t st);
cudaError_t launch_gather(const double* p, long long ld, const int* res, const long long* idx, long long M, double* out,
                          int* res_out, cudaStream_t st);
cudaError_t launch_scatter(const double* src, const long long* idx, long long M, int per, double* dst, cudaStream_t st);
cudaError_t launch_add_slices(const double* src, int nslice, long long slice_stride, long long n, double* dst,
                              cudaStream_t st);
cudaError_t launch_sum_scatter(const double* src, int nslice, long long slice_stride, const long long* idx, long long M,
                               int per, double* dst, cudaStream_t st);

}  // namespace gwf
