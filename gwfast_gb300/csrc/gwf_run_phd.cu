// Kernel instantiations for waveform model 1 (one translation unit per model so that
// the three models compile in parallel).
#include "gwf_kernels.cuh"
#include "gwf_launch.h"

namespace gwf {

template <bool EARTH, int NARM, int NG>
static cudaError_t fisher_one(const LaunchArgs& a) {
  auto k = fisher_kernel<1, EARTH, NARM, NG>;
  const int smem = kWarps * NG * NP * 32 * (int)sizeof(cd);
  cudaError_t err = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (err != cudaSuccess) return err;
  for (long long n0 = 0; n0 < a.ev.N; n0 += kMaxGrid) {
    EvBatch ev = a.ev;
    ev.n0 = n0;
    const long long cnt = (a.ev.N - n0) < kMaxGrid ? (a.ev.N - n0) : kMaxGrid;
    k<<<(unsigned)cnt, kThreads, smem, a.stream>>>(ev, a.det, a.wf, a.qnm, a.nq, a.out_arm, a.out_det, a.accum);
  }
  return cudaGetLastError();
}

template <bool EARTH, int NARM>
static cudaError_t snr_one(const LaunchArgs& a) {
  for (long long n0 = 0; n0 < a.ev.N; n0 += kMaxGrid) {
    EvBatch ev = a.ev;
    ev.n0 = n0;
    const long long cnt = (a.ev.N - n0) < kMaxGrid ? (a.ev.N - n0) : kMaxGrid;
    snr_kernel<1, EARTH, NARM><<<(unsigned)cnt, kThreads, 0, a.stream>>>(ev, a.det, a.wf, a.qnm, a.nq, a.out_arm, a.out_det, a.accum);
  }
  return cudaGetLastError();
}

cudaError_t launch_fisher_m1(const LaunchArgs& a) {
  const bool tri = a.det.shape == 1;
  if (a.det.earth) {
    if (!tri) return fisher_one<true, 1, 1>(a);
    return a.per_arm ? fisher_one<true, 2, 3>(a) : fisher_one<true, 2, 2>(a);
  }
  if (!tri) return fisher_one<false, 1, 1>(a);
  return a.per_arm ? fisher_one<false, 2, 3>(a) : fisher_one<false, 2, 2>(a);
}

cudaError_t launch_snr_m1(const LaunchArgs& a) {
  const bool tri = a.det.shape == 1;
  if (a.det.earth) return tri ? snr_one<true, 2>(a) : snr_one<true, 1>(a);
  return tri ? snr_one<false, 2>(a) : snr_one<false, 1>(a);
}

}  // namespace gwf
