// Kernel instantiations for waveform model 0 (one translation unit per model so that the
// three models compile in parallel).  Every launch pair runs the per-event set-up kernel on a
// chunk of events, then the SNR or Fisher kernel on the same chunk.
#include "gwf_launch.h"

namespace gwf {

namespace {

template <class MAIN>
cudaError_t chunked(const LaunchArgs& a, MAIN main) {
  for (long long n0 = 0; n0 < a.ev.N; n0 += kChunk) {
    EvBatch ev = a.ev;
    ev.n0 = n0;
    const long long cnt = (a.ev.N - n0) < kChunk ? (a.ev.N - n0) : kChunk;
    setup_kernel<0><<<(unsigned)((cnt + 63) / 64), 64, 0, a.stream>>>(ev, a.det, a.wf, a.qnm, a.nq, a.scratch, cnt);
    main(ev, cnt);
  }
  return cudaGetLastError();
}

template <bool EARTH, int NARM, int NG>
cudaError_t fisher_one(const LaunchArgs& a) {
  auto k = fisher_kernel<0, EARTH, NARM, NG>;
  const int smem = kWarps * NG * NP * 32 * (int)sizeof(cd);
  cudaError_t err = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (err != cudaSuccess) return err;
  return chunked(a, [&](const EvBatch& ev, long long cnt) {
    k<<<(unsigned)cnt, kThreads, smem, a.stream>>>(ev, a.det, a.scratch, a.out_arm, a.out_det, a.accum);
  });
}

template <bool EARTH, int NARM, int NG>
cudaError_t fisher_one_f32(const LaunchArgs& a) {
  auto k = fisher_kernel_f32<0, EARTH, NARM, NG>;
  const int smem = kWarps * NG * 12 * 32 * (int)sizeof(int2);
  cudaError_t err = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (err != cudaSuccess) return err;
  return chunked(a, [&](const EvBatch& ev, long long cnt) {
    k<<<(unsigned)cnt, kThreads, smem, a.stream>>>(ev, a.det, a.scratch, a.out_arm, a.out_det, a.accum);
  });
}

template <bool EARTH, int NARM>
cudaError_t snr_one(const LaunchArgs& a) {
  return chunked(a, [&](const EvBatch& ev, long long cnt) {
    snr_kernel<0, EARTH, NARM><<<(unsigned)cnt, kThreads, 0, a.stream>>>(ev, a.det, a.scratch, a.out_arm, a.out_det,
                                                                          a.accum);
  });
}

}  // namespace

size_t setup_stride_m0() { return rec_stride<0>(); }

cudaError_t launch_fisher_m0(const LaunchArgs& a) {
  const bool tri = a.det.shape == 1;
  if (a.precision == 1) {
    if (a.det.earth) {
      if (!tri) return fisher_one_f32<true, 1, 1>(a);
      return a.per_arm ? fisher_one_f32<true, 2, 3>(a) : fisher_one_f32<true, 2, 2>(a);
    }
    if (!tri) return fisher_one_f32<false, 1, 1>(a);
    return a.per_arm ? fisher_one_f32<false, 2, 3>(a) : fisher_one_f32<false, 2, 2>(a);
  }
  if (a.det.earth) {
    if (!tri) return fisher_one<true, 1, 1>(a);
    return a.per_arm ? fisher_one<true, 2, 3>(a) : fisher_one<true, 2, 2>(a);
  }
  if (!tri) return fisher_one<false, 1, 1>(a);
  return a.per_arm ? fisher_one<false, 2, 3>(a) : fisher_one<false, 2, 2>(a);
}

cudaError_t launch_snr_m0(const LaunchArgs& a) {
  const bool tri = a.det.shape == 1;
  if (a.det.earth) return tri ? snr_one<true, 2>(a) : snr_one<true, 1>(a);
  return tri ? snr_one<false, 2>(a) : snr_one<false, 1>(a);
}

}  // namespace gwf
