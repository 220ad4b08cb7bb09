// Launch descriptors shared by the per-model translation units and the C-ABI layer.
#pragma once
#include <cuda_runtime.h>
#include "gwf_kernels.cuh"

namespace gwf {

constexpr long long kMaxGrid = 1LL << 30;

struct LaunchArgs {
  EvBatch ev;
  DetDev det;
  WfDesc wf;
  const double* qnm;
  int nq;
  double* out_arm;
  double* out_det;
  int accum;
  int per_arm;
  cudaStream_t stream;
};

cudaError_t launch_fisher_m0(const LaunchArgs& a);
cudaError_t launch_fisher_m1(const LaunchArgs& a);
cudaError_t launch_fisher_m2(const LaunchArgs& a);
cudaError_t launch_snr_m0(const LaunchArgs& a);
cudaError_t launch_snr_m1(const LaunchArgs& a);
cudaError_t launch_snr_m2(const LaunchArgs& a);
cudaError_t launch_cov(const double* F, long long N, double* cov, double* eps, double* cond, cudaStream_t st);

}  // namespace gwf
