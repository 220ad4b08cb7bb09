// Mixed precision: the FP32 split-precision Fisher for every event, then FP64 for the events
// whose FP32 network Fisher is ill-conditioned. These kernels pick those events, gather their
// parameters into a compact batch and scatter the FP64 results back.
#include <cuda_runtime.h>

#include "gwf_launch.h"

namespace gwf {

namespace {

// events with condition number above thresh (or not finite) -> idx[0..count)
__global__ void select_kernel(const double* __restrict__ cond, long long N, double thresh, long long* __restrict__ idx,
                              unsigned long long* __restrict__ count) {
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  if (!(cond[n] <= thresh)) idx[atomicAdd(count, 1ull)] = n;
}

// out[k][m] = p[k * ld + idx[m]] (and the per-event resolutions, when given)
__global__ void gather_kernel(const double* __restrict__ p, long long ld, const int* __restrict__ res,
                              const long long* __restrict__ idx, long long M, double* __restrict__ out,
                              int* __restrict__ res_out) {
  const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M) return;
  const long long n = idx[m];
#pragma unroll
  for (int k = 0; k < NP; ++k) out[k * M + m] = p[k * ld + n];
  if (res) res_out[m] = res[n];
}

// dst[idx[m]][j] = src[m][j], j < per
__global__ void scatter_kernel(const double* __restrict__ src, const long long* __restrict__ idx, long long M,
                               int per, double* __restrict__ dst) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= M * per) return;
  const long long m = t / per;
  const int j = (int)(t - m * per);
  dst[idx[m] * per + j] = src[t];
}

unsigned blocks(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

}  // namespace

cudaError_t launch_select(const double* cond, long long N, double thresh, long long* idx, unsigned long long* count,
                          cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(count, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess || N <= 0) return e;
  select_kernel<<<blocks(N, 256), 256, 0, st>>>(cond, N, thresh, idx, count);
  return cudaGetLastError();
}

cudaError_t launch_gather(const double* p, long long ld, const int* res, const long long* idx, long long M, double* out,
                          int* res_out, cudaStream_t st) {
  if (M <= 0) return cudaSuccess;
  gather_kernel<<<blocks(M, 256), 256, 0, st>>>(p, ld, res, idx, M, out, res_out);
  return cudaGetLastError();
}

cudaError_t launch_scatter(const double* src, const long long* idx, long long M, int per, double* dst, cudaStream_t st) {
  if (M <= 0) return cudaSuccess;
  scatter_kernel<<<blocks(M * per, 256), 256, 0, st>>>(src, idx, M, per, dst);
  return cudaGetLastError();
}

}  // namespace gwf
