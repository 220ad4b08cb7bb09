// Mixed precision: the FP32 split-precision Fisher for every event, then FP64 for the events
// whose FP32 network Fisher is ill-conditioned. These kernels pick those events, gather their
// parameters into a compact batch and scatter the FP64 results back.
#include <cuda_runtime.h>
#include <math.h>

#include "gwf_launch.h"

namespace gwf {

namespace {

// Condition-number estimate of the diagonally equilibrated Fisher (the quantity fisherTools
// reports), one thread per event: Cholesky factor, then inverse iteration (two triangular solves
// per step, FP64) for the smallest eigenvalue and power iteration (FP32) for the largest, each
// closed by a Rayleigh quotient. Not positive definite -> infinity. Far cheaper than the Jacobi
// eigen-decomposition of the covariance kernel; only used to pick events for FP64, where a
// factor of a few does not matter: the largest eigenvalue of an equilibrated 11 x 11 matrix lies
// in [1, 11] and the Rayleigh quotients converge quadratically, so 12 and 8 steps suffice.
__global__ void __launch_bounds__(kEvBlock) cond_kernel(const double* __restrict__ F, long long N, double* __restrict__ cond,
                                                       int epw) {
  const long long n = ev_thread(epw);
  if (n < 0 || n >= N) return;
  constexpr int K = NP;
  // the factor is kept as a packed lower triangle and every loop over rows and columns is unrolled,
  // so that it stays in registers (indexed arrays would live in local memory)
  auto T = [](int i, int k) { return i * (i + 1) / 2 + k; };
  const double* f = F + n * K * K;
  double w[K], L[K * (K + 1) / 2], il[K];
#pragma unroll
  for (int i = 0; i < K; ++i) {
    const double d = f[i * K + i];
    if (!(d > 0.0)) { cond[n] = INFINITY; return; }
    w[i] = 1.0 / sqrt(d);
  }
  // Cholesky of A = diag(w) F diag(w)
#pragma unroll
  for (int j = 0; j < K; ++j) {
    double s = f[j * K + j] * w[j] * w[j];
#pragma unroll
    for (int k = 0; k < j; ++k) s -= L[T(j, k)] * L[T(j, k)];
    if (!(s > 0.0)) { cond[n] = INFINITY; return; }
    const double ljj = sqrt(s);
    L[T(j, j)] = ljj;
    il[j] = 1.0 / ljj;
#pragma unroll
    for (int i = j + 1; i < K; ++i) {
      double t = f[i * K + j] * w[i] * w[j];
#pragma unroll
      for (int k = 0; k < j; ++k) t -= L[T(i, k)] * L[T(j, k)];
      L[T(i, j)] = t * il[j];
    }
  }
  double x[K], y[K];
  // smallest eigenvalue: inverse iteration in FP64, x <- A^{-1} x by forward and back substitution;
  // each step grows |x| by up to 1 / lambda_min, so the iterate is renormalised every other step
#pragma unroll
  for (int i = 0; i < K; ++i) x[i] = (i & 1) ? -1.0 : 1.0 + 0.05 * i;
#pragma unroll 1
  for (int it = 0; it < 8; ++it) {
    if ((it & 1) == 0) {
      double s2 = 0.0;
#pragma unroll
      for (int i = 0; i < K; ++i) s2 += x[i] * x[i];
      const double r = rsqrt(s2);
#pragma unroll
      for (int i = 0; i < K; ++i) x[i] *= r;
    }
#pragma unroll
    for (int i = 0; i < K; ++i) {   // L y = x
      double s = x[i];
#pragma unroll
      for (int k = 0; k < i; ++k) s -= L[T(i, k)] * y[k];
      y[i] = s * il[i];
    }
    if (it == 7) break;
#pragma unroll
    for (int i = K - 1; i >= 0; --i) {   // L^T x = y
      double s = y[i];
#pragma unroll
      for (int k = i + 1; k < K; ++k) s -= L[T(k, i)] * x[k];
      x[i] = s * il[i];
    }
  }
  double nx = 0.0, q = 0.0;   // x^T A^{-1} x / |x|^2 = |y|^2 / |x|^2
#pragma unroll
  for (int i = 0; i < K; ++i) {
    nx += x[i] * x[i];
    q += y[i] * y[i];
  }
  const double lmin = nx / q;
  // largest eigenvalue: power iteration on A = L L^T in FP32 (on the FP32 pipe; the FP64 pipe sets
  // this kernel's time). lambda_max lies in [1, 11] and is only needed to a few per cent; rounding L
  // to FP32 moves it by ~1e-7 relative. |A x| <= 11 |x|, so twelve steps from |x| ~ 3.5 stay below
  // 1e13 without renormalisation; the Rayleigh quotient |L^T x|^2 / |x|^2 of the last iterate is
  // the estimate.
  float Lf[K * (K + 1) / 2], xf[K], yf[K];
#pragma unroll
  for (int i = 0; i < K * (K + 1) / 2; ++i) Lf[i] = f32_rn(L[i]);   // (integer rounding, off the FP64 pipe)
#pragma unroll
  for (int i = 0; i < K; ++i) xf[i] = 1.0f + 0.1f * i;
#pragma unroll 1
  for (int it = 0; it < 12; ++it) {
#pragma unroll
    for (int i = 0; i < K; ++i) {   // y = L^T x
      float s = 0.0f;
#pragma unroll
      for (int k = i; k < K; ++k) s = fmaf(Lf[T(k, i)], xf[k], s);
      yf[i] = s;
    }
    if (it == 11) break;
#pragma unroll
    for (int i = 0; i < K; ++i) {   // x = L y
      float s = 0.0f;
#pragma unroll
      for (int k = 0; k <= i; ++k) s = fmaf(Lf[T(i, k)], yf[k], s);
      xf[i] = s;
    }
  }
  float nxf = 0.0f, qf = 0.0f;
#pragma unroll
  for (int i = 0; i < K; ++i) {
    nxf = fmaf(xf[i], xf[i], nxf);
    qf = fmaf(yf[i], yf[i], qf);
  }
  const double lmax = (double)qf / (double)nxf;
  cond[n] = lmax / lmin;
}

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

// dst[idx[m]][j] = sum over s < nslice of src[s][m][j] (slices nslice_stride apart), j < per
__global__ void sum_scatter_kernel(const double* __restrict__ src, int nslice, long long slice_stride,
                                   const long long* __restrict__ idx, long long M, int per, double* __restrict__ dst) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= M * per) return;
  const long long m = t / per;
  const int j = (int)(t - m * per);
  double v = 0.0;
  for (int s = 0; s < nslice; ++s) v += src[s * slice_stride + t];
  dst[idx[m] * per + j] = v;
}

// dst[t] += sum over s < nslice of src[s][t] (slices slice_stride apart), t < n
__global__ void add_slices_kernel(const double* __restrict__ src, int nslice, long long slice_stride, long long n,
                                  double* __restrict__ dst) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  double v = dst[t];
  for (int s = 0; s < nslice; ++s) v += src[s * slice_stride + t];
  dst[t] = v;
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

cudaError_t launch_cond(const double* F, long long N, double* cond, cudaStream_t st) {
  if (N <= 0) return cudaSuccess;
  const int epw = ev_lanes(N);
  cond_kernel<<<ev_blocks(N, epw), kEvBlock, 0, st>>>(F, N, cond, epw);
  return cudaGetLastError();
}

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

cudaError_t launch_sum_scatter(const double* src, int nslice, long long slice_stride, const long long* idx, long long M,
                               int per, double* dst, cudaStream_t st) {
  if (M <= 0) return cudaSuccess;
  sum_scatter_kernel<<<blocks(M * per, 256), 256, 0, st>>>(src, nslice, slice_stride, idx, M, per, dst);
  return cudaGetLastError();
}

cudaError_t launch_add_slices(const double* src, int nslice, long long slice_stride, long long n, double* dst,
                              cudaStream_t st) {
  if (n <= 0 || nslice <= 0) return cudaSuccess;
  add_slices_kernel<<<blocks(n, 256), 256, 0, st>>>(src, nslice, slice_stride, n, dst);
  return cudaGetLastError();
}

cudaError_t launch_scatter(const double* src, const long long* idx, long long M, int per, double* dst, cudaStream_t st) {
  if (M <= 0) return cudaSuccess;
  scatter_kernel<<<blocks(M * per, 256), 256, 0, st>>>(src, idx, M, per, dst);
  return cudaGetLastError();
}

}  // namespace gwf
