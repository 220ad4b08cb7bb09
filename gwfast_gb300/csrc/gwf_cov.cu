// Batched FP64 covariance: equilibrated Cholesky inverse of NC x NC Fisher matrices (NC = 11, or 13
// for the tidal model).
//
// One thread per event.  Steps (gwfast/fisherTools.py:32-212, 'cho' path):
//  w_i = 1/sqrt(F_ii);  F' = diag(w) F diag(w)
//  eigenvalues of F' (cyclic Jacobi) -> condition number max|l|/min|l|
//  F' = L L^T; C' = L^-T L^-1 (if the factorisation fails, C' = V diag(1/l) V^T, which
//  is what gwfast's SVD fallback yields for a symmetric non-singular matrix)
//  C = diag(w) sym(C') diag(w);  eps = max |C F - 1|
#include <cuda_runtime.h>
#include <math.h>

#include "gwf_launch.h"

namespace gwf {

// cyclic Jacobi: B = A driven to diagonal form; V (if not null) accumulates the rotations. The
// eigenvectors are only needed when the Cholesky factorisation fails, so the common path runs
// without them (a third of each rotation's work) and the rare failure runs the sweeps again.
template <int NC>
__device__ void jacobi(const double* A, double* B, double* V) {
  for (int i = 0; i < NC * NC; ++i) {
    B[i] = A[i];
    if (V) V[i] = (i % (NC + 1) == 0) ? 1.0 : 0.0;
  }
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0, dia = 0.0;
    for (int p = 0; p < NC; ++p) {
      dia += B[p * NC + p] * B[p * NC + p];
      for (int q = p + 1; q < NC; ++q) off += B[p * NC + q] * B[p * NC + q];
    }
    if (off <= 1e-34 * dia) break;
    for (int p = 0; p < NC - 1; ++p)
      for (int q = p + 1; q < NC; ++q) {
        const double apq = B[p * NC + q];
        if (apq == 0.0) continue;
        const double th = (B[q * NC + q] - B[p * NC + p]) / (2.0 * apq);
        const double t = (th >= 0.0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
        const double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
        for (int k = 0; k < NC; ++k) {  // B <- B G (columns p, q)
          const double bkp = B[k * NC + p], bkq = B[k * NC + q];
          B[k * NC + p] = cs * bkp - sn * bkq;
          B[k * NC + q] = sn * bkp + cs * bkq;
        }
        for (int k = 0; k < NC; ++k) {  // B <- G^T B (rows p, q)
          const double bpk = B[p * NC + k], bqk = B[q * NC + k];
          B[p * NC + k] = cs * bpk - sn * bqk;
          B[q * NC + k] = sn * bpk + cs * bqk;
        }
        if (V)
          for (int k = 0; k < NC; ++k) {
            const double vkp = V[k * NC + p], vkq = V[k * NC + q];
            V[k * NC + p] = cs * vkp - sn * vkq;
            V[k * NC + q] = sn * vkp + cs * vkq;
          }
      }
  }
}

template <int NC>
__global__ void cov_kernel(const double* __restrict__ F, long long N, double* __restrict__ cov,
                           double* __restrict__ eps, double* __restrict__ cond) {
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const double* f = F + n * NC * NC;
  double w[NC], A[NC * NC], V[NC * NC], L[NC * NC];
  bool bad = false;
  for (int i = 0; i < NC; ++i) {
    const double d = f[i * NC + i];
    if (!(d > 0.0)) bad = true;
    w[i] = 1.0 / sqrt(d);
  }
  for (int i = 0; i < NC; ++i)
    for (int j = 0; j < NC; ++j) {
      const double a = f[i * NC + j] * w[i] * w[j];
      if (!(a == a)) bad = true;
      A[i * NC + j] = a;
    }
  double* c = cov + n * NC * NC;
  if (bad) {
    for (int i = 0; i < NC * NC; ++i) c[i] = nan("");
    if (eps) eps[n] = nan("");
    if (cond) cond[n] = nan("");
    return;
  }
  // ---- cyclic Jacobi on a copy: B -> diag (the eigenvalues, for the condition number)
  double B[NC * NC];
  jacobi<NC>(A, B, nullptr);
  double lmax = 0.0, lmin = INFINITY;
  bool negative = false;
  for (int i = 0; i < NC; ++i) {
    const double l = B[i * NC + i];
    if (l < 0.0) negative = true;
    lmax = fmax(lmax, fabs(l));
    lmin = fmin(lmin, fabs(l));
  }
  if (cond) cond[n] = lmax / lmin;
  // ---- Cholesky F' = L L^T
  bool chol_ok = !negative;
  for (int i = 0; i < NC * NC; ++i) L[i] = 0.0;
  for (int j = 0; j < NC && chol_ok; ++j) {
    double s = A[j * NC + j];
    for (int k = 0; k < j; ++k) s -= L[j * NC + k] * L[j * NC + k];
    if (!(s > 0.0)) { chol_ok = false; break; }
    const double ljj = sqrt(s);
    L[j * NC + j] = ljj;
    for (int i = j + 1; i < NC; ++i) {
      double t = A[i * NC + j];
      for (int k = 0; k < j; ++k) t -= L[i * NC + k] * L[j * NC + k];
      L[i * NC + j] = t / ljj;
    }
  }
  double C[NC * NC];
  if (chol_ok) {
    // M = L^-1 (lower triangular), C' = M^T M
    double M[NC * NC];
    for (int i = 0; i < NC * NC; ++i) M[i] = 0.0;
    for (int i = 0; i < NC; ++i) {
      M[i * NC + i] = 1.0 / L[i * NC + i];
      for (int j = 0; j < i; ++j) {
        double s = 0.0;
        for (int k = j; k < i; ++k) s += L[i * NC + k] * M[k * NC + j];
        M[i * NC + j] = -s / L[i * NC + i];
      }
    }
    for (int i = 0; i < NC; ++i)
      for (int j = 0; j < NC; ++j) {
        double s = 0.0;
        for (int k = (i > j ? i : j); k < NC; ++k) s += M[k * NC + i] * M[k * NC + j];
        C[i * NC + j] = s;
      }
  } else {   // (rare) the eigen-decomposition again, with its vectors: C' = V diag(1/l) V^T
    jacobi<NC>(A, B, V);
    for (int i = 0; i < NC; ++i)
      for (int j = 0; j < NC; ++j) {
        double s = 0.0;
        for (int k = 0; k < NC; ++k) s += V[i * NC + k] * V[j * NC + k] / B[k * NC + k];
        C[i * NC + j] = s;
      }
  }
  for (int i = 0; i < NC; ++i)
    for (int j = 0; j < NC; ++j) {
      const double s = 0.5 * (C[i * NC + j] + C[j * NC + i]);
      c[i * NC + j] = s * w[i] * w[j];
    }
  if (eps) {
    double e = 0.0;
    for (int i = 0; i < NC; ++i)
      for (int j = 0; j < NC; ++j) {
        double s = 0.0;
        for (int k = 0; k < NC; ++k) s += c[i * NC + k] * f[k * NC + j];
        e = fmax(e, fabs(s - (i == j ? 1.0 : 0.0)));
      }
    eps[n] = e;
  }
}

cudaError_t launch_cov(const double* F, long long N, double* cov, double* eps, double* cond, cudaStream_t st, int np) {
  if (N <= 0) return cudaSuccess;
  const int bs = 64;
  const long long nb = (N + bs - 1) / bs;
  if (np == 14) cov_kernel<14><<<(unsigned)nb, bs, 0, st>>>(F, N, cov, eps, cond);
  else if (np == 13) cov_kernel<13><<<(unsigned)nb, bs, 0, st>>>(F, N, cov, eps, cond);
  else if (np == 11) cov_kernel<11><<<(unsigned)nb, bs, 0, st>>>(F, N, cov, eps, cond);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}

}  // namespace gwf
