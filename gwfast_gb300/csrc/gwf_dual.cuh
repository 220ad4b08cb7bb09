// Forward-mode dual numbers for the analytic tangent of the waveform.
//
// A Dual<T, N> carries a value and its N partial derivatives with respect to the
// intrinsic parameters (Mc, eta, chi1z, chi2z).  Every waveform routine is written
// once, templated on the scalar type, and evaluated either on plain T (SNR: value
// only) or on Dual<T, 4> (Fisher: value and tangent).  The transcendental calls go
// to CUDA's own math functions; derivatives follow from the chain rule.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace gwf {

template <class T> __host__ __device__ __forceinline__ T tsqrt(T x);
template <> __host__ __device__ __forceinline__ double tsqrt(double x) { return sqrt(x); }
template <> __host__ __device__ __forceinline__ float tsqrt(float x) { return sqrtf(x); }
template <class T> __host__ __device__ __forceinline__ T tcbrt(T x);
template <> __host__ __device__ __forceinline__ double tcbrt(double x) { return cbrt(x); }
template <> __host__ __device__ __forceinline__ float tcbrt(float x) { return cbrtf(x); }
template <class T> __host__ __device__ __forceinline__ T texp(T x);
template <> __host__ __device__ __forceinline__ double texp(double x) { return exp(x); }
template <> __host__ __device__ __forceinline__ float texp(float x) { return expf(x); }
template <class T> __host__ __device__ __forceinline__ T tlog(T x);
template <> __host__ __device__ __forceinline__ double tlog(double x) { return log(x); }
template <> __host__ __device__ __forceinline__ float tlog(float x) { return logf(x); }
template <class T> __host__ __device__ __forceinline__ T tatan(T x);
template <> __host__ __device__ __forceinline__ double tatan(double x) { return atan(x); }
template <> __host__ __device__ __forceinline__ float tatan(float x) { return atanf(x); }
template <class T> __host__ __device__ __forceinline__ T tpow(T x, T y);
template <> __host__ __device__ __forceinline__ double tpow(double x, double y) { return pow(x, y); }
template <> __host__ __device__ __forceinline__ float tpow(float x, float y) { return powf(x, y); }
template <class T> __host__ __device__ __forceinline__ T ttanh(T x);
template <> __host__ __device__ __forceinline__ double ttanh(double x) { return tanh(x); }
template <> __host__ __device__ __forceinline__ float ttanh(float x) { return tanhf(x); }
template <class T> __host__ __device__ __forceinline__ void tsincos(T x, T* s, T* c);
template <> __host__ __device__ __forceinline__ void tsincos(double x, double* s, double* c) { sincos(x, s, c); }
template <> __host__ __device__ __forceinline__ void tsincos(float x, float* s, float* c) { sincosf(x, s, c); }

template <class T, int N>
struct Dual {
  T v;
  T d[N];
  Dual() = default;
  __host__ __device__ __forceinline__ Dual(T x) : v(x) {
#pragma unroll
    for (int i = 0; i < N; ++i) d[i] = T(0);
  }
  __host__ __device__ __forceinline__ static Dual seed(T x, int k) {
    Dual r(x);
    r.d[k] = T(1);
    return r;
  }
};

// ---- value access that works for plain scalars and duals
template <class T> __host__ __device__ __forceinline__ T val(T x) { return x; }
template <class T, int N> __host__ __device__ __forceinline__ T val(const Dual<T, N>& x) { return x.v; }

// ---- arithmetic
template <class T, int N>
__host__ __device__ __forceinline__ Dual<T, N> operator+(const Dual<T, N>& a, const Dual<T, N>& b) {
  Dual<T, N> r; r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <class T, int N>
__host__ __device__ __forceinline__ Dual<T, N> operator-(const Dual<T, N>& a, const Dual<T, N>& b) {
  Dual<T, N> r; r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <class T, int N>
__host__ __device__ __forceinline__ Dual<T, N> operator-(const Dual<T, N>& a) {
  Dual<T, N> r; r.v = -a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
  return r;
}
template <class T, int N>
__host__ __device__ __forceinline__ Dual<T, N> operator*(const Dual<T, N>& a, const Dual<T, N>& b) {
  Dual<T, N> r; r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.v * b.d[i] + a.d[i] * b.v;
  return r;
}
template <class T, int N>
__host__ __device__ __forceinline__ Dual<T, N> operator/(const Dual<T, N>& a, const Dual<T, N>& b) {
  Dual<T, N> r; const T ib = T(1) / b.v; r.v = a.v * ib;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
  return r;
}
// scalar on either side
template <class T, int N>
__host__ __device__ __forceinline__ Dual<T, N> operator+(const Dual<T, N>& a, T b) { Dual<T, N> r = a; r.v += b; return r; }
template <class T, int N>
__host__ __device__ __forceinline__ Dual<T, N> operator+(T b, const Dual<T, N>& a) { Dual<T, N> r = a; r.v += b; return r; }
template <class T, int N>
__host__ __device__ __forceinline__ Dual<T, N> operator-(const Dual<T, N>& a, T b) { Dual<T, N> r = a; r.v -= b; return r; }
template <class T, int N>
__host__ __device__ __forceinline__ Dual<T, N> operator-(T b, const Dual<T, N>& a) {
  Dual<T, N> r; r.v = b - a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
  return r;
}
template <class T, int N>
__host__ __device__ __forceinline__ Dual<T, N> operator*(const Dual<T, N>& a, T b) {
  Dual<T, N> r; r.v = a.v * b;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b;
  return r;
}
template <class T, int N>
__host__ __device__ __forceinline__ Dual<T, N> operator*(T b, const Dual<T, N>& a) { return a * b; }
template <class T, int N>
__host__ __device__ __forceinline__ Dual<T, N> operator/(const Dual<T, N>& a, T b) { return a * (T(1) / b); }
template <class T, int N>
__host__ __device__ __forceinline__ Dual<T, N> operator/(T a, const Dual<T, N>& b) {
  Dual<T, N> r; const T ib = T(1) / b.v; r.v = a * ib; const T s = -r.v * ib;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = s * b.d[i];
  return r;
}
template <class T, int N>
__host__ __device__ __forceinline__ Dual<T, N>& operator+=(Dual<T, N>& a, const Dual<T, N>& b) { a = a + b; return a; }
template <class T, int N>
__host__ __device__ __forceinline__ Dual<T, N>& operator-=(Dual<T, N>& a, const Dual<T, N>& b) { a = a - b; return a; }

// chain rule helper: r = f(a) with f'(a) = fp
template <class T, int N>
__host__ __device__ __forceinline__ Dual<T, N> chain(const Dual<T, N>& a, T fv, T fp) {
  Dual<T, N> r; r.v = fv;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = fp * a.d[i];
  return r;
}

// ---- elementary functions (plain overloads forward to the T versions)
template <class T> __host__ __device__ __forceinline__ T dsqrt(T x) { return tsqrt(x); }
template <class T, int N> __host__ __device__ __forceinline__ Dual<T, N> dsqrt(const Dual<T, N>& a) {
  const T s = tsqrt(a.v); return chain(a, s, T(0.5) / s);
}
template <class T> __host__ __device__ __forceinline__ T dcbrt(T x) { return tcbrt(x); }
template <class T, int N> __host__ __device__ __forceinline__ Dual<T, N> dcbrt(const Dual<T, N>& a) {
  const T s = tcbrt(a.v); return chain(a, s, s / (T(3) * a.v));
}
template <class T> __host__ __device__ __forceinline__ T dexp(T x) { return texp(x); }
template <class T, int N> __host__ __device__ __forceinline__ Dual<T, N> dexp(const Dual<T, N>& a) {
  const T e = texp(a.v); return chain(a, e, e);
}
template <class T> __host__ __device__ __forceinline__ T dlog(T x) { return tlog(x); }
template <class T, int N> __host__ __device__ __forceinline__ Dual<T, N> dlog(const Dual<T, N>& a) {
  return chain(a, tlog(a.v), T(1) / a.v);
}
template <class T> __host__ __device__ __forceinline__ T datan(T x) { return tatan(x); }
template <class T, int N> __host__ __device__ __forceinline__ Dual<T, N> datan(const Dual<T, N>& a) {
  return chain(a, tatan(a.v), T(1) / (T(1) + a.v * a.v));
}
// x**p for a constant exponent p
template <class T> __host__ __device__ __forceinline__ T dpowc(T x, T p) { return tpow(x, p); }
template <class T, int N> __host__ __device__ __forceinline__ Dual<T, N> dpowc(const Dual<T, N>& a, T p) {
  const T y = tpow(a.v, p); return chain(a, y, p * y / a.v);
}
template <class T> __host__ __device__ __forceinline__ T dtanh(T x) { return ttanh(x); }
template <class T, int N> __host__ __device__ __forceinline__ Dual<T, N> dtanh(const Dual<T, N>& a) {
  const T t = ttanh(a.v); return chain(a, t, T(1) - t * t);
}
template <class T> __host__ __device__ __forceinline__ T dabs(T x) { return x < T(0) ? -x : x; }
template <class T, int N> __host__ __device__ __forceinline__ Dual<T, N> dabs(const Dual<T, N>& a) {
  return a.v < T(0) ? -a : a;
}
template <class T> __host__ __device__ __forceinline__ void dsincos(T x, T* s, T* c) { tsincos(x, s, c); }
template <class T, int N> __host__ __device__ __forceinline__ void dsincos(const Dual<T, N>& a, Dual<T, N>* s, Dual<T, N>* c) {
  T sv, cv; tsincos(a.v, &sv, &cv);
  *s = chain(a, sv, cv); *c = chain(a, cv, -sv);
}

// ---- Dual<float, 4> on sm_100 and later: the four tangent lanes as two packed FP32x2 pairs, so an
// addition or product of duals issues two instructions for the tangent instead of four. Each lane is
// rounded exactly as the scalar operation (round to nearest); these overloads are more specialised
// than the templates above and take precedence in device code.
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
__device__ __forceinline__ float2 dq01(const Dual<float, 4>& a) { return make_float2(a.d[0], a.d[1]); }
__device__ __forceinline__ float2 dq23(const Dual<float, 4>& a) { return make_float2(a.d[2], a.d[3]); }
__device__ __forceinline__ void dset(Dual<float, 4>& r, float2 lo, float2 hi) {
  r.d[0] = lo.x; r.d[1] = lo.y; r.d[2] = hi.x; r.d[3] = hi.y;
}
__device__ __forceinline__ Dual<float, 4> operator+(const Dual<float, 4>& a, const Dual<float, 4>& b) {
  Dual<float, 4> r; r.v = a.v + b.v;
  dset(r, __fadd2_rn(dq01(a), dq01(b)), __fadd2_rn(dq23(a), dq23(b)));
  return r;
}
__device__ __forceinline__ Dual<float, 4> operator-(const Dual<float, 4>& a, const Dual<float, 4>& b) {
  Dual<float, 4> r; r.v = a.v - b.v;
  dset(r, __fadd2_rn(dq01(a), make_float2(-b.d[0], -b.d[1])), __fadd2_rn(dq23(a), make_float2(-b.d[2], -b.d[3])));
  return r;
}
__device__ __forceinline__ Dual<float, 4> operator*(const Dual<float, 4>& a, const Dual<float, 4>& b) {
  Dual<float, 4> r; r.v = a.v * b.v;
  const float2 av = make_float2(a.v, a.v), bv = make_float2(b.v, b.v);
  dset(r, __ffma2_rn(dq01(a), bv, __fmul2_rn(av, dq01(b))), __ffma2_rn(dq23(a), bv, __fmul2_rn(av, dq23(b))));
  return r;
}
__device__ __forceinline__ Dual<float, 4> operator/(const Dual<float, 4>& a, const Dual<float, 4>& b) {
  Dual<float, 4> r; const float ib = 1.0f / b.v; r.v = a.v * ib;
  const float2 nv = make_float2(-r.v, -r.v), i2 = make_float2(ib, ib);
  dset(r, __fmul2_rn(__ffma2_rn(nv, dq01(b), dq01(a)), i2), __fmul2_rn(__ffma2_rn(nv, dq23(b), dq23(a)), i2));
  return r;
}
__device__ __forceinline__ Dual<float, 4> operator*(const Dual<float, 4>& a, float b) {
  Dual<float, 4> r; r.v = a.v * b;
  const float2 b2 = make_float2(b, b);
  dset(r, __fmul2_rn(dq01(a), b2), __fmul2_rn(dq23(a), b2));
  return r;
}
__device__ __forceinline__ Dual<float, 4> operator*(float b, const Dual<float, 4>& a) { return a * b; }
__device__ __forceinline__ Dual<float, 4> operator/(float a, const Dual<float, 4>& b) {
  Dual<float, 4> r; const float ib = 1.0f / b.v; r.v = a * ib;
  const float s = -r.v * ib;
  const float2 s2 = make_float2(s, s);
  dset(r, __fmul2_rn(dq01(b), s2), __fmul2_rn(dq23(b), s2));
  return r;
}
__device__ __forceinline__ Dual<float, 4> chain(const Dual<float, 4>& a, float fv, float fp) {
  Dual<float, 4> r; r.v = fv;
  const float2 f2 = make_float2(fp, fp);
  dset(r, __fmul2_rn(dq01(a), f2), __fmul2_rn(dq23(a), f2));
  return r;
}
#endif

// select helper that keeps plain and dual code identical
template <class X> __host__ __device__ __forceinline__ X sel(bool c, const X& a, const X& b) { return c ? a : b; }

}  // namespace gwf
