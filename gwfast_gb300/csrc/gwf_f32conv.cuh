// FP64 -> FP32 rounding with integer instructions.
//
// The double -> float conversion instruction issues on the FP64 pipe, which bounds the kernels that
// use it most (the per-event FP32 records, the condition estimate's FP32 factor, the FP32 form of
// IMRPhenomHM with its FP64 mode phases). These functions do the same IEEE round-to-nearest-even on
// the bit patterns with 32-bit integer operations (ALU pipe) for results in the normal FP32 range,
// and hand every other case (FP32 subnormal or overflow, infinity, NaN) to the conversion
// instruction; signed zeros stay on the integer path. The result is the bit pattern of a plain cast.
//
// Bit layout: double = sign | 11-bit exponent e (bias 1023) | 52-bit mantissa; float = sign |
// 8-bit exponent (bias 127) | 23-bit mantissa. A double with e in [897, 1150] rounds to a normal
// float with exponent field e - 896 (or to the next binade, or to infinity from e = 1150, when the
// rounding carries out of the mantissa: adding the carry to the packed exponent|mantissa word does
// exactly that).
#pragma once
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define GWF_CONV_HD __host__ __device__ __forceinline__
#else
#define GWF_CONV_HD inline
#endif

namespace gwf {

GWF_CONV_HD uint64_t conv_bits(double v) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(v);
#else
  uint64_t u;
  memcpy(&u, &v, sizeof u);
  return u;
#endif
}
GWF_CONV_HD float conv_float(uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(b);
#else
  float f;
  memcpy(&f, &b, sizeof f);
  return f;
#endif
}

// (float)v
GWF_CONV_HD float f32_rn(double v) {
  const uint64_t u = conv_bits(v);
  const uint32_t hi = (uint32_t)(u >> 32), lo = (uint32_t)u;
  const uint32_t e = (hi >> 20) & 0x7FFu;
  if (e - 897u > 253u) {   // e outside [897, 1150] (e < 897 wraps round)
    if (((hi & 0x7FFFFFFFu) | lo) == 0u) return conv_float(hi);   // +-0
    return (float)v;
  }
  // exponent and the top 23 mantissa bits, rebased from bias 1023 to 127; 29 bits dropped
  uint32_t f = ((((hi & 0x7FFFFFFFu) << 3) | (lo >> 29)) - (896u << 23));
  const uint32_t r = lo & 0x1FFFFFFFu;
  f += (r + (f & 1u) + 0x0FFFFFFFu) >> 29;   // 1 above half, or at half with an odd result
  return conv_float(f | (hi & 0x80000000u));
}

// h = (float)v and l = (float)(v - (double)h): the FP32 pair that carries v to ~48 bits. The
// difference v - h is exact in FP64; it is the dropped 29 bits less the carry of the rounding, in
// units of 2^(E - 52) (E = e - 1023): an integer |t| <= 2^28, converted to float (the same rounding
// as the cast of v - h) and scaled by that power of two. Where the scaled result could leave the
// normal FP32 range the plain FP64 operations are used.
GWF_CONV_HD void f32_split(double v, float& h, float& l) {
  const uint64_t u = conv_bits(v);
  const uint32_t hi = (uint32_t)(u >> 32), lo = (uint32_t)u;
  const uint32_t e = (hi >> 20) & 0x7FFu;
  // e - 52 - 1023 + 127 >= 1 keeps 2^(E - 52) a normal float; e <= 1149 keeps h finite
  if (e - 949u > 200u) {
    if (((hi & 0x7FFFFFFFu) | lo) == 0u) {   // +-0: (+-0, +0)
      h = conv_float(hi);
      l = 0.0f;
      return;
    }
    h = (float)v;
    l = (float)(v - (double)h);
    return;
  }
  uint32_t f = ((((hi & 0x7FFFFFFFu) << 3) | (lo >> 29)) - (896u << 23));
  const uint32_t r = lo & 0x1FFFFFFFu;
  const uint32_t up = (r + (f & 1u) + 0x0FFFFFFFu) >> 29;
  f += up;
  const uint32_t sgn = hi & 0x80000000u;
  h = conv_float(f | sgn);
  const int32_t t = (int32_t)r - (int32_t)(up << 29);   // |v| - |h| in units of 2^(E - 52)
  const float scale = conv_float((e - 948u) << 23);     // 2^(e - 1023 - 52), exponent field e - 948
  // (an exact zero difference is +0, as v - h is in FP64)
  l = (float)(sgn ? -t : t) * scale;                    // exact scaling of the rounded integer
}

}  // namespace gwf
