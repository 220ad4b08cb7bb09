// Host check of gwf_f32conv.cuh: f32_rn(v) must give the bit pattern of (float)v, and f32_split(v)
// that of ((float)v, (float)(v - (double)(float)v)), for random bit patterns, random normal values
// over the FP32 range and beyond, round-to-nearest-even ties and near-ties, mantissas that carry into
// the exponent, and the special values. Prints the count of mismatches; exit status 1 if any.
#include "gwf_f32conv.cuh"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>

int main(int argc, char** argv) {
  const long long reps = argc > 1 ? atoll(argv[1]) : 4000000;
  std::mt19937_64 g(20261204);
  long long bad = 0, n = 0;
  auto bits = [](float f) { uint32_t u; memcpy(&u, &f, 4); return u; };
  auto chk = [&](double v) {
    ++n;
    float h, l;
    gwf::f32_split(v, h, l);
    const float h2 = (float)v, l2 = (float)(v - (double)h2);
    if (bits(gwf::f32_rn(v)) != bits(h2) || bits(h) != bits(h2) || bits(l) != bits(l2)) {
      if (bad < 5) printf("mismatch at %a\n", v);
      ++bad;
    }
  };
  for (long long i = 0; i < reps; ++i) {   // any bit pattern (NaNs, infinities, subnormals included)
    const uint64_t u = g();
    double v;
    memcpy(&v, &u, 8);
    chk(v);
  }
  for (long long i = 0; i < reps; ++i) {   // normal values from 2^-150 to 2^150, either sign
    const double m = (double)(g() >> 11) / 9007199254740992.0 + 0.5;
    chk(std::ldexp(m, (int)(g() % 300) - 150) * ((g() & 1) ? -1.0 : 1.0));
  }
  for (long long i = 0; i < reps; ++i) {   // ties, near-ties, carries, exact FP32 values
    const uint64_t e = 880 + g() % 290;
    uint64_t m = g() & 0xFFFFFFFFFFFFFull;
    const uint64_t low[5] = {0x10000000ull, 0x0FFFFFFFull, 0x10000001ull, 0x1FFFFFFFull, 0};
    const int k = (int)(g() % 6);
    m = k == 5 ? 0xFFFFFFFFFFFFFull : ((m & ~0x1FFFFFFFull) | low[k]);
    const uint64_t b = ((g() & 1) << 63) | (e << 52) | m;
    double v;
    memcpy(&v, &b, 8);
    chk(v);
  }
  const double special[] = {0.0, -0.0, 1.0, -1.0, INFINITY, -INFINITY, NAN, 3.4028234663852886e38,
                            3.4028235677973366e38, 1.1754943508222875e-38, 1e-45, 5e-324, 1e300, -1e-300};
  for (double v : special) chk(v);
  printf("checked %lld values, %lld mismatches\n", n, bad);
  return bad != 0;
}
