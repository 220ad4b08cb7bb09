// Launches for waveform model 7 (IMRPhenomNSBH, 13 Fisher parameters; FP64 only), and the xi_tide
// table the model interpolates (gwfast/waveforms.py:3286-3373), built on the device once per context.
#define GWF_MODEL 7
#include "gwf_run.cuh"

namespace gwf {

size_t setup_stride_m7() { return rec_stride<7>(); }
size_t core_bytes_m7() { return wave_bytes<7>(); }
cudaError_t launch_fisher_m7(const LaunchArgs& a) { return fisher_dispatch(a); }
cudaError_t launch_snr_m7(const LaunchArgs& a) { return snr_dispatch(a); }
cudaError_t launch_wave_m7(const LaunchArgs& a, const WaveOut& o) { return wave_dispatch(a, o); }

namespace {

// b[0] x^n + ... + b[n]
__device__ __forceinline__ double horner(const double* b, int n, double x) {
  double r = b[0];
  for (int i = 1; i <= n; ++i) r = r * x + b[i];
  return r;
}

// xi_tide at one grid node: arXiv:1509.00512 eq. 8 as a degree-10 polynomial in s = sqrt(xi),
//   s^10 - 3 mu s^8 + 2 chi mu^(3/2) s^7 - 3 q s^4 + 6 q mu s^2 - 3 q mu^2 chi^2,  mu = q C,
// and xi the largest square of its real positive roots (gwfast/waveforms.py:3310-3330 takes them
// from the companion-matrix eigenvalues). Here the real roots are isolated exactly: the real roots
// of each derivative split the positive axis into intervals on which the next polynomial up is
// monotonic, so each interval holds at most one root, found by bisection to the last bit. All roots
// lie below the Fujiwara bound 2 max |a_m|^(1/m) (the last term halved). gwfast counts as real every
// root whose imaginary part is below 1e-5; a complex pair a +- ib with small b makes a local extremum
// of the polynomial at a with |p(a)| ~ |p''(a)| b^2 / 2, so an extremum with |p| <= |p''| 0.5e-10 is
// taken as a (double) root. At spin 1 (the last spin node) the polynomial has an exact double root,
// which numpy's eigenvalues split by ~1e-8 relative; there this table holds the double root itself.
// Every loop is bounded.
__global__ void xitide_table_kernel(double* tab) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)kXiN * kXiN * kXiN) return;
  const int k = (int)(t % kXiN), j = (int)((t / kXiN) % kXiN), i = (int)(t / ((long long)kXiN * kXiN));
  const double C = xi_grid(0, i), q = xi_grid(1, j), chi = xi_grid(2, k);
  const double mu = q * C;
  const double a[11] = {1., 0., -3. * mu, 2. * chi * pow(mu, 1.5), 0., 0., -3. * q, 0., 6. * q * mu, 0.,
                        -3. * q * mu * chi * mu * chi};
  double B = 0.0;
  for (int m = 1; m <= 10; ++m) {
    const double c = fabs(a[m]) * (m == 10 ? 0.5 : 1.0);
    if (c > 0.0) B = fmax(B, pow(c, 1.0 / m));
  }
  B = 2.0 * B + 1e-300;
  double crit[10], cur[10];
  int nc = 0;
  for (int d = 1; d <= 10; ++d) {
    // the (10 - d)-th derivative, degree d
    double b[11];
    for (int m = 0; m <= d; ++m) {
      double c = a[m];
      for (int r = 0; r < 10 - d; ++r) c *= (double)(10 - m - r);
      b[m] = c;
    }
    int nr = 0;
    double lo = 0.0, plo = horner(b, d, lo);
    for (int s = 0; s <= nc; ++s) {
      const double hi = s < nc ? crit[s] : B;
      const double phi = horner(b, d, hi);
      if (plo == 0.0) {
        if (nr < 10 && (nr == 0 || cur[nr - 1] != lo)) cur[nr++] = lo;
      } else if (phi != 0.0 && ((plo < 0.0) != (phi < 0.0)) && hi > lo) {
        double l = lo, h = hi;
        const bool neg_lo = plo < 0.0;
        for (int it = 0; it < 2100; ++it) {
          const double mid = 0.5 * (l + h);
          if (!(mid > l && mid < h)) break;
          const double pm = horner(b, d, mid);
          if (pm == 0.0) { l = h = mid; break; }
          if ((pm < 0.0) == neg_lo) l = mid; else h = mid;
        }
        const double root = fabs(horner(b, d, l)) <= fabs(horner(b, d, h)) ? l : h;
        if (nr < 10) cur[nr++] = root;
      }
      lo = hi;
      plo = phi;
    }
    if (d == 10) {
      double b2[9];
      for (int m = 0; m <= 8; ++m) b2[m] = a[m] * (double)(10 - m) * (double)(9 - m);
      for (int s = 0; s < nc && nr < 10; ++s)
        if (crit[s] > 0.0 && fabs(horner(a, 10, crit[s])) <= 0.5e-10 * fabs(horner(b2, 8, crit[s]))) cur[nr++] = crit[s];
    }
    nc = nr;
    for (int r = 0; r < nr; ++r) crit[r] = cur[r];
  }
  double best = nan("");
  for (int r = 0; r < nc; ++r)
    if (crit[r] > 0.0) best = (best == best) ? fmax(best, crit[r] * crit[r]) : crit[r] * crit[r];
  tab[t] = best;
}

__global__ void xitide_eval_kernel(const double* tab, const double* C, const double* q, const double* chi, long long n,
                                   double* out) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  out[t] = xitide_interp<double>(tab, C[t], q[t], chi[t]);
}

}  // namespace

cudaError_t launch_xitide_table(double* tab, cudaStream_t st) {
  const long long n = (long long)kXiN * kXiN * kXiN;
  xitide_table_kernel<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(tab);
  return cudaGetLastError();
}

cudaError_t launch_xitide_eval(const double* tab, const double* C, const double* q, const double* chi, long long n,
                               double* out, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  xitide_eval_kernel<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(tab, C, q, chi, n, out);
  return cudaGetLastError();
}

}  // namespace gwf
