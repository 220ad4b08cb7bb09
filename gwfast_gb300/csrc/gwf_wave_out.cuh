// Strain and strain tangent written out on the event grids, and the overlap integrals of two
// waveforms. Same per-event set-up records and per-point code as the Fisher kernels; the common
// phase factor that the Fisher kernels leave out (it cancels in Re(conj(a) b)) is restored:
//   h = (F+ hp + Fx hc) e^{i Psi},  Psi = 2 pi f (tcoal + Delta t_loc) - Phi_c - Phi(f)
// (gwfast/signal.py:485-655; IMRPhenomHM: the mode phases are inside hp, hc and Phi(f) = 0).
#pragma once
#include "gwf_kernels.cuh"

namespace gwf {

enum { WAVE_DERIVS = 0, WAVE_STORE = 1, WAVE_OVERLAP = 2, WAVE_STRAIN = 3 };

// One launch of wave_out_kernel over events [n0, n0 + cnt) of the batch.
//  WAVE_DERIVS:  out[((arm * P + p) * out_n + n - out_base) * R_out + k] = d h_arm / d theta_p at
//                point k (tcoal in seconds; triangle: 3 arms, the third minus the sum of the first
//                two; P = the model's parameter count), the layout of gwfast's return_derivatives per arm
//                (signal.py:938-939).
//  WAVE_STORE:   out[(arm * out_n + n - out_base) * R_out + k] = h_arm sqrt(4 w_k / S_k), computed
//                arms only (1 or 2).
//  WAVE_OVERLAP: reads the WAVE_STORE output of the first waveform at the same place and writes,
//                summed over the arms (triangle: 3), ov[n] = sum Re(u1 conj u2), n1[n] = sum |u1|^2,
//                n2[n] = sum |u2|^2: the trapezoid integrals 4 int Re(h1 conj h2) / S df etc.
//  WAVE_STRAIN:  at the caller's frequencies f_in[(n - out_base) * f_ld + k] (f_ld = 0: one row
//                for every event) instead of the event grid (gwfast/signal.py:425-655):
//                out[(arm * out_n + n - out_base) * R_out + k] = h_arm (GWstrain), amp[same index]
//                = (A+, Ax) (GWAmplitudes), phase[(j * out_n + n - out_base) * R_out + k] with
//                j = 0: GWPhase = 2 pi f tcoal - Phicoal - Phi(f), j = 1: the strain's phase Psi =
//                GWPhase + 2 pi f Delta t_loc (the detector's delay, for the first arm's site; the
//                22-mode models). Each output may be null; triangle: 3 arms, the third minus the
//                sum of the first two.
struct WaveOut {
  int mode;
  double dphi;   // added to the phase constant (TaylorF2 with phiref_vlso: -pi)
  long long n0, cnt;
  cd* out;
  long long out_n, out_base;
  int R_out;
  double* ov;
  double* n1;
  double* n2;
  const double* f_in = nullptr;
  long long f_ld = 0;
  cd* amp = nullptr;
  double* phase = nullptr;
};

// e^{i Psi} with Psi = 2 pi f (tc [days] + D [s]) - phi: the large tc term (up to ~1e9 rad) is
// rotated separately, so that two waveforms with the same tcoal on the same grid share its
// rounding exactly and their relative phase keeps full precision
__device__ __forceinline__ cd common_phase(double f, double tc, double D, double phi) {
  const double tpf = kTwoPi * f;
  double s1, c1, s2, c2;
  sincos(tpf * (tc * kDay), &s1, &c1);
  sincos(tpf * D - phi, &s2, &c2);
  return cmul(cd{c1, s1}, cd{c2, s2});
}

template <int MODEL, bool EARTH, int NARM>
__global__ void __launch_bounds__(kThreads) wave_out_kernel(EvBatch ev, DetDev det, const unsigned char* scratch,
                                                            WaveOut o) {
  __shared__ EvUnion E;
  __shared__ ProjEv pj;
  __shared__ GridEv g;
  __shared__ ArmPat apc[NARM];
  __shared__ TimeState tsc;
  __shared__ double red[kWarps][3];
  const long long n = ev.n0 + blockIdx.x;
  if (n >= ev.N) return;
  block_load<MODEL>(E, pj, g, scratch, blockIdx.x);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (!EARTH) {
    if (tid == 0) {
      time_state(pj, pj.tc, tsc);
      for (int a = 0; a < NARM; ++a) arm_pattern(pj, det.sin_zeta, tsc.x, a, apc[a]);
    }
    __syncthreads();
  }
  constexpr int NA = NARM == 2 ? 3 : 1;
  constexpr int NPM = np_of<MODEL>();
  constexpr int NI = ndir_of<MODEL>();
  const double phic = ev.p[8 * ev.ld + n];
  const int R = g.ok ? g.R : 0;
  const long long row = n - o.out_base;
  double s[3] = {0.0, 0.0, 0.0};
  for (int k = tid; k < o.R_out; k += kThreads) {
    if (o.mode == WAVE_STRAIN) {
      cd hs[NA], am[NA];
      double gph = 0.0, psi = 0.0;
      if (g.ok) {
        const double f = o.f_in[(o.f_ld > 0 ? row * o.f_ld : 0) + k];
        cd P, C;
        double phi0, tau = 0.0;
        wave_point_full<MODEL, EARTH>(E, pj, f, log(f), P, C, phi0, tau);
        TimeState ts;
        if (EARTH) time_state(pj, pj.tc - tau / kDay, ts);
        else ts = tsc;
        const double ph_c = phic + phi0 + o.dphi;
        const cd ph = common_phase(f, pj.tc, ts.D, ph_c);
        gph = kTwoPi * f * (pj.tc * kDay) - ph_c;
        psi = gph + kTwoPi * f * ts.D;
        // amplitudes: A (1 + cos^2 i) / 2 F+ and A cos i Fx for the 22-mode models (P, C real),
        // |h+| F+ and |hx| Fx for IMRPhenomHM (gwfast/signal.py:457-463)
        const double ap = MODEL == 2 ? sqrt(P.re * P.re + P.im * P.im) : P.re;
        const double ac = MODEL == 2 ? sqrt(C.re * C.re + C.im * C.im) : C.re;
#pragma unroll
        for (int a = 0; a < NARM; ++a) {
          ArmPat apt;
          if (EARTH) arm_pattern(pj, det.sin_zeta, ts.x, a, apt);
          else apt = apc[a];
          hs[a] = cmul(cadd(cscale(P, apt.Fp), cscale(cmuli(C), apt.Fc)), ph);
          am[a] = {ap * apt.Fp, ac * apt.Fc};
        }
        if (NA == 3) {
          hs[NA - 1] = cscale(cadd(hs[0], hs[NARM - 1]), -1.0);
          am[NA - 1] = cscale(cadd(am[0], am[NARM - 1]), -1.0);
        }
      } else {
#pragma unroll
        for (int a = 0; a < NA; ++a) hs[a] = am[a] = {0.0, 0.0};
      }
#pragma unroll
      for (int a = 0; a < NA; ++a) {
        const long long ix = ((long long)a * o.out_n + row) * o.R_out + k;
        if (o.out) o.out[ix] = hs[a];
        if (o.amp) o.amp[ix] = am[a];
      }
      if (o.phase) {
        o.phase[row * o.R_out + k] = gph;
        o.phase[(o.out_n + row) * o.R_out + k] = psi;
      }
      continue;
    }
    if (k >= R) {   // no valid grid for this event: zeros
      if (o.mode == WAVE_DERIVS)
        for (int a = 0; a < NA; ++a)
          for (int p = 0; p < NPM; ++p) o.out[((long long)(a * NPM + p) * o.out_n + row) * o.R_out + k] = {0.0, 0.0};
      else if (o.mode == WAVE_STORE)
        for (int a = 0; a < NARM; ++a) o.out[((long long)a * o.out_n + row) * o.R_out + k] = {0.0, 0.0};
      continue;
    }
    double f, lnf, w;
    grid_point(g, ev.spacing, k, f, lnf, w);
    if (o.mode == WAVE_DERIVS) {
      cd P, C, dP[NI], dC[NI], dPi, dCi;
      DualOf<MODEL> tau(0.0);
      double phi0;
      wave_point_dual<MODEL, EARTH>(E, pj, f, lnf, P, C, dP, dC, dPi, dCi, tau, phi0);
      double dtn[NI];
#pragma unroll
      for (int q = 0; q < NI; ++q) dtn[q] = 0.0;
      double dphl, dphd, dphe;
      analytic_tangents<MODEL>(E, lnf, dphl, dphd, dphe);
      TimeState ts;
      if (EARTH) {
#pragma unroll
        for (int q = 0; q < NI; ++q) dtn[q] = -tau.d[q] / kDay;
        time_state(pj, pj.tc - tau.v / kDay, ts);
      } else {
        ts = tsc;
      }
      const cd ph = common_phase(f, pj.tc, ts.D, phic + phi0 + o.dphi);
      cd D[NARM][NPM];
#pragma unroll
      for (int a = 0; a < NARM; ++a) {
        ArmPat ap;
        if (EARTH) arm_pattern(pj, det.sin_zeta, ts.x, a, ap);
        else ap = apc[a];
        arm_derivs<NI>(pj, ap, ts, f, P, C, dP, dC, dPi, dCi, dtn, D[a]);
        analytic_columns<MODEL>(cadd(cscale(P, ap.Fp), cscale(cmuli(C), ap.Fc)), dphl, dphd, dphe, D[a]);
      }
#pragma unroll
      for (int a = 0; a < NA; ++a)
#pragma unroll
        for (int p = 0; p < NPM; ++p) {
          const cd v = a < NARM ? D[a][p] : cscale(cadd(D[0][p], D[NARM - 1][p]), -1.0);
          o.out[((long long)(a * NPM + p) * o.out_n + row) * o.R_out + k] = cmul(v, ph);
        }
    } else {
      cd P, C;
      double phi0, tau = 0.0;
      wave_point_full<MODEL, EARTH>(E, pj, f, lnf, P, C, phi0, tau);
      TimeState ts;
      if (EARTH) time_state(pj, pj.tc - tau / kDay, ts);
      else ts = tsc;
      const double sw = sqrt(4.0 * w / psd_at(det, f, lnf));
      const cd ph = cscale(common_phase(f, pj.tc, ts.D, phic + phi0 + o.dphi), sw);
      cd u[NARM];
#pragma unroll
      for (int a = 0; a < NARM; ++a) {
        ArmPat ap;
        if (EARTH) arm_pattern(pj, det.sin_zeta, ts.x, a, ap);
        else ap = apc[a];
        u[a] = cmul(cadd(cscale(P, ap.Fp), cscale(cmuli(C), ap.Fc)), ph);
      }
      if (o.mode == WAVE_STORE) {
#pragma unroll
        for (int a = 0; a < NARM; ++a) o.out[((long long)a * o.out_n + row) * o.R_out + k] = u[a];
      } else {
        cd v[NARM];
#pragma unroll
        for (int a = 0; a < NARM; ++a) v[a] = o.out[((long long)a * o.out_n + row) * o.R_out + k];
#pragma unroll
        for (int a = 0; a < NA; ++a) {
          const cd x = a < NARM ? v[a] : cscale(cadd(v[0], v[NARM - 1]), -1.0);
          const cd y = a < NARM ? u[a] : cscale(cadd(u[0], u[NARM - 1]), -1.0);
          s[0] += x.re * y.re + x.im * y.im;
          s[1] += x.re * x.re + x.im * x.im;
          s[2] += y.re * y.re + y.im * y.im;
        }
      }
    }
  }
  if (o.mode != WAVE_OVERLAP) return;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    double v = s[j];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if (lane == 0) red[warp][j] = v;
  }
  __syncthreads();
  if (tid < 3) {
    double v = 0.0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) v += red[w][tid];
    double* dst = tid == 0 ? o.ov : (tid == 1 ? o.n1 : o.n2);
    dst[n] = v;
  }
}

}  // namespace gwf
