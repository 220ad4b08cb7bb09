// FP32 split-precision Fisher kernel for the 22-mode models (TaylorF2, IMRPhenomD).
//
// Precision split:
//  - per event, everything parameter-dependent is evaluated in FP64 duals (the same set-up
//    as the FP64 kernel) and rounded once into an FP32 copy, with the amplitude prefactor
//    divided out so that the FP32 values are O(1);
//  - per frequency point, the waveform tangent, projection and derivative vectors run in
//    FP32 (Dual<float, 4>);
//  - Earth-rotation angles are formed as FP64 per-event reference angle + small FP32 offset
//    by angle addition, so no large FP32 argument is ever reduced;
//  - the PSD is read from an FP32 table normalised by its minimum; the Gram matrix is
//    accumulated in FP32 per 32-point tile and across tiles with Kahan compensation, then
//    summed over warps and rescaled (amplitude^2 / PSD scale) in FP64.
// The overall phase factor cancels in every Gram entry and is never formed (as in FP64).
#pragma once
#include "gwf_kernels.cuh"

namespace gwf {

struct cf { float re, im; };
__device__ __forceinline__ cf fadd(cf a, cf b) { return {a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ cf fscale(cf a, float s) { return {a.re * s, a.im * s}; }
__device__ __forceinline__ cf fmuli(cf a) { return {-a.im, a.re}; }

struct ProjF {
  float c2p, s2p, cp, ci, dcp, dci;
  float KA1[3], KA2[2], KB1[2], KB2[2];
  float dKA1[3], dKA2[2], dKB1[2], dKB2[2];
  float s2g[2], c2g[2];
  float Rc, cdcl, sdsl, sdcl, cdsl;
  float sU0, cU0;   // sin, cos of (lon - ra + 2 pi tcoal), formed in FP64
  float idL, sz;
};

struct TimeF { float D, D_th, D_ph, D_t, sx, cx; };
struct ArmF { float Fp, Fc, Fp_x, Fc_x, Fp_d, Fc_d, Fp_s, Fc_s; };
struct GridF { float lnfmin, delta, fac_w, w0, wl, fmin, fcut, df; int R; };

__device__ inline void projf_setup(ProjF& q, const ProjEv& p, double sz) {
  q.c2p = (float)p.c2p; q.s2p = (float)p.s2p; q.cp = (float)p.cp; q.ci = (float)p.ci;
  q.dcp = (float)p.dcp; q.dci = (float)p.dci;
  for (int i = 0; i < 3; ++i) { q.KA1[i] = (float)p.KA1[i]; q.dKA1[i] = (float)p.dKA1[i]; }
  for (int i = 0; i < 2; ++i) {
    q.KA2[i] = (float)p.KA2[i]; q.dKA2[i] = (float)p.dKA2[i];
    q.KB1[i] = (float)p.KB1[i]; q.dKB1[i] = (float)p.dKB1[i];
    q.KB2[i] = (float)p.KB2[i]; q.dKB2[i] = (float)p.dKB2[i];
    q.s2g[i] = (float)p.s2g[i]; q.c2g[i] = (float)p.c2g[i];
  }
  q.Rc = (float)p.Rc; q.cdcl = (float)p.cdcl; q.sdsl = (float)p.sdsl; q.sdcl = (float)p.sdcl; q.cdsl = (float)p.cdsl;
  double s, c;
  sincos(p.u0 + kTwoPi * p.tc, &s, &c);
  q.sU0 = (float)s; q.cU0 = (float)c;
  q.idL = (float)(1.0 / p.dL);
  q.sz = (float)sz;
}

// delay and sin/cos x at t_noloc = tcoal + delta (days); x = ra - lon - 2 pi t (gwfast/signal.py:401-423)
__device__ __forceinline__ void time_f(const ProjF& q, float delta, TimeF& ts) {
  float sd, cd;
  sincosf(6.2831853071795865f * delta, &sd, &cd);
  const float su = q.sU0 * cd + q.cU0 * sd, cu = q.cU0 * cd - q.sU0 * sd;
  ts.D = -q.Rc * (q.cdcl * cu + q.sdsl);
  ts.D_th = q.Rc * (q.cdsl - q.sdcl * cu);
  ts.D_ph = -q.Rc * q.cdcl * su;
  ts.D_t = 6.2831853071795865f * q.Rc * q.cdcl * su;
  float se, ce;
  sincosf(6.2831853071795865f * ts.D * (1.0f / 86400.0f), &se, &ce);
  ts.sx = -(su * ce + cu * se);
  ts.cx = cu * ce - su * se;
}

__device__ __forceinline__ void arm_f(const ProjF& q, const TimeF& ts, int arm, ArmF& ap) {
  const float sx = ts.sx, cx = ts.cx;
  const float s2x = 2.0f * sx * cx, c2x = cx * cx - sx * sx;
  const float A1 = q.KA1[0] * c2x + q.KA1[1] * cx + q.KA1[2];
  const float A2 = q.KA2[0] * s2x + q.KA2[1] * sx;
  const float B1 = q.KB1[0] * c2x + q.KB1[1] * cx;
  const float B2 = q.KB2[0] * s2x + q.KB2[1] * sx;
  const float A1x = -2.0f * q.KA1[0] * s2x - q.KA1[1] * sx;
  const float A2x = 2.0f * q.KA2[0] * c2x + q.KA2[1] * cx;
  const float B1x = -2.0f * q.KB1[0] * s2x - q.KB1[1] * sx;
  const float B2x = 2.0f * q.KB2[0] * c2x + q.KB2[1] * cx;
  const float A1d = q.dKA1[0] * c2x + q.dKA1[1] * cx + q.dKA1[2];
  const float A2d = q.dKA2[0] * s2x + q.dKA2[1] * sx;
  const float B1d = q.dKB1[0] * c2x + q.dKB1[1] * cx;
  const float B2d = q.dKB2[0] * s2x + q.dKB2[1] * sx;
  const float s2g = q.s2g[arm], c2g = q.c2g[arm];
  const float a = s2g * A1 + c2g * A2, b = c2g * B1 + s2g * B2;
  const float ax = s2g * A1x + c2g * A2x, bx = c2g * B1x + s2g * B2x;
  const float ad = s2g * A1d + c2g * A2d, bd = c2g * B1d + s2g * B2d;
  const float c2p = q.c2p, s2p = q.s2p, sz = q.sz;
  ap.Fp = sz * (a * c2p + b * s2p);     ap.Fc = sz * (b * c2p - a * s2p);
  ap.Fp_x = sz * (ax * c2p + bx * s2p); ap.Fc_x = sz * (bx * c2p - ax * s2p);
  ap.Fp_d = sz * (ad * c2p + bd * s2p); ap.Fc_d = sz * (bd * c2p - ad * s2p);
  ap.Fp_s = 2.0f * sz * (b * c2p - a * s2p); ap.Fc_s = 2.0f * sz * (-b * s2p - a * c2p);
}

// same algebra as arm_derivs (FP64) in FP32
__device__ __forceinline__ void arm_derivs_f(const ProjF& q, const ArmF& ap, const TimeF& ts, float f, cf P, cf C,
                                             const cf* dP, const cf* dC, cf dPi, cf dCi, const float* dtn, cf* out) {
  const float tp = 6.2831853071795865f;
  const cf hp = P, hc = fmuli(C);
  const cf H = fadd(fscale(hp, ap.Fp), fscale(hc, ap.Fc));
  const cf iH = fmuli(H);
  const float tpf = tp * f;
  const float G = 1.0f + ts.D_t * (1.0f / 86400.0f);
  const float x_th = -tp * ts.D_th * (1.0f / 86400.0f);
  const float x_ph = 1.0f - tp * ts.D_ph * (1.0f / 86400.0f);
  const float x_tc = -tp * G;
  const cf hx = fadd(fscale(hp, ap.Fp_x), fscale(hc, ap.Fc_x));
  const cf hd = fadd(fscale(hp, ap.Fp_d), fscale(hc, ap.Fc_d));
  const int map[4] = {I_MC, I_ETA, I_C1, I_C2};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    cf v = fadd(fscale(fmuli(dC[k]), ap.Fc), fscale(dP[k], ap.Fp));
    v = fadd(v, fscale(hx, -tp * G * dtn[k]));
    v = fadd(v, fscale(iH, tpf * ts.D_t * dtn[k]));
    out[map[k]] = v;
  }
  out[I_IO] = fadd(fscale(dPi, ap.Fp), fscale(fmuli(dCi), ap.Fc));
  out[I_DL] = fscale(H, -q.idL);
  out[I_TH] = fadd(fadd(fscale(hx, x_th), fscale(hd, -1.0f)), fscale(iH, tpf * ts.D_th));
  out[I_PH] = fadd(fscale(hx, x_ph), fscale(iH, tpf * ts.D_ph));
  out[I_PS] = fadd(fscale(hp, ap.Fp_s), fscale(hc, ap.Fc_s));
  out[I_TC] = fadd(fscale(hx, x_tc * (1.0f / 86400.0f)), fscale(iH, tpf * G));
  out[I_PC] = fscale(iH, -1.0f);
}

// np.interp on the FP32 table normalised by its minimum; outside the table the reference PSD of 1
// gives weights ~1e-46 of in-band ones, represented here as exactly zero.
__device__ __forceinline__ float psd_at_f(const DetDev& d, float f, float lnf) {
  const float* xf = d.psd_f32;
  const int n = d.npsd;
  if (!(f >= xf[0]) || f > xf[n - 1]) return INFINITY;
  int b = (int)((lnf - (float)d.acc_l0) * (float)d.acc_idl);
  b = b < 0 ? 0 : (b >= d.nacc ? d.nacc - 1 : b);
  int j = d.acc[b];
  while (j > 0 && xf[j] > f) --j;
  while (j < n - 2 && xf[j + 1] <= f) ++j;
  const float x0 = xf[j], x1 = xf[j + 1];
  const float y0 = d.psd_s32[j], y1 = d.psd_s32[j + 1];
  return y0 + (f - x0) * ((y1 - y0) / (x1 - x0));
}

union EvUnionF {
  TF2EvT<DF4> tf2;
  PhdCoreT<DF4> phd;
};

// round a struct of FP64 duals to its FP32 twin, all threads of the block; the dual at `amp_member`
// is divided by `amp` first (so the FP32 amplitude is O(1)); ends with a block barrier
template <class SRC, class DST>
__device__ inline void round_struct_par(const SRC& s, DST& d, const D4* amp_member, double amp) {
  static_assert(sizeof(SRC) == 2 * sizeof(DST), "dual structs must hold only duals");
  const double* a = reinterpret_cast<const double*>(&s);
  float* b = reinterpret_cast<float*>(&d);
  const int lo = (int)(reinterpret_cast<const double*>(amp_member) - a);
  const double inv = 1.0 / amp;
  for (int i = threadIdx.x; i < (int)(sizeof(DST) / sizeof(float)); i += blockDim.x)
    b[i] = (float)((i >= lo && i < lo + 5) ? a[i] * inv : a[i]);
  __syncthreads();
}

// 2x3 register blocks covering the upper triangle of the padded 12x12 Gram matrix
static __constant__ unsigned char kBlkR[16] = {0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 3, 3, 4, 4, 5};
static __constant__ unsigned char kBlkC[16] = {0, 1, 2, 3, 0, 1, 2, 3, 1, 2, 3, 2, 3, 2, 3, 3};

template <int MODEL, bool EARTH, int NARM, int NG>
__global__ void __launch_bounds__(kThreads, 4) fisher_kernel_f32(EvBatch ev, DetDev det, const unsigned char* scratch,
                                                                 double* out_arm, double* out_det, int accum) {
  constexpr int NQ = 12;  // padded parameter count
  extern __shared__ __align__(16) unsigned char stage_raw[];
  cf* stage = reinterpret_cast<cf*>(stage_raw);   // [warp][NG][NQ][32]
  __shared__ EvUnion E;
  __shared__ EvUnionF EF;
  __shared__ ProjEv pj;
  __shared__ ProjF pf;
  __shared__ GridEv g;
  __shared__ GridF gf;
  __shared__ ArmF apc[NARM];
  __shared__ TimeF tsc;
  __shared__ double scale;
  const long long n = ev.n0 + blockIdx.x;
  if (n >= ev.N) return;
  block_load<MODEL>(E, pj, g, scratch, blockIdx.x);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // amplitude prefactor divided out before rounding the coefficients to FP32
  const double amp = g.ok ? (MODEL == 0 ? E.tf2.ampK.v : E.phd.k.ampPref.v) : 1.0;
  if (g.ok) {
    if (MODEL == 0) round_struct_par(E.tf2, EF.tf2, &E.tf2.ampK, amp);
    else round_struct_par(E.phd.k, EF.phd, &E.phd.k.ampPref, amp);
  }
  if (tid == 0) {
    scale = amp * amp / det.psd_scale;
    projf_setup(pf, pj, det.sin_zeta);
    gf.lnfmin = (float)g.lnfmin; gf.delta = (float)g.delta; gf.fac_w = (float)g.fac_w; gf.w0 = (float)g.w0;
    gf.wl = (float)g.wl; gf.fmin = (float)g.fmin; gf.fcut = (float)g.fcut; gf.df = (float)g.df; gf.R = g.ok ? g.R : 0;
    if (!EARTH) {
      time_f(pf, 0.0f, tsc);
      for (int a = 0; a < NARM; ++a) arm_f(pf, tsc, a, apc[a]);
    }
  }
  __syncthreads();
  constexpr int NB = 16 * NG;
  constexpr int BPL = (NB + 31) / 32;
  float acc[BPL][6], cmp[BPL][6];
#pragma unroll
  for (int i = 0; i < BPL; ++i)
#pragma unroll
    for (int e = 0; e < 6; ++e) { acc[i][e] = 0.0f; cmp[i][e] = 0.0f; }
  cf* my = stage + (size_t)warp * NG * NQ * 32;
  // zero padding row (parameter 11) once
  for (int gs = 0; gs < NG; ++gs) my[(gs * NQ + 11) * 32 + lane] = {0.0f, 0.0f};
  const int R = gf.R;
  for (int base = 0; base < R; base += kThreads) {
    const int k = base + tid;
    cf D[NARM][NP];
    float sw = 0.0f;
    if (k < R) {
      float f, lnf, w;
      if (ev.spacing == 0) {
        lnf = gf.lnfmin + (float)k * gf.delta;
        if (k == R - 1) { f = gf.fcut; w = f * gf.wl; }
        else if (k == 0) { f = gf.fmin; w = f * gf.w0; }
        else { f = expf(lnf); w = f * gf.fac_w; }
      } else {
        f = (k == R - 1) ? gf.fcut : gf.fmin + (float)k * gf.df;
        lnf = logf(f);
        w = (k == 0 || k == R - 1) ? 0.5f * gf.df : gf.df;
      }
      const float S = psd_at_f(det, f, lnf);
      sw = sqrtf(4.0f * w / S);
      DF4 A, Phi;
      float dtn[4] = {0.f, 0.f, 0.f, 0.f};
      TimeF ts;
      if (MODEL == 0) {
        const float f13 = expf(lnf * (1.0f / 3.0f));
        tf2_point<DF4>(EF.tf2, f, f13, lnf, expf(lnf * (-7.0f / 6.0f)), A, Phi);
        if (EARTH) {
          const DF4 tau = tau_star_point<DF4>(EF.tf2.Ms, EF.tf2.vM, EF.tf2.eta, f13);
#pragma unroll
          for (int q = 0; q < 4; ++q) dtn[q] = -tau.d[q] * (1.0f / 86400.0f);
          time_f(pf, -tau.v * (1.0f / 86400.0f), ts);
        }
      } else {
        phd_point<DF4>(EF.phd, f, A, Phi);
        if (EARTH) {
          const DF4 tau = tau_star_point<DF4>(EF.phd.Ms, EF.phd.vM, EF.phd.eta, expf(lnf * (1.0f / 3.0f)));
#pragma unroll
          for (int q = 0; q < 4; ++q) dtn[q] = -tau.d[q] * (1.0f / 86400.0f);
          time_f(pf, -tau.v * (1.0f / 86400.0f), ts);
        }
      }
      if (!EARTH) ts = tsc;
      const cf P = {pf.cp * A.v, 0.0f}, C = {pf.ci * A.v, 0.0f};
      cf dP[4], dC[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const cf dW = {A.d[q], -A.v * Phi.d[q]};
        dP[q] = fscale(dW, pf.cp);
        dC[q] = fscale(dW, pf.ci);
      }
      const cf dPi = {pf.dcp * A.v, 0.0f}, dCi = {pf.dci * A.v, 0.0f};
#pragma unroll
      for (int a = 0; a < NARM; ++a) {
        ArmF ap;
        if (EARTH) arm_f(pf, ts, a, ap);
        else ap = apc[a];
        arm_derivs_f(pf, ap, ts, f, P, C, dP, dC, dPi, dCi, dtn, D[a]);
      }
    } else {
#pragma unroll
      for (int a = 0; a < NARM; ++a)
#pragma unroll
        for (int q = 0; q < NP; ++q) D[a][q] = {0.0f, 0.0f};
    }
#pragma unroll
    for (int q = 0; q < NP; ++q) {
      if (NG == 1) {
        my[(0 * NQ + q) * 32 + lane] = fscale(D[0][q], sw);
      } else if (NG == 2) {
        const cf u = D[0][q], v = D[1][q];
        my[(0 * NQ + q) * 32 + lane] = fscale(fadd(u, v), sw * 1.2247448713915890f);
        my[(1 * NQ + q) * 32 + lane] = fscale(fadd(u, fscale(v, -1.0f)), sw * 0.70710678118654752f);
      } else {
        const cf u = D[0][q], v = D[1][q];
        my[(0 * NQ + q) * 32 + lane] = fscale(u, sw);
        my[(1 * NQ + q) * 32 + lane] = fscale(v, sw);
        my[(2 * NQ + q) * 32 + lane] = fscale(fadd(u, v), -sw);
      }
    }
    __syncwarp();
#pragma unroll
    for (int i = 0; i < BPL; ++i) {
      const int bl = lane + 32 * i;
      if (bl < NB) {
        const int gs = bl >> 4, bi = bl & 15;
        const int r0 = 2 * kBlkR[bi], c0 = 3 * kBlkC[bi];
        const cf* base_g = my + gs * NQ * 32;
        float s[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll 4
        for (int j = 0; j < 32; ++j) {
          const cf a0 = base_g[(r0 + 0) * 32 + j], a1 = base_g[(r0 + 1) * 32 + j];
          const cf b0 = base_g[(c0 + 0) * 32 + j], b1 = base_g[(c0 + 1) * 32 + j], b2 = base_g[(c0 + 2) * 32 + j];
          s[0] += a0.re * b0.re + a0.im * b0.im;
          s[1] += a0.re * b1.re + a0.im * b1.im;
          s[2] += a0.re * b2.re + a0.im * b2.im;
          s[3] += a1.re * b0.re + a1.im * b0.im;
          s[4] += a1.re * b1.re + a1.im * b1.im;
          s[5] += a1.re * b2.re + a1.im * b2.im;
        }
#pragma unroll
        for (int e = 0; e < 6; ++e) {  // Kahan-compensated accumulation across tiles
          const float y = s[e] - cmp[i][e];
          const float t = acc[i][e] + y;
          cmp[i][e] = (t - acc[i][e]) - y;
          acc[i][e] = t;
        }
      }
    }
    __syncwarp();
  }
  // cross-warp reduction in FP64
  __syncthreads();
  double* red = reinterpret_cast<double*>(stage_raw);  // [kWarps][NG][NQ][NQ]
  for (int i = tid; i < kWarps * NG * NQ * NQ; i += kThreads) red[i] = 0.0;
  __syncthreads();
#pragma unroll
  for (int i = 0; i < BPL; ++i) {
    const int bl = lane + 32 * i;
    if (bl < NB) {
      const int gs = bl >> 4, bi = bl & 15;
      const int r0 = 2 * kBlkR[bi], c0 = 3 * kBlkC[bi];
      double* o = red + ((size_t)(warp * NG + gs) * NQ) * NQ;
#pragma unroll
      for (int e = 0; e < 6; ++e) o[(r0 + e / 3) * NQ + c0 + e % 3] = (double)acc[i][e] - (double)cmp[i][e];
    }
  }
  __syncthreads();
  const long long N = ev.N;
  const double sc = scale;
  for (int e = tid; e < NE; e += kThreads) {
    const int a = kPairA[e], b = kPairB[e];
    double sdet = 0.0;
#pragma unroll
    for (int gs = 0; gs < NG; ++gs) {
      double v = 0.0;
#pragma unroll
      for (int w = 0; w < kWarps; ++w) v += red[((size_t)(w * NG + gs) * NQ + a) * NQ + b];
      v *= sc;
      sdet += v;
      if (out_arm && (NG == 1 || NG == 3)) {
        double* o = out_arm + ((size_t)gs * N + n) * (NP * NP);
        o[a * NP + b] = v;
        o[b * NP + a] = v;
      }
    }
    if (out_det) {
      double* o = out_det + (size_t)n * (NP * NP);
      if (accum) { o[a * NP + b] += sdet; if (a != b) o[b * NP + a] += sdet; }
      else { o[a * NP + b] = sdet; o[b * NP + a] = sdet; }
    }
  }
}

}  // namespace gwf
