// FP32 split-precision Fisher kernel (TaylorF2, IMRPhenomD; IMRPhenomHM with FP64 mode phases).
//
// Precision split:
//  - per event, everything parameter-dependent is evaluated in FP64 duals (the same set-up
//    as the FP64 kernel) and rounded once into an FP32 copy, with the amplitude prefactor
//    divided out so that the FP32 values are O(1);
//  - per frequency point, the waveform tangent, projection and derivative vectors run in
//    FP32 (Dual<float, 4>);
//  - Earth-rotation angles are formed as FP64 per-event reference angle + small FP32 offset
//    by angle addition, so no large FP32 argument is ever reduced;
//  - the PSD is read from an FP32 table normalised by its minimum;
//  - the Gram matrix is accumulated exactly in fixed point: each sqrt(weight)-scaled FP32
//    derivative vector is rounded to an integer of at most 26 bits on a per-column power-of-two
//    scale (the running maximum over the warp's tiles, so the largest values keep all their
//    bits), products are formed as int32 x int32 -> int64 and summed without rounding; a growing
//    column scale shifts the sums that involve it, and the sums move to FP64 every kFlushTiles
//    tiles. Rounding each product or partial sum in FP32 instead
//    adds errors that are not a perturbation of the vectors; with equilibrated condition
//    numbers of 1e8-1e11 (typical for 11-parameter BBH Fishers) that makes the matrix
//    indefinite.
// The overall phase factor cancels in every Gram entry and is never formed (as in FP64).
#pragma once
#include <cstddef>
#include <type_traits>

#include "gwf_kernels.cuh"
#include "gwf_f32conv.cuh"

namespace gwf {

// Complex FP32 values as register pairs: additions and real scalings run as packed FP32x2
// instructions (one instruction for the real and the imaginary part, IEEE round-to-nearest each)
struct __align__(8) cf { float re, im; };
__device__ __forceinline__ float2 f2_of(cf a) { return make_float2(a.re, a.im); }
__device__ __forceinline__ cf cf_of(float2 v) { return {v.x, v.y}; }
__device__ __forceinline__ cf fadd(cf a, cf b) { return cf_of(__fadd2_rn(f2_of(a), f2_of(b))); }
__device__ __forceinline__ cf fscale(cf a, float s) { return cf_of(__fmul2_rn(f2_of(a), make_float2(s, s))); }
// a s + c
__device__ __forceinline__ cf ffma2(cf a, float s, cf c) { return cf_of(__ffma2_rn(f2_of(a), make_float2(s, s), f2_of(c))); }
__device__ __forceinline__ cf fmuli(cf a) { return {-a.im, a.re}; }

struct ProjF {
  float c2p, s2p, cp, ci, dcp, dci;
  float KA1[3], KA2[2], KB1[2], KB2[2];
  float dKA1[3], dKA2[2], dKB1[2], dKB2[2];
  float s2g[2], c2g[2];
  float Rc, cdcl, sdsl, sdcl, cdsl;
  float sU0, cU0;   // sin, cos of (lon - ra + 2 pi tcoal), formed in FP64
  float idL, sz;
  float dcs, sgn;   // (1 - |cos i|)^2 / 2 and the sign of cos i (psi column, see point_f32)
};

struct TimeF { float D, D_th, D_ph, D_t, sx, cx; };
struct ArmF { float Fp, Fc, Fp_x, Fc_x, Fp_d, Fc_d, Fp_s, Fc_s; };
struct GridF { float lnfmin, delta, fac_w, w0, wl, fmin, fcut, df, acc_l0, acc_idl; int R; };

// (the FP32 copies by f32_rn: the same values as casts, off the FP64 pipe)
__device__ inline void projf_setup(ProjF& q, const ProjEv& p, double sz) {
  q.c2p = f32_rn(p.c2p); q.s2p = f32_rn(p.s2p); q.cp = f32_rn(p.cp); q.ci = f32_rn(p.ci);
  q.dcp = f32_rn(p.dcp); q.dci = f32_rn(p.dci);
  for (int i = 0; i < 3; ++i) { q.KA1[i] = f32_rn(p.KA1[i]); q.dKA1[i] = f32_rn(p.dKA1[i]); }
  for (int i = 0; i < 2; ++i) {
    q.KA2[i] = f32_rn(p.KA2[i]); q.dKA2[i] = f32_rn(p.dKA2[i]);
    q.KB1[i] = f32_rn(p.KB1[i]); q.dKB1[i] = f32_rn(p.dKB1[i]);
    q.KB2[i] = f32_rn(p.KB2[i]); q.dKB2[i] = f32_rn(p.dKB2[i]);
    q.s2g[i] = f32_rn(p.s2g[i]); q.c2g[i] = f32_rn(p.c2g[i]);
  }
  q.Rc = f32_rn(p.Rc); q.cdcl = f32_rn(p.cdcl); q.sdsl = f32_rn(p.sdsl); q.sdcl = f32_rn(p.sdcl); q.cdsl = f32_rn(p.cdsl);
  double s, c;
  sincos(p.u0 + kTwoPi * p.tc, &s, &c);
  q.sU0 = (float)s; q.cU0 = (float)c;
  q.idL = (float)(1.0 / p.dL);
  q.sz = (float)sz;
  const double ac = 1.0 - fabs(p.ci);
  q.dcs = (float)(0.5 * ac * ac);
  q.sgn = p.ci >= 0.0 ? 1.0f : -1.0f;
}

// delay and sin/cos x at t_noloc = tcoal + delta (days); x = ra - lon - 2 pi t (gwfast/signal.py:401-423).
// (sd, cd) = sin, cos of the Earth-rotation angle 2 pi delta, which does not depend on the detector.
// The rotation by the delay D (|D| <= R_earth / c = 0.0213 s, an angle below 1.6e-6 rad) is taken as
// sin = angle, cos = 1: in FP32 those are the correctly rounded values of sin and cos of such an angle.
__device__ __forceinline__ void time_f_rot(const ProjF& q, float sd, float cd, TimeF& ts) {
  const float su = q.sU0 * cd + q.cU0 * sd, cu = q.cU0 * cd - q.sU0 * sd;
  ts.D = -q.Rc * (q.cdcl * cu + q.sdsl);
  ts.D_th = q.Rc * (q.cdsl - q.sdcl * cu);
  ts.D_ph = -q.Rc * q.cdcl * su;
  ts.D_t = 6.2831853071795865f * q.Rc * q.cdcl * su;
  const float se = 6.2831853071795865f * ts.D * (1.0f / 86400.0f);
  ts.sx = -(su + cu * se);
  ts.cx = cu - su * se;
}
__device__ __forceinline__ void time_f(const ProjF& q, float delta, TimeF& ts) {
  float sd, cd;
  sincosf(6.2831853071795865f * delta, &sd, &cd);
  time_f_rot(q, sd, cd, ts);
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
  const cf H = ffma2(hp, ap.Fp, fscale(hc, ap.Fc));
  const cf iH = fmuli(H);
  const float tpf = tp * f;
  const float G = 1.0f + ts.D_t * (1.0f / 86400.0f);
  const float x_th = -tp * ts.D_th * (1.0f / 86400.0f);
  const float x_ph = 1.0f - tp * ts.D_ph * (1.0f / 86400.0f);
  const float x_tc = -tp * G;
  const cf hx = ffma2(hp, ap.Fp_x, fscale(hc, ap.Fc_x));
  const cf hd = ffma2(hp, ap.Fp_d, fscale(hc, ap.Fc_d));
  const int map[4] = {I_MC, I_ETA, I_C1, I_C2};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    cf v = ffma2(fmuli(dC[k]), ap.Fc, fscale(dP[k], ap.Fp));
    v = ffma2(hx, -tp * G * dtn[k], v);
    v = ffma2(iH, tpf * ts.D_t * dtn[k], v);
    out[map[k]] = v;
  }
  out[I_IO] = ffma2(dPi, ap.Fp, fscale(fmuli(dCi), ap.Fc));
  out[I_DL] = fscale(H, -q.idL);
  out[I_TH] = ffma2(iH, tpf * ts.D_th, ffma2(hx, x_th, fscale(hd, -1.0f)));
  out[I_PH] = ffma2(hx, x_ph, fscale(iH, tpf * ts.D_ph));
  out[I_PS] = ffma2(hp, ap.Fp_s, fscale(hc, ap.Fc_s));
  out[I_TC] = ffma2(hx, x_tc * (1.0f / 86400.0f), fscale(iH, tpf * G));
  out[I_PC] = fscale(iH, -1.0f);
}

// np.interp on the FP32 table normalised by its minimum; outside the table the reference PSD of 1
// gives weights ~1e-46 of in-band ones, represented here as exactly zero.
__device__ __forceinline__ float psd_at_f(const DetDev& d, float f, float lnf, float acc_l0, float acc_idl) {
  const int n = d.npsd;
  if (!(f >= d.psd_f32_lo) || f > d.psd_f32_hi) return INFINITY;
  int b = (int)((lnf - acc_l0) * acc_idl);
  b = b < 0 ? 0 : (b >= d.nacc ? d.nacc - 1 : b);
  int j = __ldg(d.acc + b);
  // the segment [f_j, f_j+1) holding f (the accelerator's row is at most a step or two off)
  float4 sg = __ldg(d.psd_seg + j);
  while (j > 0 && sg.x > f) sg = __ldg(d.psd_seg + --j);
  while (j < n - 2 && sg.y <= f) sg = __ldg(d.psd_seg + ++j);
  return fmaf(f - sg.x, sg.w, sg.z);
}

union EvUnionF {
  TF2EvT<DF4> tf2;
  PhdCoreT<DF4> phd;
};

// FP32 copy of the phase-tangent basis: each FP64 coefficient derivative as a (hi, lo) float pair
struct PBF {
  float hi[22][4], lo[22][4];   // inspiral 0..12, intermediate 13..16, merger-ringdown 17..21
  float du1[4], du0[4];
  float u1, u0, k4, mg, fmrd;
};

// (the 22 basis duals are read 11 at a time, every load of a batch before any store: see round_struct)
__device__ inline void pbf_fill(const PhaseBasis& src, PBF& b, double alpha) {
  auto tan = [&](const D4& d, int q) { return q == P_CHI1 ? d.d[P_CHI1] - alpha * d.d[P_CHI2] : d.d[q]; };
  static_assert(offsetof(PhaseBasis, itm) == 13 * sizeof(D4) && offsetof(PhaseBasis, mrd) == 17 * sizeof(D4),
                "the basis duals are one array");
  const D4* bas = src.ins;
#pragma unroll 1
  for (int c0 = 0; c0 < 22; c0 += 11) {
    double t[11][4];
#pragma unroll
    for (int k = 0; k < 11; ++k)
#pragma unroll
      for (int q = 0; q < 4; ++q) t[k][q] = bas[c0 + k].d[q];
#pragma unroll
    for (int k = 0; k < 11; ++k)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const double v = q == P_CHI1 ? t[k][P_CHI1] - alpha * t[k][P_CHI2] : t[k][q];
        f32_split(v, b.hi[c0 + k][q], b.lo[c0 + k][q]);
      }
  }
  for (int q = 0; q < 4; ++q) {
    b.du1[q] = (float)tan(src.U1, q);
    b.du0[q] = (float)tan(src.U0, q);
  }
  b.u1 = (float)src.U1.v; b.u0 = (float)src.U0.v; b.k4 = (float)src.mrd[4].v;
  b.mg = (float)src.MG.v; b.fmrd = (float)src.fMRD;
}

// compensated sum of NB basis terms: each product hi * basis is split exactly into p + e (FMA), p
// is added to the running sum with an exact two-sum, and every rounding error goes to the low-order
// sum. The terms cancel strongly (the result can be far smaller than the largest term), so a plain
// FP32 sum would carry an error of an ulp of the largest partial sum. The four tangent directions run
// as two packed FP32x2 pairs (each lane of a pair rounded exactly as the scalar operation).
__device__ __forceinline__ float2 fneg2(float2 a) { return make_float2(-a.x, -a.y); }
template <int NB>
__device__ __forceinline__ void phase_terms(const PBF& b, int off, const float (&bas)[NB], float* sh, float* sl) {
#pragma unroll
  for (int hq = 0; hq < 2; ++hq) {
    float2 h_ = make_float2(0.0f, 0.0f), l_ = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int j = 0; j < NB; ++j) {
      const float2 h = *reinterpret_cast<const float2*>(&b.hi[off + j][2 * hq]);
      const float2 lo = *reinterpret_cast<const float2*>(&b.lo[off + j][2 * hq]);
      const float2 bj = make_float2(bas[j], bas[j]);
      const float2 p = __fmul2_rn(h, bj);
      const float2 e = __ffma2_rn(h, bj, fneg2(p));
      const float2 t = __fadd2_rn(h_, p);
      const float2 bp = __fadd2_rn(t, fneg2(h_));
      const float2 a1 = __fadd2_rn(h_, fneg2(__fadd2_rn(t, fneg2(bp))));
      const float2 a2 = __fadd2_rn(p, fneg2(bp));
      l_ = __fadd2_rn(l_, __fadd2_rn(__fadd2_rn(a1, a2), e));
      h_ = t;
      l_ = __ffma2_rn(lo, bj, l_);
    }
    sh[2 * hq] = h_.x;
    sh[2 * hq + 1] = h_.y;
    sl[2 * hq] = l_.x;
    sl[2 * hq + 1] = l_.y;
  }
}

// d Phi / d(Mc, eta, chi1z, chi2z) at frequency f from the basis (see PhaseBasis)
__device__ __forceinline__ void phase_tangent_f(const PBF& b, float f, float lnf, float* dphi) {
  const float x = b.mg * f;
  float sh[4], sl[4];
  if (x < (float)kPhiFJoin) {
    const float f13 = cbrtf(f);
    const float i13 = 1.0f / f13;
    const float i23 = i13 * i13;
    const float bas[13] = {i23 * i23 * i13, 1.0f / f, i23, i13, 1.0f, lnf, f13, f13 * lnf, f13 * f13,
                           f, f * f13, f * f13 * f13, f * f};
    phase_terms<13>(b, 0, bas, sh, sl);
  } else if (x < b.fmrd) {
    const float inv = 1.0f / f;
    const float bas[4] = {f, inv * inv * inv, lnf, 1.0f};
    phase_terms<4>(b, 13, bas, sh, sl);
  } else if (x < (float)kMfCut) {
    const float u = b.u1 * f - b.u0;
    const float datn = 1.0f / (1.0f + u * u);
    const float f14 = sqrtf(sqrtf(f));
    const float bas[5] = {1.0f / f, f14 * f14 * f14, f, 1.0f, atanf(u)};
    phase_terms<5>(b, 17, bas, sh, sl);
#pragma unroll
    for (int q = 0; q < 4; ++q) sl[q] = fmaf(b.k4 * datn, fmaf(b.du1[q], f, -b.du0[q]), sl[q]);
  } else {
#pragma unroll
    for (int q = 0; q < 4; ++q) { sh[q] = 0.0f; sl[q] = 0.0f; }
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) dphi[q] = sh[q] + sl[q];
}

// round a struct of FP64 duals to its FP32 twin (one thread); the dual at `amp_member` is divided
// by `amp` first, so the FP32 amplitude is O(1)
// (tangent slots: value, d/dMc, d/deta, d/dchi1, d/dchi2 per dual; the chi1 slot becomes
// d/dchi1 - alpha d/dchi2 before rounding)
template <class SRC, class DST>
__device__ inline void round_struct(const SRC& s, DST& d, const D4* amp_member, double amp, double alpha) {
  static_assert(sizeof(SRC) == 2 * sizeof(DST), "dual structs must hold only duals");
  static_assert(sizeof(D4) == 5 * sizeof(double) && sizeof(SRC) % sizeof(D4) == 0, "dual layout");
  const double* a = reinterpret_cast<const double*>(&s);
  float* b = reinterpret_cast<float*>(&d);
  const int lo = (int)(reinterpret_cast<const double*>(amp_member) - a);
  const double inv = 1.0 / amp;
  // five duals at a time, every load of a batch issued before any of its stores: the two records
  // do not overlap, but the compiler cannot tell, and a plain loop waits for each load in turn
  constexpr int n = (int)(sizeof(DST) / sizeof(float)), B = 25;
#pragma unroll 1
  for (int i0 = 0; i0 < n; i0 += B) {
    double v[B];
#pragma unroll
    for (int k = 0; k < B; ++k)
      if (i0 + k < n) v[k] = a[i0 + k];
#pragma unroll
    for (int k = 0; k < B; ++k) {
      if (i0 + k < n) {
        double x = v[k];
        if (k % 5 == 1 + P_CHI1) x -= alpha * v[k + 1];   // i0 is a multiple of 5: i % 5 == k % 5
        b[i0 + k] = f32_rn(x);
      }
    }
  }
  // the amplitude dual again, divided by amp (a select inside the loop above would have made the
  // compiler multiply every word)
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    double x = a[lo + k];
    if (k == 1 + P_CHI1) x -= alpha * a[lo + k + 1];
    b[lo + k] = f32_rn(x * inv);
  }
}

// tau_star (3.5PN time to coalescence, gwfast/waveforms.py:878-901, :1299-1322) in the FP32 form.
// tau = T0 v^-8 P(v), T0 = (5/256) Ms / eta, v = vM f^(1/3), P(v) = 1 + sum_{k=2..7} a_k v^k with the
// a_k polynomials in eta (a_6 also carries a6l ln(16 v^2)). The parameters enter only through Ms, eta
// and vM, and v's tangent is v d ln vM, so per point
//   d tau = tau d ln T0 + T0 v^-8 [ (v P'(v) - 8 P(v)) d ln vM + (dP/deta)(v) d eta ]:
// three polynomials in v with per-event coefficients (formed once per event in FP64) instead of the
// four-direction dual arithmetic of the eta polynomials at every point; ln(16 v^2) comes from ln f.
struct TauF {
  float T0, lnv0, lg0;   // (5/256) Ms / eta; ln vM; ln 16 + 2 ln vM (ln(16 v^2) = lg0 + 2/3 ln f)
  float a[6], b[6];      // a_2..a_7 (a_6 without its log term) and their eta derivatives
  float dlnT0[4], dlnv[4], deta[4];   // tangents (chi1 slot: d/dchi1 - alpha d/dchi2)
};
constexpr double kTauA6l = 3424.0 / 105.0;

__device__ inline void tau_setup(TauF& t, const D4& Ms, const D4& vM, const D4& eta_, double alpha) {
  const double eta = eta_.v, e2 = eta * eta;
  const double a[6] = {743. / 252. + 11. / 3. * eta, -32. / 5. * kPi,
                       3058673. / 508032. + 5429. / 504. * eta + 617. / 72. * e2,
                       -(7729. / 252. - 13. / 3. * eta) * kPi,
                       -10052469856691. / 23471078400. + 128. / 3. * kPi * kPi + 6848. / 105. * kEulerGamma
                           + (3147553127. / 3048192. - 451. / 12. * kPi * kPi) * eta - 15211. / 1728. * e2
                           + 25565. / 1296. * e2 * eta,
                       (-15419335. / 127008. - 75703. / 756. * eta + 14809. / 378. * e2) * kPi};
  const double b[6] = {11. / 3., 0.0, 5429. / 504. + 2. * 617. / 72. * eta, 13. / 3. * kPi,
                       3147553127. / 3048192. - 451. / 12. * kPi * kPi - 2. * 15211. / 1728. * eta
                           + 3. * 25565. / 1296. * e2,
                       (-75703. / 756. + 2. * 14809. / 378. * eta) * kPi};
  for (int k = 0; k < 6; ++k) { t.a[k] = (float)a[k]; t.b[k] = (float)b[k]; }
  t.T0 = (float)(5.0 / 256.0 * Ms.v / eta);
  const double lnv0 = log(vM.v);
  t.lnv0 = (float)lnv0;
  t.lg0 = (float)(log(16.0) + 2.0 * lnv0);
  auto tan = [&](const D4& d, int q) { return q == P_CHI1 ? d.d[P_CHI1] - alpha * d.d[P_CHI2] : d.d[q]; };
  const double ims = 1.0 / Ms.v, ieta = 1.0 / eta, ivm = 1.0 / vM.v;
  for (int q = 0; q < 4; ++q) {
    t.dlnT0[q] = (float)(tan(Ms, q) * ims - tan(eta_, q) * ieta);
    t.dlnv[q] = (float)(tan(vM, q) * ivm);
    t.deta[q] = (float)tan(eta_, q);
  }
}

// tau_star (s) and its tangent at ln f
__device__ __forceinline__ void tau_point_f32(const TauF& t, float lnf, float& tau, float (&dtau)[4]) {
  const float lnv = fmaf(lnf, 1.0f / 3.0f, t.lnv0);
  const float v = expf(lnv), iv8 = expf(-8.0f * lnv);
  const float lg = fmaf(lnf, 2.0f / 3.0f, t.lg0);
  const float a6e = fmaf((float)kTauA6l, lg, t.a[4]);
  // P / v^2 - 1 / v^2, v P' / v^2, (dP/deta) / v^2 by Horner from v^5 down
  float p = t.a[5], dp = 7.0f * t.a[5], q = t.b[5];
  p = fmaf(p, v, a6e);  dp = fmaf(dp, v, fmaf(6.0f, a6e, 2.0f * (float)kTauA6l));  q = fmaf(q, v, t.b[4]);
  p = fmaf(p, v, t.a[3]);  dp = fmaf(dp, v, 5.0f * t.a[3]);  q = fmaf(q, v, t.b[3]);
  p = fmaf(p, v, t.a[2]);  dp = fmaf(dp, v, 4.0f * t.a[2]);  q = fmaf(q, v, t.b[2]);
  p = fmaf(p, v, t.a[1]);  dp = fmaf(dp, v, 3.0f * t.a[1]);  q = fmaf(q, v, t.b[1]);
  p = fmaf(p, v, t.a[0]);  dp = fmaf(dp, v, 2.0f * t.a[0]);  q = fmaf(q, v, t.b[0]);
  const float v2 = v * v;
  const float P = fmaf(p, v2, 1.0f);
  const float c = t.T0 * iv8;
  tau = c * P;
  const float gv = c * fmaf(dp, v2, -8.0f * P), ge = c * q * v2;
#pragma unroll
  for (int k = 0; k < 4; ++k) dtau[k] = fmaf(tau, t.dlnT0[k], fmaf(gv, t.dlnv[k], ge * t.deta[k]));
}

// IMRPhenomD amplitude in the FP32 form (gwfast/waveforms.py:1155-1254). In the inspiral region
// A = ampPref x^(-7/6) S(x), S = 1 + sum_k c_k x^(k/3) (k = 2..9; c_k = a23, a1, a43, a53, a2, r1, r2, r3),
// x = MG f with tangent x d ln MG, so
//   d ln A = d ln ampPref + (-7/6 + x S'(x) / S) d ln MG + (sum_k d c_k x^(k/3)) / S:
// the basis powers once, then scalar sums, instead of dual products of every term. Elsewhere the dual
// evaluation of complete_amp_shape.
__device__ __forceinline__ DF4 phd_amp_f32(const PhdCoreT<DF4>& k, float f) {
  const float xv = k.MG.v * f;
  if (!(xv < (float)kAmpFJoin)) return phd_amp_point<DF4>(k, f);
  const float x13 = cbrtf(xv), x23 = x13 * x13, x2 = xv * xv;
  const float bas[8] = {x23, xv, xv * x13, xv * x23, x2, x2 * x13, x2 * x23, x2 * xv};
  const DF4* c[8] = {&k.a23, &k.a1, &k.a43, &k.a53, &k.a2, &k.r1, &k.r2, &k.r3};
  float S = 1.0f, xS = 0.0f, T[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float cb = c[j]->v * bas[j];
    S += cb;
    xS = fmaf((float)(j + 2) * (1.0f / 3.0f), cb, xS);
#pragma unroll
    for (int q = 0; q < 4; ++q) T[q] = fmaf(c[j]->d[q], bas[j], T[q]);
  }
  const float xm76 = 1.0f / (xv * sqrtf(x13));
  const float iP = 1.0f / k.ampPref.v, iS = 1.0f / S;
  DF4 A;
  A.v = k.ampPref.v * xm76 * S;
  const float gx = -7.0f / 6.0f + xS * iS, iMG = 1.0f / k.MG.v;
#pragma unroll
  for (int q = 0; q < 4; ++q)
    A.d[q] = A.v * (k.ampPref.d[q] * iP + gx * k.MG.d[q] * iMG + T[q] * iS);
  return A;
}

// The detector-independent part of one frequency point: hp = P, hc = i C without the common phase,
// their tangents in (Mc, eta, chi1z, chi2z), the iota derivatives, Q = P - s C (s = sign cos iota, see
// project_f32) and, with Earth rotation, tau_star and its tangent. The amplitude prefactor is
// divided out (restored with the Gram scale).
struct WaveF {
  cf P, C, dP[4], dC[4], dPi, dCi, Q;
  float tau;      // tau_star (s)
  float dtn[4];   // d t_noloc / d theta_k (days)
};

// The 22-mode waveform at one point in compact form: amplitude A, the tangent dW = dA - i A dPhi of
// W = A e^{-i Phi} (common phase dropped) and the time to coalescence. The strain's polarisations are
// W times per-event constants (hp = cp W, hx = i ci W): the single-detector kernels project this form
// directly (arm_derivs_22), the detector groups expand it per detector (expand22).
struct Wave22 {
  float A;
  cf dW[4];
  float tau;      // tau_star (s)
  float dtn[4];   // d t_noloc / d theta_k (days)
};

template <int MODEL, bool EARTH>
__device__ __forceinline__ void wave22_f32(const EvUnionF& EF, const PBF& pbf, const TauF& tf, float f, float lnf,
                                           Wave22& w) {
  DF4 A;
  float dphi[4];
  phase_tangent_f(pbf, f, lnf, dphi);
  w.tau = 0.0f;
#pragma unroll
  for (int q = 0; q < 4; ++q) w.dtn[q] = 0.0f;
  if (MODEL == 0) {
    const float f13 = cbrtf(f);
    A = EF.tf2.ampK * (1.0f / (f * sqrtf(f13)));
  } else {
    A = phd_amp_f32(EF.phd, f);
  }
  if (EARTH) {
    float dtau[4];
    tau_point_f32(tf, lnf, w.tau, dtau);
#pragma unroll
    for (int q = 0; q < 4; ++q) w.dtn[q] = -dtau[q] * (1.0f / 86400.0f);
  }
  w.A = A.v;
#pragma unroll
  for (int q = 0; q < 4; ++q) w.dW[q] = {A.d[q], -A.v * dphi[q]};
}

// the full polarisations and tangents of the compact waveform with one detector's projection record
// (the detector groups expand per detector: measured faster there than projecting the compact form)
__device__ __forceinline__ void expand22(const Wave22& c, const ProjF& pf, WaveF& w) {
  w.tau = c.tau;
#pragma unroll
  for (int q = 0; q < 4; ++q) w.dtn[q] = c.dtn[q];
  w.P = {pf.cp * c.A, 0.0f};
  w.C = {pf.ci * c.A, 0.0f};
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    w.dP[q] = fscale(c.dW[q], pf.cp);
    w.dC[q] = fscale(c.dW[q], pf.ci);
  }
  w.dPi = {pf.dcp * c.A, 0.0f};
  w.dCi = {pf.dci * c.A, 0.0f};
  w.Q = {c.A * pf.dcs, 0.0f};   // P - s C = A (cp - s ci) = A (1 - |cos i|)^2 / 2
}

// The detector part: derivative vectors d h / d theta of every arm (11 parameters) and the strain.
// The psi slot holds Delta = dh/dpsi - 2 s dh/dPhicoal instead of dh/dpsi: with dh/dpsi =
// 2 (Fx P - i F+ C) and dh/dPhicoal = -i (F+ P + i Fx C), Delta = 2 (P - s C)(Fx + i s F+). Near
// face-on and face-off dh/dpsi is almost exactly 2 s dh/dPhicoal; forming the small difference
// directly keeps its FP32 relative accuracy (the Gram of the original columns is restored in FP64
// at the end).
template <bool EARTH, int NARM>
__device__ __forceinline__ void project_f32_rot(const WaveF& w, const ProjF& pf, const ArmF* apc, const TimeF& tsc,
                                                float f, float sd, float cd, cf (&D)[NARM][NP], cf (&H)[NARM]) {
  TimeF ts;
  if (EARTH) time_f_rot(pf, sd, cd, ts);
  else ts = tsc;
#pragma unroll
  for (int a = 0; a < NARM; ++a) {
    ArmF ap;
    if (EARTH) arm_f(pf, ts, a, ap);
    else ap = apc[a];
    arm_derivs_f(pf, ap, ts, f, w.P, w.C, w.dP, w.dC, w.dPi, w.dCi, w.dtn, D[a]);
    const float wr = ap.Fc, wi = pf.sgn * ap.Fp;
    D[a][I_PS] = {2.0f * (w.Q.re * wr - w.Q.im * wi), 2.0f * (w.Q.re * wi + w.Q.im * wr)};
    H[a] = ffma2(w.P, ap.Fp, fscale(fmuli(w.C), ap.Fc));   // the strain (common phase dropped)
  }
}

// sin and cos of the point's Earth-rotation angle 2 pi delta, delta = -tau_star / day
__device__ __forceinline__ void rot_sc_tau(float tau, float& sd, float& cd) {
  sincosf(6.2831853071795865f * (-tau * (1.0f / 86400.0f)), &sd, &cd);
}
__device__ __forceinline__ void rot_sc(const WaveF& w, float& sd, float& cd) { rot_sc_tau(w.tau, sd, cd); }

template <bool EARTH, int NARM>
__device__ __forceinline__ void project_f32(const WaveF& w, const ProjF& pf, const ArmF* apc, const TimeF& tsc, float f,
                                            cf (&D)[NARM][NP], cf (&H)[NARM]) {
  float sd = 0.0f, cd = 1.0f;
  if (EARTH) rot_sc(w, sd, cd);
  project_f32_rot<EARTH, NARM>(w, pf, apc, tsc, f, sd, cd, D, H);
}

// The 22-mode models' arm vectors straight from the compact waveform: with hp = cp W and hx = i ci W
// (W = A e^{-i Phi}, common phase dropped), hp F+ + hx Fx = A (cp F+, ci Fx) and the intrinsic
// tangents are dW (cp F+ + i ci Fx); the same algebra as arm_derivs_f, without the expanded copies
// of the polarisations and their tangents (ET triangle launch, 10^4 events: 2.272 -> 2.250 ms; the
// detector groups were faster expanding per detector, 2.386 against 2.434 ms).
// H: the arm's strain. The psi slot holds Delta = 2 A (1 - |cos i|)^2 / 2 (Fx + i s F+) (see
// project_f32_rot).
__device__ __forceinline__ void arm_derivs_22(const ProjF& q, const ArmF& ap, const TimeF& ts, float f, const Wave22& w,
                                              cf* out, cf& H) {
  const float tp = 6.2831853071795865f;
  const float cpA = q.cp * w.A, ciA = q.ci * w.A;
  const float Kr = q.cp * ap.Fp, Ki = q.ci * ap.Fc;   // dh = dW (Kr + i Ki)
  H = {cpA * ap.Fp, ciA * ap.Fc};
  const cf iH = fmuli(H);
  const float tpf = tp * f;
  const float G = 1.0f + ts.D_t * (1.0f / 86400.0f);
  const float x_th = -tp * ts.D_th * (1.0f / 86400.0f);
  const float x_ph = 1.0f - tp * ts.D_ph * (1.0f / 86400.0f);
  const float x_tc = -tp * G;
  const cf hx = {cpA * ap.Fp_x, ciA * ap.Fc_x};
  const cf hd = {cpA * ap.Fp_d, ciA * ap.Fc_d};
  const int map[4] = {I_MC, I_ETA, I_C1, I_C2};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    cf v = ffma2(fmuli(w.dW[k]), Ki, fscale(w.dW[k], Kr));
    v = ffma2(hx, -tp * G * w.dtn[k], v);
    v = ffma2(iH, tpf * ts.D_t * w.dtn[k], v);
    out[map[k]] = v;
  }
  out[I_IO] = {q.dcp * w.A * ap.Fp, q.dci * w.A * ap.Fc};
  out[I_DL] = fscale(H, -q.idL);
  out[I_TH] = ffma2(iH, tpf * ts.D_th, ffma2(hx, x_th, fscale(hd, -1.0f)));
  out[I_PH] = ffma2(hx, x_ph, fscale(iH, tpf * ts.D_ph));
  const float qd = 2.0f * w.A * q.dcs;
  out[I_PS] = {qd * ap.Fc, qd * q.sgn * ap.Fp};
  out[I_TC] = ffma2(hx, x_tc * (1.0f / 86400.0f), fscale(iH, tpf * G));
  out[I_PC] = fscale(iH, -1.0f);
}

template <bool EARTH, int NARM>
__device__ __forceinline__ void project22_rot(const Wave22& w, const ProjF& pf, const ArmF* apc, const TimeF& tsc, float f,
                                              float sd, float cd, cf (&D)[NARM][NP], cf (&H)[NARM]) {
  TimeF ts;
  if (EARTH) time_f_rot(pf, sd, cd, ts);
  else ts = tsc;
#pragma unroll
  for (int a = 0; a < NARM; ++a) {
    ArmF ap;
    if (EARTH) arm_f(pf, ts, a, ap);
    else ap = apc[a];
    arm_derivs_22(pf, ap, ts, f, w, D[a], H[a]);
  }
}

template <int MODEL, bool EARTH, int NARM>
__device__ __forceinline__ void point_f32(const EvUnionF& EF, const PBF& pbf, const ProjF& pf, const TauF& tf,
                                          const ArmF* apc, const TimeF& tsc, float f, float lnf, cf (&D)[NARM][NP],
                                          cf (&H)[NARM]) {
  Wave22 w;
  wave22_f32<MODEL, EARTH>(EF, pbf, tf, f, lnf, w);
  float sd = 0.0f, cd = 1.0f;
  if (EARTH) rot_sc_tau(w.tau, sd, cd);
  project22_rot<EARTH, NARM>(w, pf, apc, tsc, f, sd, cd, D, H);
}

// ------------------------------------------------------------------ IMRPhenomHM, split precision
// Per event the model record exists twice: FP64 values (for the mode phases) and FP32 duals (for
// amplitudes and tangents, the amplitude prefactor divided out as for the 22-mode models). Per
// point every mode phase is evaluated in FP64 and reduced modulo 2 pi before it reaches FP32: the
// phases reach 1e4-1e5 rad at low frequency, and their differences between modes set the
// interference in the mode sum, so FP32 could not carry them to the ~1e-7 rad the sum needs.
// Amplitudes, phase tangents, harmonics and the mode sums run in FP32 duals.
struct HMF32 {
  HMEvT<DF4> e32;
  HMEvT<double> e64;
  // per mode: 1 / amp_, 1 / rho and 1 / (fdamp rho tau), so that the FP64 mode phases divide only by
  // the frequency (complete_phase_hm64)
  double inv_amp[6], inv_rho[6], iden[6];
};
struct NoRec {};

// FP64 dual -> FP32 dual, with the chi1 tangent replaced by d/dchi1 - alpha d/dchi2 (see
// setup_f32_kernel) and value and tangents multiplied by scale
__device__ inline DF4 to_df4(const D4& d, double alpha, double scale) {
  DF4 r;
  r.v = f32_rn(d.v * scale);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const double t = q == P_CHI1 ? d.d[P_CHI1] - alpha * d.d[P_CHI2] : d.d[q];
    r.d[q] = f32_rn(t * scale);
  }
  return r;
}

constexpr int kHMModeDuals = 20;   // leading dual members of HMModeT (rho ... hi4)

// src[0..n) -> FP32 duals f32[] and FP64 values f64[], dual `scaled` multiplied by scale; five duals at
// a time, every load of a batch before any store (see round_struct)
__device__ inline void conv_duals(const D4* src, DF4* f32, double* f64, int n, double alpha, int scaled, double scale) {
#pragma unroll 1
  for (int i0 = 0; i0 < n; i0 += 5) {
    D4 t[5];
#pragma unroll
    for (int k = 0; k < 5; ++k)
      if (i0 + k < n) t[k] = src[i0 + k];
#pragma unroll
    for (int k = 0; k < 5; ++k)
      if (i0 + k < n) {
        f32[i0 + k] = to_df4(t[k], alpha, 1.0);
        f64[i0 + k] = t[k].v;
      }
  }
  // the scaled dual again (a select of the scale inside the loop would multiply every word)
  if (scaled >= 0 && scaled < n) f32[scaled] = to_df4(src[scaled], alpha, scale);
}

__device__ inline void hm_round(const HMEv& s, HMF32& d, double amp, double alpha) {
  static_assert(sizeof(PhdCoreT<D4>) % sizeof(D4) == 0, "core holds only duals");
  static_assert(sizeof(PhdCoreT<D4>) / sizeof(D4) == sizeof(PhdCoreT<DF4>) / sizeof(DF4) &&
                sizeof(PhdCoreT<D4>) / sizeof(D4) == sizeof(PhdCoreT<double>) / sizeof(double), "core layouts");
  static_assert(offsetof(HMModeT<D4>, yp) == kHMModeDuals * sizeof(D4) &&
                offsetof(HMModeT<DF4>, yp) >= kHMModeDuals * sizeof(DF4) &&
                offsetof(HMModeT<double>, yp) == kHMModeDuals * sizeof(double), "mode layouts");
  const int n = (int)(sizeof(PhdCoreT<D4>) / sizeof(D4));
  const D4* a = reinterpret_cast<const D4*>(&s.k);
  DF4* b = reinterpret_cast<DF4*>(&d.e32.k);
  double* c = reinterpret_cast<double*>(&d.e64.k);
  const D4* ampm = &s.k.ampPref;
  conv_duals(a, b, c, n, alpha, (int)(ampm - a), 1.0 / amp);
  d.e32.phi0 = to_df4(s.phi0, alpha, 1.0);
  d.e64.phi0 = s.phi0.v;
  for (int m = 0; m < 6; ++m) {
    const HMMode& sm = s.md[m];
    HMModeT<DF4>& fm = d.e32.md[m];
    HMModeT<double>& vm = d.e64.md[m];
    const D4* sa = reinterpret_cast<const D4*>(&sm);
    DF4* fa = reinterpret_cast<DF4*>(&fm);
    double* va = reinterpret_cast<double*>(&vm);
    conv_duals(sa, fa, va, kHMModeDuals, alpha, -1, 1.0);
    fm.yp = vm.yp = sm.yp; fm.yc = vm.yc = sm.yc; fm.dyp = vm.dyp = sm.dyp; fm.dyc = vm.dyc = sm.dyc;
    fm.ysp = vm.ysp = sm.ysp; fm.ysm = vm.ysm = sm.ysm; fm.shift = vm.shift = sm.shift;
    fm.l = vm.l = sm.l; fm.m = vm.m = sm.m;
    d.inv_amp[m] = 1.0 / sm.amp_.v;
    d.inv_rho[m] = 1.0 / sm.rho.v;
    d.iden[m] = 1.0 / (s.k.fdamp.v * sm.rho.v * sm.tau.v);
  }
}

// FP64 inspiral phase of the IMRPhenomD core at x' = x * ai (as ins_phase in gwf_model.cuh), from the
// per-point values cbrt(pi x), 1 / cbrt(pi x), log(pi x) and 1 / (pi x) shared by all modes: the mode
// phases of the inspiral region differ only by the scale ai = 2 / m of their argument, so
// cbrt(pi x ai) = cbrt(pi x) cbrt(ai) and log(pi x ai) = log(pi x) + log(ai), and each mode costs a
// short polynomial instead of its own cube root and logarithm.
struct InsShared { double x13, ix13, lx, ixp; };

// (1 / ai = m / 2 exactly; ieta = 1 / eta, formed once per point: the FP64 pipe sets this kernel's
// speed, and each FP64 division is a dozen of its instructions)
__device__ __forceinline__ double ins_phase_scaled(const PhdCoreT<double>& k, const InsShared& b, double x, int m,
                                                   double ieta) {
  // cbrt(ai), 1 / cbrt(ai), log(ai) for ai = 2 / m, m = 1..4
  constexpr double kCb[5] = {0.0, 1.2599210498948731648, 1.0, 0.87358046473629886905, 0.79370052598409973738};
  constexpr double kICb[5] = {0.0, 0.79370052598409973738, 1.0, 1.1447142425533318678, 1.2599210498948731648};
  constexpr double kLg[5] = {0.0, 0.69314718055994530942, 0.0, -0.40546510810816438198, -0.69314718055994530942};
  const double x13 = b.x13 * kCb[m];
  const double ix13 = b.ix13 * kICb[m];
  const double ix23 = ix13 * ix13;
  const double ixp = b.ixp * (0.5 * m);
  const double lx = (b.lx + kLg[m]) * (1.0 / 3.0);
  const double tf2 = ix23 * ixp + k.pn.c2 * ixp + k.pn.c3 * ix23 + k.pn.c4 * ix13 + k.pn.c5 + k.pn.c5l * lx
                     + (k.pn.c6 + k.pn.c6l * lx) * x13 + k.pn.c7 * x13 * x13;
  const double m13 = x13 * 0.68278406325529573;
  return k.pn.A * tf2 + (k.sig[0] * x + 0.75 * k.sig[1] * x * m13 + 0.6 * k.sig[2] * x * m13 * m13
                         + 0.5 * k.sig[3] * x * x) * ieta;
}

// complete_phase<double> for the FP32 form's mode phases with the event's reciprocals (ieta = 1 / eta,
// iden = 1 / (fdamp rho tau)): the intermediate and merger-ringdown pieces then divide only by x
__device__ __forceinline__ double complete_phase_hm64(const PhdCoreT<double>& k, double x, double C1, double C2,
                                                      double rho, double iden, double ieta) {
  if (x < kPhiFJoin) return ins_phase<double>(k, x);
  if (x < k.fMRD) {
    const double ix = 1.0 / x;
    return (k.bet[0] * x - k.bet[2] * (1.0 / 3.0) * ix * ix * ix + k.bet[1] * log(x)) * ieta + k.C1Int + k.C2Int * x;
  }
  if (x < kMfCut) {
    const double x14 = sqrt(sqrt(x));
    return (-k.alp[1] / x + (4.0 / 3.0) * k.alp[2] * x14 * x14 * x14 + k.alp[0] * x
            + k.alp[3] * rho * atan((x - k.alp[4] * k.fring) * iden)) * ieta + C1 + C2 * x;
  }
  return 0.0;
}

// IMRPhenomHM at one point, FP32 form: the detector-independent part (as wave_f32). Q = P - s C is
// summed over the modes from the harmonic differences yp - s yc formed in FP64, so it keeps FP32
// relative accuracy near face-on and face-off.
template <bool EARTH>
__device__ __forceinline__ void wave_f32_hm(const HMF32& H, const ProjF& pf, const TauF& tf, float f, float lnf, WaveF& w) {
  const HMEvT<DF4>& e = H.e32;
  const HMEvT<double>& v = H.e64;
  const double x64 = v.k.MG * (double)f;
  const DF4 x = e.k.MG * f;
  const double lin64 = v.k.t0 * (x64 - v.k.fRef);
  const DF4 lin = e.k.t0 * (x - e.k.fRef);
  const bool spos = pf.sgn > 0.0f;
  constexpr double kAi[5] = {0.0, 2.0, 1.0, 2.0 / 3.0, 0.5};   // ai = 2 / m
  const double ieta = 1.0 / v.k.eta;
  InsShared ins;
  if (x64 < 2.0 * kPhiFJoin) {   // some mode argument x * 2 / m lies in the inspiral region
    const double xp = kPi * x64;
    ins.x13 = cbrt(xp);
    ins.ix13 = 1.0 / ins.x13;
    ins.lx = log(xp);
    ins.ixp = 1.0 / xp;
  }
  cf P = {0.0f, 0.0f}, C = {0.0f, 0.0f}, dPi = {0.0f, 0.0f}, dCi = {0.0f, 0.0f}, Q = {0.0f, 0.0f};
  cf (&dP)[4] = w.dP;
  cf (&dC)[4] = w.dC;
#pragma unroll
  for (int q = 0; q < 4; ++q) { dP[q] = {0.0f, 0.0f}; dC[q] = {0.0f, 0.0f}; }
#pragma unroll 1
  for (int mode = 0; mode < 6; ++mode) {
    const HMModeT<DF4>& m = e.md[mode];
    const HMModeT<double>& mv = v.md[mode];
    const double ai64 = kAi[mv.m];
    const float ai = 2.0f / (float)m.m;
    // amplitude: frequency map chosen on the FP64 argument, as the FP64 kernel does
    DF4 fs;
    if (x64 < mv.fia) fs = x * ai;
    else if (x64 < mv.frlm) fs = x * m.ama + m.bma;
    else fs = x - m.frlm + e.k.fring;
    DF4 amp = e.k.ampPref * (1.0f / (fs * dsqrt(dcbrt(fs)))) * complete_amp_shape(e.k, fs);
    if (mode != 1) {
      amp = amp * hm_absH(m, mode, x) * hm_absH(m, mode, fs) / hm_absH(m, mode, x * ai);
      if (!(amp.v == amp.v)) amp = DF4(0.0f);   // nan_to_num at equal mass (gwfast/waveforms.py:2582)
    }
    // phase: value in FP64, tangent in FP32
    double ph64;
    DF4 ph;
    if (x64 < mv.fip) {
      const double xa = x64 * ai64;
      ph64 = (xa < kPhiFJoin ? ins_phase_scaled(v.k, ins, xa, mv.m, ieta)
                             : complete_phase_hm64(v.k, xa, mv.C1, mv.C2, mv.rho, H.iden[mode], ieta)) * (0.5 * mv.m);
      ph = complete_phase<DF4>(e.k, x * ai, m.C1, m.C2, m.rho, m.tau) / ai;
    } else if (x64 < mv.frlm) {
      ph64 = mv.PhDBA - mv.PhDB
             + complete_phase_hm64(v.k, x64 * mv.amp_ + mv.bmp, mv.C1, mv.C2, mv.rho, H.iden[mode], ieta) * H.inv_amp[mode];
      ph = m.PhDBA - m.PhDB + complete_phase<DF4>(e.k, x * m.amp_ + m.bmp, m.C1, m.C2, m.rho, m.tau) / m.amp_;
    } else {
      ph64 = mv.phC - mv.PhDC
             + complete_phase_hm64(v.k, x64 * mv.rho, mv.C1, mv.C2, mv.rho, H.iden[mode], ieta) * H.inv_rho[mode];
      ph = m.phC - m.PhDC + complete_phase<DF4>(e.k, x * m.rho, m.C1, m.C2, m.rho, m.tau) / m.rho;
    }
    ph64 = ph64 - lin64 - (double)mv.m * v.phi0 + mv.shift;
    ph = ph - lin - (float)m.m * e.phi0;   // its value is not used
    const double red = ph64 - kTwoPi * rint(ph64 * (1.0 / kTwoPi));
    float sn, cs;
    sincosf(f32_rn(red), &sn, &cs);
    // mode term amp e^{-i phase} and its tangent (d amp - i amp d phase) e^{-i phase}
    const float a = amp.v;
    const cf M = {a * cs, -a * sn};
    const float yp = (float)m.yp, yc = (float)m.yc;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float re0 = amp.d[q], im0 = -a * ph.d[q];
      const cf dM = {re0 * cs + im0 * sn, im0 * cs - re0 * sn};
      dP[q] = fadd(dP[q], fscale(dM, yp));
      dC[q] = fadd(dC[q], fscale(dM, yc));
    }
    P = fadd(P, fscale(M, yp));
    C = fadd(C, fscale(M, yc));
    dPi = fadd(dPi, fscale(M, (float)m.dyp));
    dCi = fadd(dCi, fscale(M, (float)m.dyc));
    Q = fadd(Q, fscale(M, (float)(spos ? m.ysp : m.ysm)));
  }
  w.P = P; w.C = C; w.dPi = dPi; w.dCi = dCi; w.Q = Q;
  w.tau = 0.0f;
#pragma unroll
  for (int q = 0; q < 4; ++q) w.dtn[q] = 0.0f;
  if (EARTH) {
    float dtau[4];
    tau_point_f32(tf, lnf, w.tau, dtau);
#pragma unroll
    for (int q = 0; q < 4; ++q) w.dtn[q] = -dtau[q] * (1.0f / 86400.0f);
  }
}

template <bool EARTH, int NARM>
__device__ __forceinline__ void point_f32_hm(const HMF32& H, const ProjF& pf, const TauF& tf, const ArmF* apc,
                                             const TimeF& tsc, float f, float lnf, cf (&D)[NARM][NP], cf (&Hs)[NARM]) {
  WaveF w;
  wave_f32_hm<EARTH>(H, pf, tf, f, lnf, w);
  project_f32<EARTH, NARM>(w, pf, apc, tsc, f, D, Hs);
}

// 2x3 register blocks covering the upper triangle of the padded 12x12 Gram matrix
static __constant__ unsigned char kBlkR[16] = {0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 3, 3, 4, 4, 5};
static __constant__ unsigned char kBlkC[16] = {0, 1, 2, 3, 0, 1, 2, 3, 1, 2, 3, 2, 3, 2, 3, 3};

// fixed-point Gram accumulation
constexpr int kQBits = 25;        // quantised |value| <= 2^25: the largest values of a column keep all 24 FP32 bits
constexpr int kQMinExp = -100;    // floor of the running column exponents
constexpr int kFlushTiles = 64;   // per tile |sum| <= 32 x 2 x 2^50 = 2^56, so 64 tiles stay below 2^62
// staging row stride in int2: a lane of the Gram loop reads row r0 (or c0) at column j while the
// other lanes of its half-warp read other rows at the same column; with 33 (odd) those rows fall
// in different banks (32 would put all of them in one bank: 6-way conflicts)
constexpr int kSR = 33;

// Gram slots per warp: one per Gram set, or, for a single set, one per half-warp (the two halves
// of a warp split each tile's points between them)
template <int NG>
__host__ __device__ constexpr int gram_slots() { return NG == 1 ? 2 : NG; }

// add the integer sums (at scale 2^-(M_r + M_c - 2 (kQBits - 1))) to the FP64 Gram of this warp;
// every (slot, entry) has exactly one owning lane
template <int NG, int NQ, int BPL, int NB>
__device__ __forceinline__ void flush_fixed(long long (&acc)[BPL][6], const int* M, double* fl, int lane) {
#pragma unroll
  for (int i = 0; i < BPL; ++i) {
    const int bl = (NG == 1 ? (lane & 15) : lane + 32 * i);
    if (bl < NB) {
      const int gs = bl >> 4, bi = bl & 15;
      const int slot = NG == 1 ? (lane >> 4) : gs;
      const int r0 = 2 * kBlkR[bi], c0 = 3 * kBlkC[bi];
      const int* m = M + gs * NQ;
#pragma unroll
      for (int e = 0; e < 6; ++e) {
        const int r = r0 + e / 3, c = c0 + e % 3;
        // exact power of two: the exponent lies in [2 kQMinExp - 48, 254 - 48], inside the normal range
        const double p2 = __longlong_as_double((long long)(1023 + m[r] + m[c] - 2 * (kQBits - 1)) << 52);
        fl[(slot * NQ + r) * NQ + c] += (double)acc[i][e] * p2;
        acc[i][e] = 0ll;
      }
    }
  }
}

// FP32 form of one event record: everything the per-point loop reads, rounded once per event by
// setup_f32_kernel (one thread per event) from the FP64 record
template <int MODEL>
struct __align__(16) F32Rec {
  double scale;     // Gram scale amp^2 / psd_scale (first three: the segment reduction reads them)
  double psi_sgn;   // sign of cos(iota): the psi column is Delta (see point_f32)
  double chi_alpha; // the chi1z tangent is d/dchi1 - alpha d/dchi2 (see setup_f32_kernel)
  double lnfmin, delta;
  typename std::conditional<MODEL == 2, HMF32, EvUnionF>::type ef;
  typename std::conditional<MODEL == 2, NoRec, PBF>::type pbf;
  ProjF pf;
  TauF tf;
  ArmF apc[2];
  TimeF tsc;
  GridF gf;
};
template <int MODEL>
__host__ __device__ constexpr size_t f32_stride() { return ((sizeof(F32Rec<MODEL>) + 15) / 16) * 16; }

template <int MODEL>
__global__ void __launch_bounds__(kEvBlock) setup_f32_kernel(DetDev det, const unsigned char* scratch, unsigned char* scratch32,
                                                             long long count, int narm, int earth, int epw) {
  const long long i = ev_thread(epw);
  if (i < 0 || i >= count) return;
  const unsigned char* rec = scratch + i * rec_stride<MODEL>();
  const SetupHdr& h = *reinterpret_cast<const SetupHdr*>(rec);
  const EvUnion& E = *reinterpret_cast<const EvUnion*>(rec + sizeof(SetupHdr));
  F32Rec<MODEL>& r = *reinterpret_cast<F32Rec<MODEL>*>(scratch32 + i * f32_stride<MODEL>());
  const GridEv& g = h.g;
  // chi1z and chi2z enter the phase almost only through one combination, so d/dchi1 and d/dchi2
  // are nearly parallel and their information sits in a small difference. The FP32 form carries
  // d/dchi1 - alpha d/dchi2 instead, alpha from the spin-orbit (f^-2/3) phase coefficient,
  // which that combination cancels in FP64; write_gram restores d/dchi1 in FP64.
  double alpha = 0.0, amp = 1.0;
  if constexpr (MODEL == 2) {
    if (g.ok) {
      amp = E.hm.k.ampPref.v;
      const double c1 = E.hm.k.pn.c3.d[P_CHI1], c2 = E.hm.k.pn.c3.d[P_CHI2];
      if (fabs(c2) > 1e-300 && isfinite(c1 / c2)) alpha = c1 / c2;
      hm_round(E.hm, r.ef, amp, alpha);
    }
  } else {
    const PhaseBasis& pb = *rec_basis<MODEL>(scratch, i);
    if (g.ok) {
      amp = MODEL == 0 ? E.tf2.ampK.v : E.phd.k.ampPref.v;
      const double c1 = pb.ins[2].d[P_CHI1], c2 = pb.ins[2].d[P_CHI2];
      if (fabs(c2) > 1e-300 && isfinite(c1 / c2)) alpha = c1 / c2;
      pbf_fill(pb, r.pbf, alpha);
      if (MODEL == 0) round_struct(E.tf2, r.ef.tf2, &E.tf2.ampK, amp, alpha);
      else round_struct(E.phd.k, r.ef.phd, &E.phd.k.ampPref, amp, alpha);
    }
  }
  r.chi_alpha = alpha;
  if (g.ok) {
    if constexpr (MODEL == 0) tau_setup(r.tf, E.tf2.Ms, E.tf2.vM, E.tf2.eta, alpha);
    else if constexpr (MODEL == 1) tau_setup(r.tf, E.phd.k.Ms, E.phd.k.vM, E.phd.k.eta, alpha);
    else tau_setup(r.tf, E.hm.k.Ms, E.hm.k.vM, E.hm.k.eta, alpha);
  }
  r.scale = amp * amp / det.psd_scale;
  projf_setup(r.pf, h.pj, det.sin_zeta);
  r.psi_sgn = r.pf.sgn;
  GridF& gf = r.gf;
  gf.lnfmin = (float)g.lnfmin; gf.delta = (float)g.delta; gf.fac_w = (float)g.fac_w; gf.w0 = (float)g.w0;
  gf.wl = (float)g.wl; gf.fmin = (float)g.fmin; gf.fcut = (float)g.fcut; gf.df = (float)g.df; gf.R = g.ok ? g.R : 0;
  gf.acc_l0 = (float)det.acc_l0; gf.acc_idl = (float)det.acc_idl;
  r.lnfmin = g.lnfmin;
  r.delta = g.delta;
  if (!earth) {
    time_f(r.pf, 0.0f, r.tsc);
    for (int a = 0; a < narm; ++a) arm_f(r.pf, r.tsc, a, r.apc[a]);
  }
}

// The other detectors of a group share detector 0's frequency grid and model record (same fmin, fmax
// and Earth-rotation flag, hence the same reference frequency), and the group kernel reads only their
// projection from their FP32 record slot: the pattern-function constants in FP64, rounded once
// (one thread per event). Nothing else of their slot is written.
template <int MODEL>
__global__ void __launch_bounds__(kEvBlock) proj_f32_kernel(EvBatch ev, DetDev det, unsigned char* scratch32, long long count,
                                                            int narm, int earth, int epw) {
  const long long i = ev_thread(epw);
  const long long n = ev.n0 + i;
  if (i < 0 || i >= count || n >= ev.N) return;
  const double* p = ev.p;
  const long long ld = ev.ld;
  ProjEv pj;
  proj_setup(pj, det, p[3 * ld + n], p[4 * ld + n], p[5 * ld + n], p[6 * ld + n], p[7 * ld + n], p[2 * ld + n]);
  F32Rec<MODEL>& r = *reinterpret_cast<F32Rec<MODEL>*>(scratch32 + i * f32_stride<MODEL>());
  projf_setup(r.pf, pj, det.sin_zeta);
  if (!earth) {
    time_f(r.pf, 0.0f, r.tsc);
    for (int a = 0; a < narm; ++a) arm_f(r.pf, r.tsc, a, r.apc[a]);
  }
}

// FP64 set-up records copied from another detector of the same grid: only the projection header is
// the detector's own (events ev.n0 .. of a gathered batch, records 0 .. count - 1)
template <int MODEL>
__global__ void __launch_bounds__(kEvBlock) proj_patch_kernel(EvBatch ev, DetDev det, unsigned char* scratch, long long count,
                                                              int epw) {
  const long long i = ev_thread(epw);
  const long long n = ev.n0 + i;
  if (i < 0 || i >= count || n >= ev.N) return;
  const double* p = ev.p;
  const long long ld = ev.ld;
  SetupHdr& h = *reinterpret_cast<SetupHdr*>(scratch + i * rec_stride<MODEL>());
  proj_setup(h.pj, det, p[3 * ld + n], p[4 * ld + n], p[5 * ld + n], p[6 * ld + n], p[7 * ld + n], p[2 * ld + n]);
}

// per-block state of the FP32 kernels (shared memory); the staging area is dynamic shared memory
template <int MODEL, int NG>
struct F32State {
  F32Rec<MODEL> r;
  int colM[2][kWarps][NG * 12];                      // running column exponents, double-buffered
  double fl[kWarps][gram_slots<NG>()][12][12];       // FP64 Gram per warp and slot
  double gsum[NG * NEX];                             // Gram per set (and strain products), summed over warps
  int badw[kWarps];
  long long rec;
};

template <int MODEL, int NG>
__device__ inline void f32_prepare(const unsigned char* scratch32, long long rec, F32State<MODEL, NG>& S) {
  const uint4* src = reinterpret_cast<const uint4*>(scratch32 + rec * f32_stride<MODEL>());
  uint4* dst = reinterpret_cast<uint4*>(&S.r);
  for (int i = threadIdx.x; i < (int)(sizeof(F32Rec<MODEL>) / 16); i += blockDim.x) dst[i] = src[i];
  if (threadIdx.x == 0) S.rec = rec;
  __syncthreads();
}

// FP32 frequency grid of one event, traversed by a block of kThreads in steps of kThreads points
// (warp w takes points base + 32 w + lane). Geometric grid: f_k = f_tile exp(lane delta),
// ln f_k = ln f_tile + lane delta, with the tile anchors formed in FP64; each lane computes the
// anchor of one of the warp's next 32 tiles, and the tiles read them by shuffle.
struct GridIterF {
  float anc_f = 0.0f, anc_l = 0.0f;
  int it0 = -1000000;
  // call once per step, by all lanes of the warp; returns the point's f, ln f and trapezoid weight
  template <int MODEL>
  __device__ __forceinline__ void step(const F32Rec<MODEL>& r, int spacing, int base, int lane, int warp) {
    const int it = base / kThreads;
    if (spacing == 0 && it - it0 >= 32) {
      it0 = it;
      const double l = r.lnfmin + (double)(((long long)(it + lane) * kWarps + warp) * 32) * r.delta;
      anc_f = (float)exp(l);
      anc_l = (float)l;
    }
    ftile = __shfl_sync(0xffffffffu, anc_f, (it - it0) & 31);
    ltile = __shfl_sync(0xffffffffu, anc_l, (it - it0) & 31);
  }
  template <int MODEL>
  __device__ __forceinline__ void point(const F32Rec<MODEL>& r, int spacing, int k, int lane, float& f, float& lnf,
                                        float& w) const {
    const GridF& gf = r.gf;
    const int R = gf.R;
    if (spacing == 0) {
      lnf = fmaf((float)lane, gf.delta, ltile);
      if (k == R - 1) { f = gf.fcut; w = f * gf.wl; }
      else if (k == 0) { f = gf.fmin; w = f * gf.w0; }
      else { f = ftile * expf((float)lane * gf.delta); w = f * gf.fac_w; }
    } else {
      f = (k == R - 1) ? gf.fcut : gf.fmin + (float)k * gf.df;
      lnf = logf(f);
      w = (k == 0 || k == R - 1) ? 0.5f * gf.df : gf.df;
    }
  }
  float ftile = 0.0f, ltile = 0.0f;
};

// Gram of points [k0, k1) (k0 a multiple of kThreads) into S.gsum, summed over warps
template <int MODEL, bool EARTH, int NARM, int NG>
__device__ inline void f32_item(const EvBatch& ev, const DetDev& det, F32State<MODEL, NG>& S, int2* stage, int k0, int k1,
                                bool sd) {
  constexpr int NQ = 12;  // padded parameter count
  const F32Rec<MODEL>& r = S.r;
  const GridF& gf = r.gf;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int NB = 16 * NG;
  constexpr int BPL = (NB + 31) / 32;
  long long acc[BPL][6];
#pragma unroll
  for (int i = 0; i < BPL; ++i)
#pragma unroll
    for (int e = 0; e < 6; ++e) acc[i][e] = 0ll;
  int2* my = stage + (size_t)warp * NG * NQ * kSR;
  auto& colM = S.colM;
  auto& fl = S.fl;
  // zero padding row (parameter 11) once; running column exponents start below any value
  for (int gs = 0; gs < NG; ++gs) my[(gs * NQ + 11) * kSR + lane] = make_int2(0, 0);
  for (int i = lane; i < 2 * NG * NQ; i += 32) (&colM[i / (NG * NQ)][warp][0])[i % (NG * NQ)] = kQMinExp;
  for (int i = lane; i < gram_slots<NG>() * NQ * NQ; i += 32) (&fl[warp][0][0][0])[i] = 0.0;
  if (lane == 0) S.badw[warp] = 0;
  int par = 0, tiles = 0;
  GridIterF grid;
  bool moved = false, bad = false;
  __syncwarp();
  for (int base = k0; base < k1; base += kThreads) {
    const int k = base + tid;
    cf D[NARM][NP], Hs[NARM];
    float sw = 0.0f;
    grid.step(r, ev.spacing, base, lane, warp);
    if (k < k1) {
      float f, lnf, w;
      grid.point(r, ev.spacing, k, lane, f, lnf, w);
      const float Sn = psd_at_f(det, f, lnf, gf.acc_l0, gf.acc_idl);
      sw = sqrtf(4.0f * w / Sn);
      if constexpr (MODEL == 2) point_f32_hm<EARTH, NARM>(r.ef, r.pf, r.tf, r.apc, r.tsc, f, lnf, D, Hs);
      else point_f32<MODEL, EARTH, NARM>(r.ef, r.pbf, r.pf, r.tf, r.apc, r.tsc, f, lnf, D, Hs);
    } else {
#pragma unroll
      for (int a = 0; a < NARM; ++a) {
#pragma unroll
        for (int q = 0; q < NP; ++q) D[a][q] = {0.0f, 0.0f};
        Hs[a] = {0.0f, 0.0f};
      }
    }
    // Quantise the sqrt(weight)-scaled derivative vectors to integers, |q| <= 2^kQBits,
    // on a per-column power-of-two scale that follows the largest magnitude this warp has seen.
    // The rounding is a perturbation of the vectors themselves, so the accumulated Gram matrix
    // stays an exact Gram matrix of slightly perturbed vectors (positive semidefinite).
    const int* Mo = &colM[par][warp][0];
    int* Mn = &colM[par ^ 1][warp][0];
#pragma unroll
    for (int gs = 0; gs < NG; ++gs)
#pragma unroll
      for (int q = 0; q <= NP; ++q) {   // column NP: the strain itself, staged only for SNR derivatives
        if (q == NP && !sd) break;
        const cf d0 = q < NP ? D[0][q] : Hs[0], d1 = q < NP ? D[NARM - 1][q] : Hs[NARM - 1];
        cf u;
        if (NG == 1) u = fscale(d0, sw);
        else if (NG == 2) u = gs == 0 ? fscale(fadd(d0, d1), sw * 1.2247448713915890f)
                                      : fscale(fadd(d0, fscale(d1, -1.0f)), sw * 0.70710678118654752f);
        else u = gs == 0 ? fscale(d0, sw) : gs == 1 ? fscale(d1, sw) : fscale(fadd(d0, d1), -sw);
        const int mold = Mo[gs * NQ + q];
        const unsigned bits = max(__float_as_uint(fabsf(u.re)), __float_as_uint(fabsf(u.im)));
        const int e = (int)(__reduce_max_sync(0xffffffffu, bits) >> 23) - 127;
        bad |= e > 127;                                   // Inf or NaN somewhere in the tile
        const int mnew = min(max(mold, e), 127);
        moved |= mnew != mold;
        if (lane == 0) Mn[gs * NQ + q] = mnew;
        const float s = __int_as_float((127 + kQBits - 1 - mnew) << 23);   // 2^(kQBits-1-mnew), exact scaling
        const int qr = __float2int_rn(u.re * s);
        const int qi = __float2int_rn(u.im * s);
        my[(gs * NQ + q) * kSR + lane] = make_int2(qr, qi);
      }
    __syncwarp();
#pragma unroll
    for (int i = 0; i < BPL; ++i) {
      const int bl = (NG == 1 ? (lane & 15) : lane + 32 * i);
      if (bl < NB) {
        const int gs = bl >> 4, bi = bl & 15;
        const int r0 = 2 * kBlkR[bi], c0 = 3 * kBlkC[bi];
        const int2* base_g = my + gs * NQ * kSR;
        if (moved) {   // rescale the running sums to the new column scales
          const int* mo = Mo + gs * NQ;
          const int* mn = Mn + gs * NQ;
#pragma unroll
          for (int e = 0; e < 6; ++e) {
            const int r = r0 + e / 3, c = c0 + e % 3;
            const int sh = (mn[r] - mo[r]) + (mn[c] - mo[c]);
            acc[i][e] = sh >= 63 ? 0ll : (acc[i][e] >> sh);
          }
        }
        const int j0 = NG == 1 ? 16 * (lane >> 4) : 0;
        constexpr int NJ = NG == 1 ? 16 : 32;
#pragma unroll 4
        for (int jj = 0; jj < NJ; ++jj) {
          const int j = j0 + jj;
          const int2 a0 = base_g[(r0 + 0) * kSR + j], a1 = base_g[(r0 + 1) * kSR + j];
          const int2 b0 = base_g[(c0 + 0) * kSR + j], b1 = base_g[(c0 + 1) * kSR + j], b2 = base_g[(c0 + 2) * kSR + j];
          acc[i][0] += (long long)a0.x * b0.x + (long long)a0.y * b0.y;
          acc[i][1] += (long long)a0.x * b1.x + (long long)a0.y * b1.y;
          acc[i][2] += (long long)a0.x * b2.x + (long long)a0.y * b2.y;
          acc[i][3] += (long long)a1.x * b0.x + (long long)a1.y * b0.y;
          acc[i][4] += (long long)a1.x * b1.x + (long long)a1.y * b1.y;
          acc[i][5] += (long long)a1.x * b2.x + (long long)a1.y * b2.y;
        }
      }
    }
    par ^= 1;
    moved = false;
    if (++tiles == kFlushTiles) {   // keep |sum| < 2^63: move the integer sums into FP64
      flush_fixed<NG, NQ, BPL, NB>(acc, &colM[par][warp][0], &fl[warp][0][0][0], lane);
      tiles = 0;
    }
    __syncwarp();
  }
  flush_fixed<NG, NQ, BPL, NB>(acc, &colM[par][warp][0], &fl[warp][0][0][0], lane);
  if (lane == 0 && bad) S.badw[warp] = 1;
  __syncthreads();
  // sum over warps in FP64, per Gram set; NaN if any tile held Inf or NaN
  int anybad = 0;
#pragma unroll
  for (int w = 0; w < kWarps; ++w) anybad |= S.badw[w];
  const double* red = &fl[0][0][0][0];  // [kWarps][gram_slots][NQ][NQ]
  constexpr int NS = gram_slots<NG>();
  for (int e = tid; e < NG * NEX; e += kThreads) {
    const int gs = e / NEX, pe = e % NEX;
    const int a = pe < NE ? kPairA[pe] : pe - NE, b = pe < NE ? kPairB[pe] : NP;   // (a, NP): strain products
    double v = 0.0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
      v += red[((size_t)(w * NS + gs) * NQ + a) * NQ + b];
      if (NG == 1) v += red[((size_t)(w * NS + 1) * NQ + a) * NQ + b];
    }
    S.gsum[e] = anybad ? __longlong_as_double(0x7ff8000000000000ll) : (pe >= NE && !sd ? 0.0 : v);
  }
  __syncthreads();
}

template <int MODEL, bool EARTH, int NARM, int NG>
__global__ void __launch_bounds__(kThreads, 5) fisher_kernel_f32(EvBatch ev, DetDev det, const unsigned char* scratch32,
                                                                 double* out_arm, double* out_det, double* out_sd_arm,
                                                                 double* out_sd_det, int accum) {
  extern __shared__ __align__(16) unsigned char stage_raw[];
  __shared__ F32State<MODEL, NG> S;
  const long long n = ev.n0 + blockIdx.x;
  if (n >= ev.N) return;
  f32_prepare<MODEL, NG>(scratch32, blockIdx.x, S);
  f32_item<MODEL, EARTH, NARM, NG>(ev, det, S, reinterpret_cast<int2*>(stage_raw), 0, S.r.gf.R, out_sd_arm || out_sd_det);
  write_gram<NG>(S.gsum, S.r.scale, ColMix{2.0 * S.r.psi_sgn, S.r.chi_alpha}, n, ev.N, out_arm, out_det, out_sd_arm,
                 out_sd_det, accum);
}

template <int MODEL, bool EARTH, int NARM, int NG>
__global__ void __launch_bounds__(kThreads, 5) fisher_seg_kernel_f32(EvBatch ev, DetDev det, const unsigned char* scratch32,
                                                                     long long count, SegInfo si, int sd) {
  extern __shared__ __align__(16) unsigned char stage_raw[];
  __shared__ F32State<MODEL, NG> S;
  if (threadIdx.x == 0) S.rec = -1;
  __syncthreads();
  long long item, rec;
  int k0;
  while (next_item(si, count, item, rec, k0)) {
    if (S.rec != rec) f32_prepare<MODEL, NG>(scratch32, rec, S);
    const int R = S.r.gf.R;
    const int k1 = k0 + si.seg < R ? k0 + si.seg : R;
    f32_item<MODEL, EARTH, NARM, NG>(ev, det, S, reinterpret_cast<int2*>(stage_raw), k0, k1, sd != 0);
    double* o = si.partial + item * (NG * NEX);
    for (int e = threadIdx.x; e < NG * NEX; e += blockDim.x) o[e] = S.gsum[e];
  }
}

// ------------------------------------------------------------------ detector groups
// Detectors that share the frequency grid (same fmin, fmax, Earth-rotation flag) share the
// waveform at every point: hp, hc and their tangents do not depend on the detector. For the network
// total, one block per event evaluates the waveform once per point and projects it onto every
// detector of the group; all their derivative vectors are accumulated into one exact Gram (the
// network Gram is the Gram of all detectors' vectors together), so the waveform cost is paid once
// per group instead of once per detector.
constexpr int kMaxGroup = 4;

struct GroupDev {
  DetDev det[kMaxGroup];
  float wr[kMaxGroup];   // sqrt(psd_scale of detector 0 / psd_scale of detector d): common Gram scale
  int same_psd[kMaxGroup];   // detector d has detector d - 1's PSD table (and scale): same weight per point
  int nd;
  long long slice;       // bytes between the FP32 record areas of consecutive detectors
};

struct GroupProj {
  ProjF pf[kMaxGroup];
  ArmF apc[kMaxGroup][2];
  TimeF tsc[kMaxGroup];
};

// TRI: the group holds a triangle; without one the triangle branch (and its registers) is left out
template <int MODEL, bool EARTH, bool TRI>
__device__ inline void f32_item_group(const EvBatch& ev, const GroupDev& g, F32State<MODEL, 1>& S, const GroupProj& gp,
                                      int2* stage, int k1) {
  constexpr int NQ = 12;
  const F32Rec<MODEL>& r = S.r;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  long long acc[1][6];
#pragma unroll
  for (int e = 0; e < 6; ++e) acc[0][e] = 0ll;
  int2* my = stage + (size_t)warp * NQ * kSR;
  auto& colM = S.colM;
  auto& fl = S.fl;
  my[11 * kSR + lane] = make_int2(0, 0);   // padding row (no strain column here)
  for (int i = lane; i < 2 * NQ; i += 32) colM[i / NQ][warp][i % NQ] = kQMinExp;
  for (int i = lane; i < gram_slots<1>() * NQ * NQ; i += 32) (&fl[warp][0][0][0])[i] = 0.0;
  if (lane == 0) S.badw[warp] = 0;
  int par = 0, tiles = 0;
  bool moved = false, bad = false;
  const int bi = lane & 15;
  const int r0 = 2 * kBlkR[bi], c0 = 3 * kBlkC[bi];
  const int j0 = 16 * (lane >> 4);
  __syncwarp();
  // one vector per lane (the lane's point) into the Gram: quantise, stage, accumulate (as f32_item,
  // one Gram set, the two half-warps taking 16 points each)
  auto add = [&](const cf (&u)[NP]) {
    const int* Mo = &colM[par][warp][0];
    int* Mn = &colM[par ^ 1][warp][0];
#pragma unroll
    for (int q = 0; q < NP; ++q) {
      const int mold = Mo[q];
      const unsigned bits = max(__float_as_uint(fabsf(u[q].re)), __float_as_uint(fabsf(u[q].im)));
      const int e = (int)(__reduce_max_sync(0xffffffffu, bits) >> 23) - 127;
      bad |= e > 127;
      const int mnew = min(max(mold, e), 127);
      moved |= mnew != mold;
      if (lane == 0) Mn[q] = mnew;
      const float sc = __int_as_float((127 + kQBits - 1 - mnew) << 23);
      my[q * kSR + lane] = make_int2(__float2int_rn(u[q].re * sc), __float2int_rn(u[q].im * sc));
    }
    __syncwarp();
    if (moved) {
#pragma unroll
      for (int e = 0; e < 6; ++e) {
        const int rr = r0 + e / 3, cc = c0 + e % 3;
        const int sh = (Mn[rr] - Mo[rr]) + (Mn[cc] - Mo[cc]);
        acc[0][e] = sh >= 63 ? 0ll : (acc[0][e] >> sh);
      }
    }
#pragma unroll 4
    for (int jj = 0; jj < 16; ++jj) {
      const int j = j0 + jj;
      const int2 a0 = my[(r0 + 0) * kSR + j], a1 = my[(r0 + 1) * kSR + j];
      const int2 b0 = my[(c0 + 0) * kSR + j], b1 = my[(c0 + 1) * kSR + j], b2 = my[(c0 + 2) * kSR + j];
      acc[0][0] += (long long)a0.x * b0.x + (long long)a0.y * b0.y;
      acc[0][1] += (long long)a0.x * b1.x + (long long)a0.y * b1.y;
      acc[0][2] += (long long)a0.x * b2.x + (long long)a0.y * b2.y;
      acc[0][3] += (long long)a1.x * b0.x + (long long)a1.y * b0.y;
      acc[0][4] += (long long)a1.x * b1.x + (long long)a1.y * b1.y;
      acc[0][5] += (long long)a1.x * b2.x + (long long)a1.y * b2.y;
    }
    par ^= 1;
    moved = false;
    if (++tiles == kFlushTiles) {
      flush_fixed<1, NQ, 1, 16>(acc, &colM[par][warp][0], &fl[warp][0][0][0], lane);
      tiles = 0;
    }
    __syncwarp();
  };
  GridIterF grid;
  const int nd = g.nd;
  float sw = 0.0f;
  for (int base = 0; base < k1; base += kThreads) {
    const int k = base + tid;
    grid.step(r, ev.spacing, base, lane, warp);
    const bool valid = k < k1;
    float f = 0.0f, lnf = 0.0f, w = 0.0f;
    // the waveform once per point for the group: the 22-mode models keep its compact form across
    // the detector loop and expand it per detector (fewer live registers across the loop)
    WaveF wv;
    Wave22 wc;
    if (valid) {
      grid.point(r, ev.spacing, k, lane, f, lnf, w);
      if constexpr (MODEL == 2) wave_f32_hm<EARTH>(r.ef, r.pf, r.tf, f, lnf, wv);
      else wave22_f32<MODEL, EARTH>(r.ef, r.pbf, r.tf, f, lnf, wc);
    }
    float sd = 0.0f, cd = 1.0f;   // the Earth-rotation angle is the same for every detector
    if (EARTH && valid) {
      if constexpr (MODEL == 2) rot_sc_tau(wv.tau, sd, cd);
      else rot_sc_tau(wc.tau, sd, cd);
    }
    for (int d = 0; d < nd; ++d) {
      const DetDev& det = g.det[d];
      if (!(d > 0 && g.same_psd[d]))   // (a detector sharing the previous one's table reuses its weight)
        sw = valid ? sqrtf(4.0f * w / psd_at_f(det, f, lnf, (float)det.acc_l0, (float)det.acc_idl)) * g.wr[d] : 0.0f;
      if constexpr (MODEL != 2) {
        if (valid) expand22(wc, gp.pf[d], wv);
      }
      cf u[NP];
      if (!TRI || det.shape == 0) {
        cf D[1][NP], Hs[1];
        if (valid) project_f32_rot<EARTH, 1>(wv, gp.pf[d], gp.apc[d], gp.tsc[d], f, sd, cd, D, Hs);
#pragma unroll
        for (int q = 0; q < NP; ++q) u[q] = valid ? fscale(D[0][q], sw) : cf{0.0f, 0.0f};
        add(u);
      } else {
        // triangle total: G(U) + G(V) + G(U+V) = G(sqrt(3/2)(U+V)) + G(sqrt(1/2)(U-V))
        cf D[2][NP], Hs[2];
        if (valid) project_f32_rot<EARTH, 2>(wv, gp.pf[d], gp.apc[d], gp.tsc[d], f, sd, cd, D, Hs);
#pragma unroll
        for (int q = 0; q < NP; ++q) u[q] = valid ? fscale(fadd(D[0][q], D[1][q]), sw * 1.2247448713915890f) : cf{0.0f, 0.0f};
        add(u);
#pragma unroll
        for (int q = 0; q < NP; ++q)
          u[q] = valid ? fscale(fadd(D[0][q], fscale(D[1][q], -1.0f)), sw * 0.70710678118654752f) : cf{0.0f, 0.0f};
        add(u);
      }
    }
  }
  flush_fixed<1, NQ, 1, 16>(acc, &colM[par][warp][0], &fl[warp][0][0][0], lane);
  if (lane == 0 && bad) S.badw[warp] = 1;
  __syncthreads();
  int anybad = 0;
#pragma unroll
  for (int w = 0; w < kWarps; ++w) anybad |= S.badw[w];
  const double* red = &fl[0][0][0][0];
  constexpr int NS = gram_slots<1>();
  for (int e = tid; e < NEX; e += kThreads) {
    double v = 0.0;
    if (e < NE) {
      const int a = kPairA[e], b = kPairB[e];
#pragma unroll
      for (int w = 0; w < kWarps; ++w)
        v += red[((size_t)(w * NS) * NQ + a) * NQ + b] + red[((size_t)(w * NS + 1) * NQ + a) * NQ + b];
    }
    S.gsum[e] = anybad ? __longlong_as_double(0x7ff8000000000000ll) : v;
  }
  __syncthreads();
}

// Six blocks per SM (80 registers) for the 22-mode models: the fixed-latency FP32 chains are its top
// stall and two more warps per SM outweigh the extra spills (IMRPhenomD, L1 + H1, 10^4 events:
// 2.688 ms against 2.729 ms at five blocks and 96 registers; seven blocks, 72 registers, 2.45 ms
// against 2.39 ms once the compact waveform cut the spills). IMRPhenomHM as well, since its FP64 mode
// phases lost their divisions (ETS + CE1Id + CE2NM, 2 * 10^4 events: FP32 form 178.7 k Fisher/s at
// six blocks, 175.4 k at five, 168.9 k at four; 174.5 k at seven against 178.4 k at six in another
// run). (The triangle kernel was slower at six: 2.390 against 2.305 ms.)
template <int MODEL>
__host__ __device__ constexpr int group_min_blocks() { return 6; }

template <int MODEL, bool EARTH, bool TRI>
__global__ void __launch_bounds__(kThreads, group_min_blocks<MODEL>()) fisher_group_kernel_f32(EvBatch ev, GroupDev g,
                                                                       const unsigned char* scratch32, double* out_det,
                                                                       int accum) {
  extern __shared__ __align__(16) unsigned char stage_raw[];
  __shared__ F32State<MODEL, 1> S;
  __shared__ GroupProj gp;
  const long long n = ev.n0 + blockIdx.x;
  if (n >= ev.N) return;
  if ((int)threadIdx.x < g.nd) {   // the projection pieces of every detector of the group
    const int d = threadIdx.x;
    const F32Rec<MODEL>& rd =
        *reinterpret_cast<const F32Rec<MODEL>*>(scratch32 + d * g.slice + (size_t)blockIdx.x * f32_stride<MODEL>());
    gp.pf[d] = rd.pf;
    gp.apc[d][0] = rd.apc[0];
    gp.apc[d][1] = rd.apc[1];
    gp.tsc[d] = rd.tsc;
  }
  f32_prepare<MODEL, 1>(scratch32, blockIdx.x, S);
  f32_item_group<MODEL, EARTH, TRI>(ev, g, S, gp, reinterpret_cast<int2*>(stage_raw), S.r.gf.R);
  write_gram<1>(S.gsum, S.r.scale, ColMix{2.0 * S.r.psi_sgn, S.r.chi_alpha}, n, ev.N, nullptr, out_det, nullptr, nullptr,
                accum);
}

// ------------------------------------------------------------------ detector groups, FP64
// The FP64 network total of detectors that share the grid (same fmin, fmax, Earth-rotation flag),
// as the FP32 group kernel: per point the waveform and its tangent once (the FP64 dual
// evaluation, about two thirds of one detector's work), then each detector's Earth-rotation time,
// pattern functions, derivative vectors and PSD weight, all accumulated into one Gram (the Gram of
// the network is the Gram of all its detectors' vectors). The model record and the grid are detector
// 0's; every detector's projection header comes from its own set-up record slice. The Gram entries
// are summed in FP64 as in the per-detector kernel, only in another order across detectors.
struct GroupDev64 {
  DetDev det[kMaxGroup];
  const unsigned char* rec[kMaxGroup];   // each detector's set-up records
  int same_psd[kMaxGroup];               // detector d has detector d - 1's PSD table: the same weight
  int nd;
};

template <int MODEL, bool EARTH>
struct F64GroupState {
  F64State<1, 1, np_of<MODEL>()> S;   // detector 0's record (model, grid) and the Gram
  ProjEv pj[kMaxGroup];
  ArmPat ap[kMaxGroup];                // without Earth rotation: each detector's pattern functions
  TimeState ts[kMaxGroup];
};

template <int MODEL, bool EARTH>
__device__ inline void f64g_prepare(const GroupDev64& g, long long rec, F64GroupState<MODEL, EARTH>& G) {
  block_load<MODEL>(G.S.E, G.S.pj, G.S.g, g.rec[0], rec, (MODEL == 0 || MODEL == 1) ? &G.S.pb : nullptr);
  if constexpr (MODEL == 0 || MODEL == 1) {
    if (threadIdx.x == 32 && G.S.g.ok) {
      if constexpr (MODEL == 0) tau_setup_d(G.S.td, G.S.E.tf2.Ms, G.S.E.tf2.vM, G.S.E.tf2.eta);
      else {
        tau_setup_d(G.S.td, G.S.E.phd.k.Ms, G.S.E.phd.k.vM, G.S.E.phd.k.eta);
        amp_setup_d(G.S.td, G.S.E.phd.k.ampPref, G.S.E.phd.k.MG);
      }
    }
  }
  if ((int)threadIdx.x < g.nd) {
    const int d = threadIdx.x;
    G.pj[d] = reinterpret_cast<const SetupHdr*>(g.rec[d] + rec * rec_stride<MODEL>())->pj;
    if (!EARTH) {
      time_state(G.pj[d], G.pj[d].tc, G.ts[d]);
      arm_pattern(G.pj[d], g.det[d].sin_zeta, G.ts[d].x, 0, G.ap[d]);
    }
  }
  if (threadIdx.x == 0) G.S.rec = rec;
  __syncthreads();
}

// Gram of points [k0, k1) of the group into G.S.gsum (summed over warps; no strain products).
// TRI: the group holds a triangle, whose two combined vectors sqrt(3/2)(U + V) and sqrt(1/2)(U - V)
// (its three arms' total, as in the per-detector kernel) both go into the Gram; the staging area
// then has a second set of rows.
template <int MODEL, bool EARTH, bool TRI>
__device__ inline void f64g_item(const EvBatch& ev, const GroupDev64& g, F64GroupState<MODEL, EARTH>& G, cd* stage,
                                 int k0, int k1) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int NPM = np_of<MODEL>();
  constexpr int NEM = ne_of(NPM), NEXM = nex_of(NPM);
  constexpr int NPS = NPM + 1;
  constexpr int NI = ndir_of<MODEL>();
  constexpr int EPT = (NEM + 31) / 32;
  double acc[EPT];
  int ea[EPT], eb[EPT];
  bool own[EPT];
#pragma unroll
  for (int i = 0; i < EPT; ++i) {
    acc[i] = 0.0;
    const int e = lane + 32 * i;
    own[i] = e < NEM;
    ea[i] = eb[i] = 0;
    if (own[i]) pair_n(NPM, e, ea[i], eb[i]);
  }
  constexpr int NSET = TRI ? 2 : 1;
  cd* my = stage + (size_t)warp * NSET * NPS * kSR64;
  const int nd = g.nd;
  double sw = 0.0;
  // accumulate the rows of staging set gs into this lane's entries
  auto gram = [&](int gs) {
    const cd* base_s = my + gs * NPS * kSR64;
#pragma unroll
    for (int i = 0; i < EPT; ++i) {
      if (own[i]) {
        const cd* ra = base_s + ea[i] * kSR64;
        const cd* rb = base_s + eb[i] * kSR64;
        double s2 = 0.0;
#pragma unroll 8
        for (int j = 0; j < 32; ++j) s2 += ra[j].re * rb[j].re + ra[j].im * rb[j].im;
        acc[i] += s2;
      }
    }
  };
  for (int base = k0; base < k1; base += kThreads) {
    const int k = base + tid;
    const bool valid = k < k1;
    double f = 0.0, lnf = 0.0, w = 0.0;
    cd P, C, dP[NI], dC[NI], dPi, dCi;
    DualOf<MODEL> tau(0.0);
    double phi0, dtn[NI], dphl = 0.0, dphd = 0.0, dphe = 0.0;
#pragma unroll
    for (int q = 0; q < NI; ++q) dtn[q] = 0.0;
    if (valid) {
      grid_point(G.S.g, ev.spacing, k, f, lnf, w);
      wave_point_dual<MODEL, EARTH>(G.S.E, G.S.pj, f, lnf, P, C, dP, dC, dPi, dCi, tau, phi0,
                                    (MODEL == 0 || MODEL == 1) ? &G.S.pb : nullptr,
                                    (MODEL == 0 || MODEL == 1) ? &G.S.td : nullptr);
      if (EARTH) {
#pragma unroll
        for (int q = 0; q < NI; ++q) dtn[q] = -tau.d[q] / kDay;
      }
      analytic_tangents<MODEL>(G.S.E, lnf, dphl, dphd, dphe);
    }
    for (int d = 0; d < nd; ++d) {
      const bool tri = TRI && g.det[d].shape == 1;
      TimeState ts;
      if (valid) {
        if (!(d > 0 && g.same_psd[d])) sw = sqrt(4.0 * w / psd_at(g.det[d], f, lnf));
        if (EARTH) time_state(G.pj[d], G.S.pj.tc - tau.v / kDay, ts);
        else ts = G.ts[d];
      }
      for (int a = 0; a < (tri ? 2 : 1); ++a) {
        cd D[NPS];
        if (valid) {
          ArmPat ap;
          if (EARTH || a > 0) arm_pattern(G.pj[d], g.det[d].sin_zeta, ts.x, a, ap);
          else ap = G.ap[d];
          arm_derivs<NI>(G.pj[d], ap, ts, f, P, C, dP, dC, dPi, dCi, dtn, D);
          analytic_columns<MODEL>(cadd(cscale(P, ap.Fp), cscale(cmuli(C), ap.Fc)), dphl, dphd, dphe, D);
        }
        if (!tri) {
#pragma unroll
          for (int q = 0; q < NPM; ++q) my[q * kSR64 + lane] = valid ? cscale(D[q], sw) : cd{0.0, 0.0};
        } else if (a == 0) {   // the first arm, weighted, waits in set 1's rows
#pragma unroll
          for (int q = 0; q < NPM; ++q) my[(NPS + q) * kSR64 + lane] = valid ? cscale(D[q], sw) : cd{0.0, 0.0};
        } else {               // U + V into set 0, U - V into set 1 (this lane's own slots)
#pragma unroll
          for (int q = 0; q < NPM; ++q) {
            const cd u = my[(NPS + q) * kSR64 + lane], v = valid ? cscale(D[q], sw) : cd{0.0, 0.0};
            my[q * kSR64 + lane] = cscale(cadd(u, v), 1.2247448713915890);
            my[(NPS + q) * kSR64 + lane] = cscale(cadd(u, cscale(v, -1.0)), 0.70710678118654752);
          }
        }
      }
      __syncwarp();
      gram(0);
      if (tri) gram(1);
      __syncwarp();
    }
  }
  // cross-warp reduction through the staging area
  __syncthreads();
  double* red = reinterpret_cast<double*>(stage);   // [kWarps][NEM]
#pragma unroll
  for (int i = 0; i < EPT; ++i)
    if (own[i]) red[warp * NEM + lane + 32 * i] = acc[i];
  __syncthreads();
  for (int e = tid; e < NEXM; e += kThreads) {
    double s2 = 0.0;
    if (e < NEM) {
#pragma unroll
      for (int wp = 0; wp < kWarps; ++wp) s2 += red[wp * NEM + e];
    }
    G.S.gsum[e] = s2;
  }
  __syncthreads();
}

template <int MODEL, bool EARTH, bool TRI>
__global__ void __launch_bounds__(kThreads) fisher_group_kernel64(EvBatch ev, GroupDev64 g, double* out_det, int accum) {
  extern __shared__ __align__(16) unsigned char stage_raw[];
  __shared__ F64GroupState<MODEL, EARTH> G;
  const long long n = ev.n0 + blockIdx.x;
  if (n >= ev.N) return;
  f64g_prepare<MODEL, EARTH>(g, blockIdx.x, G);
  f64g_item<MODEL, EARTH, TRI>(ev, g, G, reinterpret_cast<cd*>(stage_raw), 0, G.S.g.ok ? G.S.g.R : 0);
  write_gram<1, np_of<MODEL>()>(G.S.gsum, 1.0, ColMix{0.0, 0.0}, n, ev.N, nullptr, out_det, nullptr, nullptr, accum);
}

template <int MODEL, bool EARTH, bool TRI>
__global__ void __launch_bounds__(kThreads) fisher_group_seg_kernel64(EvBatch ev, GroupDev64 g, long long count,
                                                                      SegInfo si) {
  static_assert(np_of<MODEL>() == NP, "segmented launches carry 11-parameter partial Grams");
  extern __shared__ __align__(16) unsigned char stage_raw[];
  __shared__ F64GroupState<MODEL, EARTH> G;
  if (threadIdx.x == 0) G.S.rec = -1;
  __syncthreads();
  long long item, rec;
  int k0;
  while (next_item(si, count, item, rec, k0)) {
    if (G.S.rec != rec) f64g_prepare<MODEL, EARTH>(g, rec, G);
    const int R = G.S.g.ok ? G.S.g.R : 0;
    const int k1 = k0 + si.seg < R ? k0 + si.seg : R;
    f64g_item<MODEL, EARTH, TRI>(ev, g, G, reinterpret_cast<cd*>(stage_raw), k0, k1);
    double* o = si.partial + item * NEX;
    for (int e = threadIdx.x; e < NEX; e += blockDim.x) o[e] = G.S.gsum[e];
  }
}

// FP64 SNR of a group of detectors on one grid (gwfast/signal.py:658-777 per detector): the waveform
// value and the time to coalescence once per point for the group, then each detector's pattern
// functions and PSD weight. Outputs per detector as snr_kernel: its arms' sums at out_arm[d] (slot a at
// out_arm[d] + a N, when not null) and the network total 4 sum over all arms into out_det.
struct GroupSNR64 {
  DetDev det[kMaxGroup];
  const unsigned char* rec[kMaxGroup];   // each detector's set-up records (d > 0: the header is read)
  double* out_arm[kMaxGroup];
  int same_psd[kMaxGroup];
  int nd;
};

template <int MODEL, bool EARTH, bool TRI>
__global__ void __launch_bounds__(kThreads) snr_group_kernel64(EvBatch ev, GroupSNR64 g, double* out_det, int accum) {
  __shared__ EvUnion E;
  __shared__ GridEv gr;
  __shared__ ProjEv pj[kMaxGroup];
  __shared__ ArmPat apc[kMaxGroup][2];
  __shared__ double red[kWarps][kMaxGroup * 3];
  const long long n = ev.n0 + blockIdx.x;
  if (n >= ev.N) return;
  block_load<MODEL>(E, pj[0], gr, g.rec[0], blockIdx.x);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nd = g.nd;
  if (tid < nd) {
    const int d = tid;
    if (d > 0) pj[d] = reinterpret_cast<const SetupHdr*>(g.rec[d] + (size_t)blockIdx.x * rec_stride<MODEL>())->pj;
    if (!EARTH) {
      TimeState ts;
      time_state(pj[d], pj[d].tc, ts);
      for (int a = 0; a < (g.det[d].shape == 1 ? 2 : 1); ++a) arm_pattern(pj[d], g.det[d].sin_zeta, ts.x, a, apc[d][a]);
    }
  }
  __syncthreads();
  double s[kMaxGroup][3];
#pragma unroll
  for (int d = 0; d < kMaxGroup; ++d) s[d][0] = s[d][1] = s[d][2] = 0.0;
  const int R = gr.ok ? gr.R : 0;
  for (int k = tid; k < R; k += kThreads) {
    double f, lnf, w;
    grid_point(gr, ev.spacing, k, f, lnf, w);
    double ap, ac, tau = 0.0;
    wave_point_val<MODEL, EARTH>(E, pj[0], f, lnf, ap, ac, tau);
    double ws = 0.0;
#pragma unroll
    for (int d = 0; d < kMaxGroup; ++d) {
      if (d >= nd) break;
      if (!(d > 0 && g.same_psd[d])) ws = w / psd_at(g.det[d], f, lnf);
      const bool tri = TRI && g.det[d].shape == 1;
      double Fp[2], Fc[2];
      if (EARTH) {
        TimeState ts;
        time_state(pj[d], pj[0].tc - tau / kDay, ts);
        for (int a = 0; a < (tri ? 2 : 1); ++a) {
          ArmPat p;
          arm_pattern(pj[d], g.det[d].sin_zeta, ts.x, a, p);
          Fp[a] = p.Fp;
          Fc[a] = p.Fc;
        }
      } else {
        for (int a = 0; a < (tri ? 2 : 1); ++a) { Fp[a] = apc[d][a].Fp; Fc[a] = apc[d][a].Fc; }
      }
      const double p1 = ap * Fp[0], c1 = ac * Fc[0];
      s[d][0] += ws * (p1 * p1 + c1 * c1);
      if (tri) {
        const double p2 = ap * Fp[1], c2 = ac * Fc[1];
        s[d][1] += ws * (p2 * p2 + c2 * c2);
        const double p3 = p1 + p2, c3 = c1 + c2;
        s[d][2] += ws * (p3 * p3 + c3 * c3);
      }
    }
  }
#pragma unroll
  for (int d = 0; d < kMaxGroup; ++d)
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      double v = s[d][a];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) red[warp][d * 3 + a] = v;
    }
  __syncthreads();
  if (tid == 0) {
    double tot = 0.0;
    for (int d = 0; d < nd; ++d) {
      const int na = g.det[d].shape == 1 ? 3 : 1;
      for (int a = 0; a < na; ++a) {
        double v = 0.0;
        for (int wp = 0; wp < kWarps; ++wp) v += red[wp][d * 3 + a];
        if (g.out_arm[d]) g.out_arm[d][(size_t)a * ev.N + n] = v;
        tot += 4.0 * v;
      }
    }
    if (out_det) out_det[n] = accum ? out_det[n] + tot : tot;
  }
}

// ------------------------------------------------------------------ FP32 SNR
// Per arm: scale * sum_k w_k / S_k (|h+|^2 F+^2 + |hx|^2 Fx^2) with the amplitudes, the pattern
// functions and the Earth-rotation time in FP32; each thread sums its points with Kahan compensation,
// the block sums in FP64. Outputs as snr_kernel. For the 22-mode models |h+| = A cp and |hx| = A ci;
// for IMRPhenomHM they are the moduli of the two mode sums, each mode phase evaluated in FP64 and
// reduced modulo 2 pi as in the FP32 Fisher kernel (only the values of wave_f32_hm are used; its
// tangent arithmetic is dead code here), and the h+ hx cross term is left out, as gwfast's
// GWAmplitudes does for higher modes (gwfast/signal.py:457-460).
template <int MODEL, bool EARTH, int NARM>
__global__ void __launch_bounds__(kThreads) snr_kernel_f32(EvBatch ev, DetDev det, const unsigned char* scratch32,
                                                           double* out_arm, double* out_det, int accum) {
  __shared__ F32Rec<MODEL> r;
  __shared__ double red[kWarps][3];
  const long long n = ev.n0 + blockIdx.x;
  if (n >= ev.N) return;
  {
    const uint4* src = reinterpret_cast<const uint4*>(scratch32 + (size_t)blockIdx.x * f32_stride<MODEL>());
    uint4* dst = reinterpret_cast<uint4*>(&r);
    for (int i = threadIdx.x; i < (int)(sizeof(F32Rec<MODEL>) / 16); i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int NA = NARM == 2 ? 3 : 1;
  float sum[NA], cmp[NA];
#pragma unroll
  for (int a = 0; a < NA; ++a) { sum[a] = 0.0f; cmp[a] = 0.0f; }
  const int R = r.gf.R;
  GridIterF grid;
  for (int base = 0; base < R; base += kThreads) {
    const int k = base + tid;
    grid.step(r, ev.spacing, base, lane, warp);
    if (k >= R) continue;
    float f, lnf, w;
    grid.point(r, ev.spacing, k, lane, f, lnf, w);
    const float ws = w / psd_at_f(det, f, lnf, r.gf.acc_l0, r.gf.acc_idl);
    float ap, ac;
    TimeF ts;
    if constexpr (MODEL == 2) {
      WaveF wv;
      wave_f32_hm<EARTH>(r.ef, r.pf, r.tf, f, lnf, wv);
      ap = sqrtf(wv.P.re * wv.P.re + wv.P.im * wv.P.im);
      ac = sqrtf(wv.C.re * wv.C.re + wv.C.im * wv.C.im);
      if (EARTH) time_f(r.pf, -wv.tau * (1.0f / 86400.0f), ts);
    } else {
      float A;
      if (MODEL == 0) {
        const float f13 = cbrtf(f);
        A = r.ef.tf2.ampK.v * (1.0f / (f * sqrtf(f13)));
        if (EARTH) time_f(r.pf, -tau_star_point<float>(r.ef.tf2.Ms, r.ef.tf2.vM, r.ef.tf2.eta, f13) * (1.0f / 86400.0f), ts);
      } else {
        A = phd_amp_point<float>(r.ef.phd, f);
        if (EARTH) time_f(r.pf, -tau_star_point<float>(r.ef.phd.Ms, r.ef.phd.vM, r.ef.phd.eta, cbrtf(f)) * (1.0f / 86400.0f), ts);
      }
      ap = A * r.pf.cp;
      ac = A * r.pf.ci;
    }
    float p[2], c[2];
#pragma unroll
    for (int a = 0; a < NARM; ++a) {
      ArmF pat;
      if (EARTH) arm_f(r.pf, ts, a, pat);
      else pat = r.apc[a];
      p[a] = ap * pat.Fp;
      c[a] = ac * pat.Fc;
    }
    float term[NA];
    term[0] = ws * (p[0] * p[0] + c[0] * c[0]);
    if (NARM == 2) {
      term[1] = ws * (p[1] * p[1] + c[1] * c[1]);
      const float p3 = p[0] + p[1], c3 = c[0] + c[1];
      term[2] = ws * (p3 * p3 + c3 * c3);
    }
#pragma unroll
    for (int a = 0; a < NA; ++a) {   // Kahan
      const float y = term[a] - cmp[a];
      const float t = sum[a] + y;
      cmp[a] = (t - sum[a]) - y;
      sum[a] = t;
    }
  }
#pragma unroll
  for (int a = 0; a < NA; ++a) {
    double v = (double)sum[a] - (double)cmp[a];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp][a] = v;
  }
  __syncthreads();
  if (tid == 0) {
    double tot = 0.0;
    for (int a = 0; a < NA; ++a) {
      double v = 0.0;
      for (int w = 0; w < kWarps; ++w) v += red[w][a];
      v *= r.scale;
      if (out_arm) out_arm[(size_t)a * ev.N + n] = v;
      tot += 4.0 * v;
    }
    if (out_det) out_det[n] = accum ? out_det[n] + tot : tot;
  }
}

// FP32 SNR of a group of detectors on one grid: the waveform value and the time to coalescence (and
// the Earth-rotation angle) once per point for the group, then each detector's pattern functions and
// PSD weight, as snr_kernel_f32 per detector. Detector d's projection comes from its FP32 record slot;
// its sums are scaled by its own amplitude^2 / PSD normalisation (detector 0's times sr[d]).
struct GroupSNR32 {
  DetDev det[kMaxGroup];
  double* out_arm[kMaxGroup];
  double sr[kMaxGroup];      // psd_scale of detector 0 / psd_scale of detector d
  int same_psd[kMaxGroup];
  int nd;
  long long slice;           // bytes between the FP32 record areas of consecutive detectors
};

template <int MODEL, bool EARTH, bool TRI>
__global__ void __launch_bounds__(kThreads) snr_group_kernel_f32(EvBatch ev, GroupSNR32 g, const unsigned char* scratch32,
                                                                 double* out_det, int accum) {
  __shared__ F32Rec<MODEL> r;
  __shared__ GroupProj gp;
  __shared__ double red[kWarps][kMaxGroup * 3];
  const long long n = ev.n0 + blockIdx.x;
  if (n >= ev.N) return;
  {
    const uint4* src = reinterpret_cast<const uint4*>(scratch32 + (size_t)blockIdx.x * f32_stride<MODEL>());
    uint4* dst = reinterpret_cast<uint4*>(&r);
    for (int i = threadIdx.x; i < (int)(sizeof(F32Rec<MODEL>) / 16); i += blockDim.x) dst[i] = src[i];
  }
  const int nd = g.nd;
  if ((int)threadIdx.x < nd) {
    const int d = threadIdx.x;
    const F32Rec<MODEL>& rd =
        *reinterpret_cast<const F32Rec<MODEL>*>(scratch32 + d * g.slice + (size_t)blockIdx.x * f32_stride<MODEL>());
    gp.pf[d] = rd.pf;
    gp.apc[d][0] = rd.apc[0];
    gp.apc[d][1] = rd.apc[1];
    gp.tsc[d] = rd.tsc;
  }
  __syncthreads();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  float sum[kMaxGroup][3], cmp[kMaxGroup][3];
#pragma unroll
  for (int d = 0; d < kMaxGroup; ++d)
#pragma unroll
    for (int a = 0; a < 3; ++a) sum[d][a] = cmp[d][a] = 0.0f;
  const int R = r.gf.R;
  GridIterF grid;
  for (int base = 0; base < R; base += kThreads) {
    const int k = base + tid;
    grid.step(r, ev.spacing, base, lane, warp);
    if (k >= R) continue;
    float f, lnf, w;
    grid.point(r, ev.spacing, k, lane, f, lnf, w);
    float ap, ac, tau = 0.0f;
    if constexpr (MODEL == 2) {
      WaveF wv;
      wave_f32_hm<EARTH>(r.ef, r.pf, r.tf, f, lnf, wv);
      ap = sqrtf(wv.P.re * wv.P.re + wv.P.im * wv.P.im);
      ac = sqrtf(wv.C.re * wv.C.re + wv.C.im * wv.C.im);
      tau = wv.tau;
    } else {
      float A;
      if (MODEL == 0) {
        const float f13 = cbrtf(f);
        A = r.ef.tf2.ampK.v * (1.0f / (f * sqrtf(f13)));
        if (EARTH) tau = tau_star_point<float>(r.ef.tf2.Ms, r.ef.tf2.vM, r.ef.tf2.eta, f13);
      } else {
        A = phd_amp_point<float>(r.ef.phd, f);
        if (EARTH) tau = tau_star_point<float>(r.ef.phd.Ms, r.ef.phd.vM, r.ef.phd.eta, cbrtf(f));
      }
      ap = A * r.pf.cp;
      ac = A * r.pf.ci;
    }
    float sd = 0.0f, cd = 1.0f;   // the Earth-rotation angle is the same for every detector
    if (EARTH) rot_sc_tau(tau, sd, cd);
    float ws = 0.0f;
#pragma unroll
    for (int d = 0; d < kMaxGroup; ++d) {
      if (d >= nd) break;
      const DetDev& det = g.det[d];
      if (!(d > 0 && g.same_psd[d])) ws = w / psd_at_f(det, f, lnf, (float)det.acc_l0, (float)det.acc_idl);
      const bool tri = TRI && det.shape == 1;
      TimeF ts;
      if (EARTH) time_f_rot(gp.pf[d], sd, cd, ts);
      float p[2], c[2];
      for (int a = 0; a < (tri ? 2 : 1); ++a) {
        ArmF pat;
        if (EARTH) arm_f(gp.pf[d], ts, a, pat);
        else pat = gp.apc[d][a];
        p[a] = ap * pat.Fp;
        c[a] = ac * pat.Fc;
      }
      float term[3];
      term[0] = ws * (p[0] * p[0] + c[0] * c[0]);
      term[1] = term[2] = 0.0f;
      if (tri) {
        term[1] = ws * (p[1] * p[1] + c[1] * c[1]);
        const float p3 = p[0] + p[1], c3 = c[0] + c[1];
        term[2] = ws * (p3 * p3 + c3 * c3);
      }
#pragma unroll
      for (int a = 0; a < 3; ++a) {   // Kahan
        const float y = term[a] - cmp[d][a];
        const float t = sum[d][a] + y;
        cmp[d][a] = (t - sum[d][a]) - y;
        sum[d][a] = t;
      }
    }
  }
#pragma unroll
  for (int d = 0; d < kMaxGroup; ++d)
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      double v = (double)sum[d][a] - (double)cmp[d][a];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) red[warp][d * 3 + a] = v;
    }
  __syncthreads();
  if (tid == 0) {
    double tot = 0.0;
    for (int d = 0; d < nd; ++d) {
      const int na = g.det[d].shape == 1 ? 3 : 1;
      const double sc = r.scale * g.sr[d];
      for (int a = 0; a < na; ++a) {
        double v = 0.0;
        for (int wp = 0; wp < kWarps; ++wp) v += red[wp][d * 3 + a];
        v *= sc;
        if (g.out_arm[d]) g.out_arm[d][(size_t)a * ev.N + n] = v;
        tot += 4.0 * v;
      }
    }
    if (out_det) out_det[n] = accum ? out_det[n] + tot : tot;
  }
}

}  // namespace gwf
