// Waveform models on the device: TaylorF2_RestrictedPN, IMRPhenomD, IMRPhenomHM.
//
// Per event, a setup routine evaluates every parameter-dependent coefficient as a
// Dual<double, 4> (value + d/d{Mc, eta, chi1z, chi2z}); per frequency point the
// routines below are templated on the scalar S (plain T for the SNR, Dual<T, 4>
// for the Fisher tangent).  Formulas follow gwfast 1.1.2 (citations per routine);
// the IMRPhenomD intermediate amplitude is evaluated in Newton-Hermite form (the
// same quartic that gwfast writes out as delta_0..delta_4).
#pragma once
#include "gwf_consts.cuh"

namespace gwf {

using D4 = Dual<double, 4>;
enum { P_MC = 0, P_ETA = 1, P_CHI1 = 2, P_CHI2 = 3, P_LT = 4, P_DLT = 5 };   // tangent slots (4, 5: tidal model)
using D6 = Dual<double, 6>;   // IMRPhenomD_NRTidalv2: the tidal parameters enter the set-up non-linearly

// coefficient access: per-event coefficients are stored as duals (D4 for FP64, DF4 for FP32);
// a per-point scalar S of matching precision reads either the full dual or its value.
using DF4 = Dual<float, 4>;
template <class S, class C> struct CoT;
template <class U, int N> struct CoT<U, Dual<U, N>> {
  __device__ __forceinline__ static U get(const Dual<U, N>& c) { return c.v; }
};
template <class U, int N> struct CoT<Dual<U, N>, Dual<U, N>> {
  __device__ __forceinline__ static Dual<U, N> get(const Dual<U, N>& c) { return c; }
};
template <> struct CoT<double, double> { __device__ __forceinline__ static double get(double c) { return c; } };
template <class S, class C> __device__ __forceinline__ S co(const C& c) { return CoT<S, C>::get(c); }

template <class S> struct Real;
template <> struct Real<double> { typedef double T; };
template <> struct Real<float> { typedef float T; };
template <class U, int N> struct Real<Dual<U, N>> { typedef U T; };

template <class D>
__device__ __forceinline__ D seta_of(const D& eta) {
  // sqrt(1-4 eta) guarded at equal mass (gwfast/waveforms.py:759)
  return eta.v < 0.25 ? dsqrt(1.0 - 4.0 * eta) : D(0.0);
}

// ------------------------------------------------------------------ PN phase coefficients
template <class C> struct PNCT { C A, c2, c3, c4, c5, c5l, c6, c6l, c7; };
using PNC = PNCT<D4>;

// TaylorF2 coefficients, gwfast/waveforms.py:784-812; drop_ss removes the 3PN spin-spin part as
// IMRPhenomD does (gwfast/waveforms.py:1077). dq1, dq2: spin-induced quadrupole moments minus 1
// (zero for black holes), as IMRPhenomD_NRTidalv2 (gwfast/waveforms.py:1461-1467) and TaylorF2 with
// use_QuadMonTid (:794-806) use them.
template <class D>
__device__ inline PNCT<D> pn_coeffs(const D& eta, const D& chi1, const D& chi2, bool spin_ho, bool drop_ss,
                                    const D& dq1 = D(0.0), const D& dq2 = D(0.0)) {
  const D seta = seta_of(eta);
  const D m1 = 0.5 * (1.0 + seta), m2 = 0.5 * (1.0 - seta);
  const D chis = 0.5 * (chi1 + chi2), chia = 0.5 * (chi1 - chi2);
  const D eta2 = eta * eta;
  PNCT<D> c;
  c.A = 3.0 / (128.0 * eta);
  c.c2 = 3715. / 756. + 55. / 9. * eta;
  c.c3 = -16. * kPi + (113. / 3.) * seta * chia + (113. / 3. - 76. / 3. * eta) * chis;
  const D m1s = m1 * m1 * chi1 * chi1, m2s = m2 * m2 * chi2 * chi2;
  c.c4 = 5. / 72. * (3058.673 / 7.056 + 5429. / 7. * eta + 617. * eta2) + ((247. - 721.) / 4.8) * eta * chi1 * chi2
         + ((-720. + 1. + 240. - 7.) / 9.6) * (m1s + m2s);
  // spin-induced quadrupole moments QuadMon_i = 1 + dq_i (tidal models, gwfast/waveforms.py:1461)
  c.c4 = c.c4 - 50.0 * (dq1 * m1s + dq2 * m2s);
  const D t5 = (732985. / 2268. - 24260. / 81. * eta - 340. / 9. * eta2) * chis
                + (732985. / 2268. + 140. / 9. * eta) * seta * chia;
  c.c5 = 38645. * kPi / 756. - 65. * kPi / 9. * eta - t5;
  c.c5l = 3.0 * c.c5;
  D six = 11583.231236531 / 4.694215680 - 640. / 3. * kPi * kPi - 684.8 / 2.1 * kEulerGamma
           + (-15737.765635 / 3.048192 + 225.5 / 1.2 * kPi * kPi) * eta + 76.055 / 1.728 * eta2
           - 127.825 / 1.296 * eta2 * eta - log(4.0) * (684.8 / 2.1)
           + kPi * chi1 * m1 * (1490. / 3. + 260. * m1) + kPi * chi2 * m2 * (1490. / 3. + 260. * m2);
  // the quadrupole excess of the 3PN spin-spin terms (:806, :1464-1467; zero for black holes)
  six = six + (4703.5 / 8.4 + 2935. / 6. * m1 - 120. * m1 * m1) * m1s * dq1
            + (4703.5 / 8.4 + 2935. / 6. * m2 - 120. * m2 * m2) * m2s * dq2;
  if (!drop_ss) {
    const D ss1 = (4703.5 / 8.4 - 4108.25 / 6.72) + (2935. / 6. - 108.5 / 1.2) * m1 + (125.5 / 3.6 - 120.) * m1 * m1;
    const D ss2 = (4703.5 / 8.4 - 4108.25 / 6.72) + (2935. / 6. - 108.5 / 1.2) * m2 + (125.5 / 3.6 - 120.) * m2 * m2;
    six = six + (326.75 / 1.12 + 557.5 / 1.8 * eta) * eta * chi1 * chi2 + ss1 * m1s + ss2 * m2s;
  }
  c.c6 = six;
  c.c6l = D(-6848. / 21.);
  D sev = 77096675. * kPi / 254016. + 378515. * kPi / 1512. * eta - 74045. * kPi / 756. * eta2;
  D cs = -25150083775. / 3048192. + 10566655595. / 762048. * eta - 1042165. / 3024. * eta2 + 5345. / 36. * eta2 * eta;
  D ca = -25150083775. / 3048192. + 26804935. / 6048. * eta - 1985. / 48. * eta2;
  if (spin_ho) {
    cs = cs + (14585. / 8. - 7270. * eta + 80. * eta2) * chia * chia;
    sev = sev + (14585. / 24. - 475. / 6. * eta + 100. / 3. * eta2) * chis * chis * chis
          + seta * ((14585. / 24. - 2380. * eta) * chia * chia * chia + (14585. / 8. - 107.5 * eta) * chia * chis * chis);
  }
  c.c7 = sev + cs * chis + seta * ca * chia;
  return c;
}

// ------------------------------------------------------------------ TaylorF2 (gwfast/waveforms.py:697-953)
template <class C> struct TF2EvT {
  PNCT<C> pn;
  C eta;
  C Ms;      // total mass in seconds
  C vM;      // (pi Ms)^(1/3)
  C lnvM;
  C ampK;    // amplitude without f^(-7/6)
};
using TF2Ev = TF2EvT<D4>;

// TaylorF2 options (WfDesc::flags): phase referenced at the last stable orbit, cut at twice the Kerr
// ISCO, spin-induced quadrupole moments from the tidal deformabilities
enum { kTF2Vlso = 1, kTF2KerrIsco = 2, kTF2QuadMon = 4 };

__device__ inline void tf2_setup(TF2Ev& e, const D4& Mc, const D4& eta, const D4& chi1, const D4& chi2, double dL,
                                 bool spin_ho, int flags = 0, const D4& dq1 = D4(0.0), const D4& dq2 = D4(0.0)) {
  e.pn = pn_coeffs(eta, chi1, chi2, spin_ho, false, dq1, dq2);
  // phiref_vlso: the 2.5PN constant times (1 - 3 ln v_lso), v_lso = 1/sqrt(6) (gwfast/waveforms.py:816-818);
  // its log partner keeps the plain coefficient
  if (flags & kTF2Vlso) e.pn.c5 = e.pn.c5 * (1.0 + 1.5 * log(6.0));
  e.eta = eta;
  e.Ms = Mc * kG3 / dpowc(eta, 0.6);
  e.vM = dcbrt(kPi * e.Ms);
  e.lnvM = dlog(e.vM);
  // sqrt(5/24) pi^(-2/3) c/dL (G Mc)^(5/6)  (gwfast/waveforms.py:875)
  e.ampK = (sqrt(5.0 / 24.0) * pow(kPi, -2.0 / 3.0) * kCGpc / dL) * dpowc(kG3 * Mc, 5.0 / 6.0);
}

// TaylorF2 with the tidal terms (gwfast/waveforms.py:849-855, PhysRevD.89.103012): the phase
// series gains (-39/2 LambdaTilde) v^10 + (-3115/64 LambdaTilde + 6595/364 sqrt(1-4 eta) deltaLambda) v^12.
// LambdaTilde and deltaLambda are Fisher parameters of their own (their tangents are formed
// analytically per point); the coefficients carry the eta tangent of sqrt(1 - 4 eta).
template <class C> struct TF2TEvT {
  TF2EvT<C> b;
  C t10, t12;   // series coefficients of v^10 and v^12
  C s12;        // d t12 / d deltaLambda
  // use_QuadMonTid: d c4 / d LambdaTilde, d c4 / d deltaLambda, d c6 / d LambdaTilde, d c6 / d deltaLambda
  // (the quadrupole moments follow Lambda1, Lambda2); zero otherwise
  double q4l, q4d, q6l, q6d;
};
using TF2TEv = TF2TEvT<D4>;

template <class D> __device__ inline void lam12_of(const D& lt, const D& dlt, const D& eta, D& l1, D& l2);
template <class D> __device__ inline D quad_mon(const D& lam);

__device__ inline void tf2t_setup(TF2TEv& e, const D4& Mc, const D4& eta, const D4& chi1, const D4& chi2, double dL,
                                  bool spin_ho, double lam_t, double del_lam, int flags = 0) {
  e.q4l = e.q4d = e.q6l = e.q6d = 0.0;
  if (flags & kTF2QuadMon) {
    // quadrupole moments with their eta tangent (Lambda1, Lambda2 depend on eta at fixed LambdaTilde,
    // deltaLambda), then their tangents in (LambdaTilde, deltaLambda) for the analytic columns
    D4 l1, l2;
    lam12_of(D4(lam_t), D4(del_lam), eta, l1, l2);
    const D4 q1 = quad_mon(l1), q2 = quad_mon(l2);
    tf2_setup(e.b, Mc, eta, chi1, chi2, dL, spin_ho, flags, q1 - 1.0, q2 - 1.0);
    typedef Dual<double, 2> D2;
    D2 k1, k2;
    lam12_of(D2::seed(lam_t, 0), D2::seed(del_lam, 1), D2(eta.v), k1, k2);
    const D2 r1 = quad_mon(k1), r2 = quad_mon(k2);
    const double sv = eta.v < 0.25 ? sqrt(1.0 - 4.0 * eta.v) : 0.0;
    const double m1 = 0.5 * (1.0 + sv), m2 = 0.5 * (1.0 - sv);
    const double a1 = m1 * m1 * chi1.v * chi1.v, a2 = m2 * m2 * chi2.v * chi2.v;
    const double b1 = (4703.5 / 8.4 + 2935. / 6. * m1 - 120. * m1 * m1) * a1;
    const double b2 = (4703.5 / 8.4 + 2935. / 6. * m2 - 120. * m2 * m2) * a2;
    e.q4l = -50.0 * (a1 * r1.d[0] + a2 * r2.d[0]);
    e.q4d = -50.0 * (a1 * r1.d[1] + a2 * r2.d[1]);
    e.q6l = b1 * r1.d[0] + b2 * r2.d[0];
    e.q6d = b1 * r1.d[1] + b2 * r2.d[1];
  } else {
    tf2_setup(e.b, Mc, eta, chi1, chi2, dL, spin_ho, flags);
  }
  e.t10 = D4(-19.5 * lam_t);
  e.s12 = (6595.0 / 364.0) * seta_of(eta);
  e.t12 = (-3115.0 / 64.0) * lam_t + e.s12 * del_lam;
}

// eccentric TaylorF2 (gwfast/waveforms.py:814-845; low-eccentricity phase to 3PN, arXiv:1605.00304):
// the series gains K e0^2 (v0/v)^(19/3) S(v, v0), K = -2355/1462, with v0 = (pi M f0)^(1/3) at the
// eccentricity's reference frequency f0 (the lowest grid frequency unless fRef_ecc is given). Written
// as a polynomial in v, S = s0 + s2 v^2 + ... + s6 v^6 + sl ln(16 v^2) v^6, whose coefficients depend on
// v0 and eta; (v0/v)^(19/3) = (f0/f)^(19/9) carries no parameter. Stored already multiplied by
// A K e0^2 (A = 3/(128 eta)). With f0 the lowest grid frequency the record depends on the detector.
template <class C> struct TF2EEvT {
  TF2TEvT<C> t;   // tidal part zero without the tidal terms
  C es[6];        // A K e0^2 times s0, s2, s3, s4, s5, s6
  C el;           // A K e0^2 times the ln(16 v^2) v^6 coefficient
  double ecc, lnf0;
};
using TF2EEv = TF2EEvT<D4>;

__device__ inline void tf2e_ref(TF2EEv& e, double fmin_hz, double fref_ecc) {
  const double f0 = fref_ecc > 0.0 ? fref_ecc : fmin_hz;
  e.lnf0 = log(f0);
  const D4& eta = e.t.b.eta;
  const D4 eta2 = eta * eta, eta3 = eta2 * eta;
  const D4 v0 = e.t.b.vM * exp(e.lnf0 / 3.0);
  const D4 w2 = v0 * v0, w3 = w2 * v0, w4 = w2 * w2, w5 = w4 * v0, w6 = w3 * w3;
  const D4 lw = log(16.0) + 2.0 * dlog(v0);   // ln(16 v0^2)
  const double pi2 = kPi * kPi, l2 = log(2.0), l3 = log(3.0);
  const D4 twoV = 29.9076223 / 8.1976608 + 18.766963 / 2.927736 * eta;
  const D4 twoV0 = 2.833 / 1.008 - 19.7 / 3.6 * eta;
  const double threeV = -28.19123 / 2.82600 * kPi, threeV0 = 37.7 / 7.2 * kPi;
  const D4 fourV4 = 16.237683263 / 3.330429696 + 241.33060753 / 9.71375328 * eta + 156.2608261 / 6.9383952 * eta2;
  const D4 fourV2V02 = 84.7282939759 / 8.2632420864 - 7.18901219 / 3.68894736 * eta - 36.97091711 / 1.05398496 * eta2;
  const D4 fourV04 = -1.193251 / 3.048192 - 66.317 / 9.072 * eta + 18.155 / 1.296 * eta2;
  const D4 fiveV5 = kPi * (-28.31492681 / 1.18395270 - 115.52066831 / 2.70617760 * eta);
  const D4 fiveV3V02 = kPi * (-79.86575459 / 2.84860800 + 55.5367231 / 1.0173600 * eta);
  const D4 fiveV2V03 = kPi * (112.751736071 / 5.902315776 + 70.75145051 / 2.10796992 * eta);
  const D4 fiveV05 = kPi * (76.4881 / 9.0720 - 94.9457 / 2.2680 * eta);
  const D4 sixV6 = -436.03153867072577087 / 1.32658535116800000 + 53.6803271 / 1.9782000 * kEulerGamma
                   + 157.22503703 / 3.25555200 * pi2 + (2991.72861614477 / 6.89135247360 - 15.075413 / 1.446912 * pi2) * eta
                   + 345.5209264991 / 4.1019955200 * eta2 + 506.12671711 / 8.78999040 * eta3
                   + 384.3505163 / 5.9346000 * l2 - 112.1397129 / 1.7584000 * l3;
  const D4 sixV4V02 = 46.001356684079 / 3.357073133568 + 253.471410141755 / 5.874877983744 * eta
                      - 169.3852244423 / 2.3313007872 * eta2 - 307.833827417 / 2.497822272 * eta3;
  const double sixV3V03 = -106.2809371 / 2.0347200 * pi2;
  const D4 sixV2V04 = -3.56873002170973 / 2.49880440692736 - 260.399751935005 / 8.924301453312 * eta
                      + 15.0484695827 / 3.5413894656 * eta2 + 340.714213265 / 3.794345856 * eta3;
  const D4 sixV06 = 265.31900578691 / 1.68991764480 - 33.17 / 1.26 * kEulerGamma + 12.2833 / 1.0368 * pi2
                    + (91.55185261 / 5.48674560 - 3.977 / 1.152 * pi2) * eta - 5.732473 / 1.306368 * eta2
                    - 30.90307 / 1.39968 * eta3 + 87.419 / 1.890 * l2 - 260.01 / 5.60 * l3;
  const D4 pre = e.t.b.pn.A * ((-2.355 / 1.462) * e.ecc * e.ecc);
  e.es[0] = pre * (1.0 + twoV0 * w2 + threeV0 * w3 + fourV04 * w4 + fiveV05 * w5 + (sixV06 - 33.17 / 2.52 * lw) * w6);
  e.es[1] = pre * (twoV + fourV2V02 * w2 + fiveV2V03 * w3 + sixV2V04 * w4);
  e.es[2] = pre * (threeV + fiveV3V02 * w2 + sixV3V03 * w3);
  e.es[3] = pre * (fourV4 + sixV4V02 * w2);
  e.es[4] = pre * fiveV5;
  e.es[5] = pre * sixV6;
  e.el = pre * (53.6803271 / 3.9564000);
}

__device__ inline void tf2e_setup(TF2EEv& e, const D4& Mc, const D4& eta, const D4& chi1, const D4& chi2, double dL,
                                  bool spin_ho, double lam_t, double del_lam, int flags, double ecc, double fmin_hz,
                                  double fref_ecc) {
  tf2t_setup(e.t, Mc, eta, chi1, chi2, dL, spin_ho, lam_t, del_lam, flags);
  e.ecc = ecc;
  tf2e_ref(e, fmin_hz, fref_ecc);
}

// eccentric part of the phase, (f0/f)^(19/9) S(v) / v^5, at v = (pi M f)^(1/3), ln v = lnv
template <class S, class C>
__device__ __forceinline__ S tf2_ecc_phase(const TF2EEvT<C>& e, const S& v, const S& lnv, typename Real<S>::T lnf) {
  typedef typename Real<S>::T T;
  const S v2 = v * v, v3 = v2 * v;
  const S ser = co<S>(e.es[0])
                + v2 * (co<S>(e.es[1]) + v * (co<S>(e.es[2]) + v * (co<S>(e.es[3]) + v * (co<S>(e.es[4]) + v * co<S>(e.es[5])))))
                + co<S>(e.el) * (T(log(16.0)) + T(2) * lnv) * v3 * v3;
  return ser * (exp(T(19.0 / 9.0) * (T(e.lnf0) - lnf)) / (v2 * v3));
}

// the tidal part of the phase, A (t10 v^10 + t12 v^12) / v^5, at v = (pi M f)^(1/3)
template <class S, class C>
__device__ __forceinline__ S tf2_tidal_phase(const TF2TEvT<C>& e, const S& v) {
  const S v2 = v * v;
  return co<S>(e.b.pn.A) * (v2 * v2 * v) * (co<S>(e.t10) + co<S>(e.t12) * v2);
}

// TF2 phase (without the constant offset, which cancels in every output) and amplitude.
template <class S, class C>
__device__ __forceinline__ void tf2_point(const TF2EvT<C>& e, typename Real<S>::T f, typename Real<S>::T f13,
                                          typename Real<S>::T lnf, typename Real<S>::T fm76, S& amp, S& phase) {
  typedef typename Real<S>::T T;
  const S v = co<S>(e.vM) * f13;
  const S lnv = co<S>(e.lnvM) + lnf * T(1.0 / 3.0);
  const S v2 = v * v;
  const S v3 = v2 * v;
  const S ser = T(1) + co<S>(e.pn.c2) * v2 + co<S>(e.pn.c3) * v3 + co<S>(e.pn.c4) * v2 * v2
                + (co<S>(e.pn.c5) + co<S>(e.pn.c5l) * lnv) * v2 * v3
                + (co<S>(e.pn.c6) + co<S>(e.pn.c6l) * lnv) * v3 * v3 + co<S>(e.pn.c7) * v3 * v3 * v;
  phase = co<S>(e.pn.A) * ser / (v2 * v3);
  amp = co<S>(e.ampK) * fm76;
}

// 3.5PN time to coalescence shared by the three models (gwfast/waveforms.py:878-901, :1299-1322, :2712-2735)
template <class S, class C>
__device__ __forceinline__ S tau_star_point(const C& Ms, const C& vM, const C& eta_, typename Real<S>::T f13) {
  typedef typename Real<S>::T T;
  const S eta = co<S>(eta_);
  const S v = co<S>(vM) * f13;
  const S v2 = v * v;
  const S v4 = v2 * v2;
  const S eta2 = eta * eta;
  const S pre = T(5.0 / 256.0) * co<S>(Ms) / (eta * v4 * v4);
  const S t05 = T(1) + (T(743. / 252.) + T(11. / 3.) * eta) * v2 - T(32. / 5. * kPi) * v2 * v
                + (T(3058673. / 508032.) + T(5429. / 504.) * eta + T(617. / 72.) * eta2) * v4
                - (T(7729. / 252.) - T(13. / 3.) * eta) * T(kPi) * v4 * v;
  const S t6 = (T(-10052469856691. / 23471078400. + 128. / 3. * kPi * kPi + 6848. / 105. * kEulerGamma)
                + (T(3147553127. / 3048192. - 451. / 12. * kPi * kPi)) * eta - T(15211. / 1728.) * eta2
                + T(25565. / 1296.) * eta2 * eta + T(3424. / 105.) * dlog(T(16) * v2)) * v4 * v2;
  const S t7 = (T(-15419335. / 127008.) - T(75703. / 756.) * eta + T(14809. / 378.) * eta2) * T(kPi) * v4 * v2 * v;
  return pre * (t05 + t6 + t7);
}

// Per-event coefficients of the FP64 Fisher kernels' point evaluation (TaylorF2, IMRPhenomD), formed
// in the CTA prologue so that a point costs a few FMAs instead of four-direction dual arithmetic.
// tau_star: the polynomial above, tau = T0 v^-8 P(v), T0 = (5/256) Ms / eta, v = vM f^(1/3),
// P(v) = 1 + sum_{k=2..7} a_k v^k (a_6 with its a6l ln(16 v^2) part); the parameters enter only
// through Ms, eta and vM, and v's tangent is v d ln vM, so
//   d tau = tau d ln T0 + T0 v^-8 [(v P' - 8 P) d ln vM + (dP/deta) d eta].
// IMRPhenomD's inspiral amplitude (phd_amp_d): the log-derivatives of its prefactor and of MG.
struct TauD {
  double T0, lg0;        // (5/256) Ms / eta; ln 16 + 2 ln vM (ln(16 v^2) = lg0 + 2/3 ln f)
  double vM;
  double a[6], b[6];     // a_2..a_7 (a_6 without its log term) and their eta derivatives
  double dlnT0[4], dlnv[4], deta[4];
  double dlnP[4], dlnMG[4];   // d ln ampPref, d ln MG (IMRPhenomD)
};
constexpr double kTauA6ld = 3424.0 / 105.0;

__device__ inline void tau_setup_d(TauD& t, const D4& Ms, const D4& vM, const D4& eta_) {
  const double eta = eta_.v, e2 = eta * eta;
  t.a[0] = 743. / 252. + 11. / 3. * eta;
  t.a[1] = -32. / 5. * kPi;
  t.a[2] = 3058673. / 508032. + 5429. / 504. * eta + 617. / 72. * e2;
  t.a[3] = -(7729. / 252. - 13. / 3. * eta) * kPi;
  t.a[4] = -10052469856691. / 23471078400. + 128. / 3. * kPi * kPi + 6848. / 105. * kEulerGamma
           + (3147553127. / 3048192. - 451. / 12. * kPi * kPi) * eta - 15211. / 1728. * e2 + 25565. / 1296. * e2 * eta;
  t.a[5] = (-15419335. / 127008. - 75703. / 756. * eta + 14809. / 378. * e2) * kPi;
  t.b[0] = 11. / 3.;
  t.b[1] = 0.0;
  t.b[2] = 5429. / 504. + 2. * 617. / 72. * eta;
  t.b[3] = 13. / 3. * kPi;
  t.b[4] = 3147553127. / 3048192. - 451. / 12. * kPi * kPi - 2. * 15211. / 1728. * eta + 3. * 25565. / 1296. * e2;
  t.b[5] = (-75703. / 756. + 2. * 14809. / 378. * eta) * kPi;
  t.T0 = 5.0 / 256.0 * Ms.v / eta;
  t.vM = vM.v;
  t.lg0 = log(16.0) + 2.0 * log(vM.v);
  const double ims = 1.0 / Ms.v, ieta = 1.0 / eta, ivm = 1.0 / vM.v;
  for (int q = 0; q < 4; ++q) {
    t.dlnT0[q] = Ms.d[q] * ims - eta_.d[q] * ieta;
    t.dlnv[q] = vM.d[q] * ivm;
    t.deta[q] = eta_.d[q];
  }
}

// the amplitude part of TauD (IMRPhenomD)
__device__ inline void amp_setup_d(TauD& t, const D4& ampPref, const D4& MG) {
  const double ip = 1.0 / ampPref.v, img = 1.0 / MG.v;
  for (int q = 0; q < 4; ++q) {
    t.dlnP[q] = ampPref.d[q] * ip;
    t.dlnMG[q] = MG.d[q] * img;
  }
}

// tau_star (s) and its tangent at f^(1/3) = f13, ln f = lnf
__device__ __forceinline__ D4 tau_point_d(const TauD& t, double f13, double lnf) {
  const double v = t.vM * f13, v2 = v * v;
  const double iv = 1.0 / v, iv2 = iv * iv, iv4 = iv2 * iv2;
  const double lg = fma(lnf, 2.0 / 3.0, t.lg0);
  const double a6e = fma(kTauA6ld, lg, t.a[4]);
  // (P - 1) / v^2, v P' / v^2 and (dP/deta) / v^2 by Horner from v^5 down
  double p = t.a[5], dp = 7.0 * t.a[5], q = t.b[5];
  p = fma(p, v, a6e);  dp = fma(dp, v, fma(6.0, a6e, 2.0 * kTauA6ld));  q = fma(q, v, t.b[4]);
  p = fma(p, v, t.a[3]);  dp = fma(dp, v, 5.0 * t.a[3]);  q = fma(q, v, t.b[3]);
  p = fma(p, v, t.a[2]);  dp = fma(dp, v, 4.0 * t.a[2]);  q = fma(q, v, t.b[2]);
  p = fma(p, v, t.a[1]);  dp = fma(dp, v, 3.0 * t.a[1]);  q = fma(q, v, t.b[1]);
  p = fma(p, v, t.a[0]);  dp = fma(dp, v, 2.0 * t.a[0]);  q = fma(q, v, t.b[0]);
  const double P = fma(p, v2, 1.0);
  const double c = t.T0 * iv4 * iv4;
  D4 r;
  r.v = c * P;
  const double gv = c * fma(dp, v2, -8.0 * P), ge = c * q * v2;
#pragma unroll
  for (int k = 0; k < 4; ++k) r.d[k] = fma(r.v, t.dlnT0[k], fma(gv, t.dlnv[k], ge * t.deta[k]));
  return r;
}

// ------------------------------------------------------------------ IMRPhenomD core
template <class C> struct PhdCoreT {
  C eta, MG, Ms, vM;      // MG = M * G/c^3 (s); Ms = MG; vM = (pi MG)^(1/3) for tau_star
  C fring, fdamp;
  PNCT<C> pn;
  C sig[4], bet[3], alp[5], gam[3];
  C C1Int, C2Int, fMRD, PhiIntTemp, DPhiIntTemp, C1MRD, C2MRD;
  C a23, a1, a43, a53, a2, r1, r2, r3;    // inspiral amplitude
  C fpA;                                  // amplitude peak (gwfast/waveforms.py:1193)
  C f2;                                   // middle collocation node
  C h0, h1, h2, h3, h4;                   // Newton-Hermite coefficients of the intermediate amplitude
  C ampPref;                              // Overallamp * amp0 (model-dependent normalisation)
  C t0;
  C fRef, phiRef;                         // detector-dependent (fRef = M G fmin)
};
using PhdCore = PhdCoreT<D4>;

template <class D>
__device__ __forceinline__ D fit11(int k, const D& eta, const D& xi) {
  const double* c = kFits[k];
  const D e2 = eta * eta;
  return c[0] + c[1] * eta + (c[2] + c[3] * eta + c[4] * e2 + (c[5] + c[6] * eta + c[7] * e2) * xi
                              + (c[8] + c[9] * eta + c[10] * e2) * xi * xi) * xi;
}

// The same fit on duals. It depends on the parameters only through eta and xi, so the value and
// the two partial derivatives are formed in plain arithmetic and the N tangents by the chain rule
// at the end: ~30 FP64 operations instead of ~110 of dual arithmetic. The per-event set-up is bound
// by the FP64 pipe and evaluates 19 of these fits per event.
template <class T, int N>
__device__ __forceinline__ Dual<T, N> fit11(int k, const Dual<T, N>& eta, const Dual<T, N>& xi) {
  const double* c = kFits[k];
  const T e = eta.v, x = xi.v, e2 = e * e;
  const T A = c[2] + c[3] * e + c[4] * e2, B = c[5] + c[6] * e + c[7] * e2, C = c[8] + c[9] * e + c[10] * e2;
  Dual<T, N> r;
  r.v = c[0] + c[1] * e + (A + B * x + C * x * x) * x;
  // d/deta and d/dxi of c0 + c1 e + (A + B x + C x^2) x
  const T fe = c[1] + ((c[3] + 2.0 * c[4] * e) + ((c[6] + 2.0 * c[7] * e) + (c[9] + 2.0 * c[10] * e) * x) * x) * x;
  const T fx = A + (2.0 * B + 3.0 * C * x) * x;
#pragma unroll
  for (int q = 0; q < N; ++q) r.d[q] = fe * eta.d[q] + fx * xi.d[q];
  return r;
}

// final spin (gwfast/waveforms.py:1256-1276) and radiated energy (:1278-1297)
template <class D>
__device__ inline D final_spin(const D& eta, const D& chi1, const D& chi2) {
  const D seta = seta_of(eta);
  const D m1 = 0.5 * (1.0 + seta), m2 = 0.5 * (1.0 - seta);
  const D s = m1 * m1 * chi1 + m2 * m2 * chi2;
  const D e2 = eta * eta;
  return eta * (3.4641016151377544 - 4.399247300629289 * eta + 9.397292189321194 * e2 - 13.180949901606242 * e2 * eta)
         + eta * (s * ((1.0 / eta - 0.0850917821418767 - 5.837029316602263 * eta) + (0.1014665242971878 - 2.0967746996832157 * eta) * s))
         + eta * (s * ((-1.3546806617824356 + 4.108962025369336 * eta) * s * s + (-0.8676969352555539 + 2.064046835273906 * eta) * s * s * s));
}
template <class D>
__device__ inline D radiated_energy(const D& eta, const D& chi1, const D& chi2) {
  const D seta = seta_of(eta);
  const D m1 = 0.5 * (1.0 + seta), m2 = 0.5 * (1.0 - seta);
  const D s = (m1 * m1 * chi1 + m2 * m2 * chi2) / (m1 * m1 + m2 * m2);
  const D e2 = eta * eta;
  const D ens = eta * (0.055974469826360077 + 0.5809510763115132 * eta - 0.9606726679372312 * e2 + 3.352411249771192 * e2 * eta);
  return ens * (1. + (-0.0030302335878845507 - 2.0066110851351073 * eta + 7.7050567802399215 * e2) * s)
         / (1. + (-0.6714403054720589 - 1.4756929437702908 * eta + 7.304676214885011 * e2) * s);
}

// ---- phase pieces (argument x = M f), gwfast/waveforms.py:1079-1153, :2497-2501
template <class S, class C>
__device__ __forceinline__ S ins_phase(const PhdCoreT<C>& k, const S& x) {
  typedef typename Real<S>::T T;
  const S xp = T(kPi) * x;
  const S x13 = dcbrt(xp);
  const S ix13 = T(1) / x13;
  const S ix23 = ix13 * ix13;
  const S lx = dlog(xp) * T(1.0 / 3.0);
  const S tf2 = ix23 / xp + co<S>(k.pn.c2) / xp + co<S>(k.pn.c3) * ix23 + co<S>(k.pn.c4) * ix13 + co<S>(k.pn.c5)
                + co<S>(k.pn.c5l) * lx + (co<S>(k.pn.c6) + co<S>(k.pn.c6l) * lx) * x13 + co<S>(k.pn.c7) * x13 * x13;
  const S m13 = x13 * T(0.68278406325529573);  // x^(1/3) = (pi x)^(1/3) / pi^(1/3)
  const S eta = co<S>(k.eta);
  return co<S>(k.pn.A) * tf2 + (co<S>(k.sig[0]) * x + T(0.75) * co<S>(k.sig[1]) * x * m13
                                + T(0.6) * co<S>(k.sig[2]) * x * m13 * m13 + T(0.5) * co<S>(k.sig[3]) * x * x) / eta;
}

template <class S, class C>
__device__ __forceinline__ S int_phase_raw(const PhdCoreT<C>& k, const S& x) {
  typedef typename Real<S>::T T;
  return (co<S>(k.bet[0]) * x - co<S>(k.bet[2]) / (T(3) * x * x * x) + co<S>(k.bet[1]) * dlog(x)) / co<S>(k.eta);
}

template <class S, class C>
__device__ __forceinline__ S mrd_phase_raw(const PhdCoreT<C>& k, const S& x, const S& rho, const S& tau) {
  typedef typename Real<S>::T T;
  const S x14 = dsqrt(dsqrt(x));
  return (-co<S>(k.alp[1]) / x + T(4.0 / 3.0) * co<S>(k.alp[2]) * x14 * x14 * x14 + co<S>(k.alp[0]) * x
          + co<S>(k.alp[3]) * rho * datan((x - co<S>(k.alp[4]) * co<S>(k.fring)) / (co<S>(k.fdamp) * rho * tau))) / co<S>(k.eta);
}

// complete phase with the Mf < 0.2 cut (gwfast/waveforms.py:1145, :2499)
template <class S, class C>
__device__ __forceinline__ S complete_phase(const PhdCoreT<C>& k, const S& x, const S& C1, const S& C2, const S& rho, const S& tau) {
  typedef typename Real<S>::T T;
  const T xv = val(x);
  if (xv < T(kPhiFJoin)) return ins_phase(k, x);
  if (xv < T(val(k.fMRD))) return int_phase_raw(k, x) + co<S>(k.C1Int) + co<S>(k.C2Int) * x;
  if (xv < T(kMfCut)) return mrd_phase_raw(k, x, rho, tau) + C1 + C2 * x;
  return S(T(0));
}

// ---- amplitude pieces, gwfast/waveforms.py:1198-1254
template <class S, class C>
__device__ __forceinline__ S ins_amp(const PhdCoreT<C>& k, const S& x) {
  typedef typename Real<S>::T T;
  const S x13 = dcbrt(x);
  const S x23 = x13 * x13;
  return T(1) + x23 * co<S>(k.a23) + x * x13 * co<S>(k.a43) + x * x23 * co<S>(k.a53) + x * x * x13 * co<S>(k.r1)
         + x * x * x23 * co<S>(k.r2) + x * (co<S>(k.a1) + x * co<S>(k.a2) + x * x * co<S>(k.r3));
}

template <class S, class C>
__device__ __forceinline__ S mrd_amp(const PhdCoreT<C>& k, const S& x) {
  const S fr = co<S>(k.fring), fdg3 = co<S>(k.fdamp) * co<S>(k.gam[2]);
  const S dx = x - fr;
  return dexp(-dx * co<S>(k.gam[1]) / fdg3) * (fdg3 * co<S>(k.gam[0])) / (dx * dx + fdg3 * fdg3);
}

template <class S, class C>
__device__ __forceinline__ S complete_amp_shape(const PhdCoreT<C>& k, const S& x) {
  typedef typename Real<S>::T T;
  const T xv = val(x);
  if (xv < T(kAmpFJoin)) return ins_amp(k, x);
  if (xv < T(val(k.fpA))) {
    const S u = x - T(kAmpFJoin);
    return co<S>(k.h0) + u * (co<S>(k.h1) + u * (co<S>(k.h2) + (x - co<S>(k.f2)) * (co<S>(k.h3) + (x - co<S>(k.fpA)) * co<S>(k.h4))));
  }
  if (xv < T(kMfCut)) return mrd_amp(k, x);
  return S(T(0));
}

// ---- per-event setup of the IMRPhenomD core given fring, fdamp
template <class D>
__device__ inline void phenom_core_setup(PhdCoreT<D>& k, const D& Mc, const D& eta, const D& chi1, const D& chi2,
                                         const D& fring, const D& fdamp, const D& dq1 = D(0.0), const D& dq2 = D(0.0)) {
  k.eta = eta;
  k.MG = Mc * kG3 / dpowc(eta, 0.6);
  k.Ms = k.MG;
  k.vM = dcbrt(kPi * k.MG);
  k.fring = fring;
  k.fdamp = fdamp;
  const D seta = seta_of(eta);
  const D chis = 0.5 * (chi1 + chi2), chia = 0.5 * (chi1 - chi2);
  const D xi = chis * (1.0 - eta * (76.0 / 113.0)) + seta * chia - 1.0;
  for (int i = 0; i < 4; ++i) k.sig[i] = fit11(FIT_SIGMA1 + i, eta, xi);
  for (int i = 0; i < 3; ++i) k.bet[i] = fit11(FIT_BETA1 + i, eta, xi);
  for (int i = 0; i < 5; ++i) k.alp[i] = fit11(FIT_ALPHA1 + i, eta, xi);
  for (int i = 0; i < 3; ++i) k.gam[i] = fit11(FIT_GAMMA1 + i, eta, xi);
  k.pn = pn_coeffs(eta, chi1, chi2, false, true, dq1, dq2);
  // inspiral -> intermediate C1 join at Mf = 0.018 (gwfast/waveforms.py:1098-1120)
  {
    const double fj = kPhiFJoin;
    const double x = kPi * fj;
    const double x13 = cbrt(x);
    const double lx = log(x) / 3.0;
    // d/dMf of the inspiral phase
    const D dtf2 = (-5. / 3.) * pow(x, -8. / 3.) - k.pn.c2 / (x * x) - (2. / 3.) * k.pn.c3 * pow(x, -5. / 3.)
                    - (1. / 3.) * k.pn.c4 * pow(x, -4. / 3.) + k.pn.c5l / (3. * x) + k.pn.c6l * (x13 / (3. * x))
                    + (k.pn.c6 + k.pn.c6l * lx) * (x13 / (3. * x)) + (2. / 3.) * k.pn.c7 * (x13 * x13 / x);
    const D dins = k.pn.A * dtf2 * kPi + (k.sig[0] + k.sig[1] * cbrt(fj) + k.sig[2] * cbrt(fj) * cbrt(fj) + k.sig[3] * fj) / eta;
    const D dint = (k.bet[0] + k.bet[2] / (fj * fj * fj * fj) + k.bet[1] / fj) / eta;
    k.C2Int = dins - dint;
    const D xj(fj);
    const D insj = ins_phase<D>(k, xj);
    k.C1Int = insj - int_phase_raw<D>(k, xj) - k.C2Int * fj;
  }
  // intermediate -> merger-ringdown at 0.5 fring (gwfast/waveforms.py:1122-1129)
  k.fMRD = 0.5 * fring;
  {
    const D& fm = k.fMRD;
    k.PhiIntTemp = int_phase_raw<D>(k, fm) + k.C1Int + k.C2Int * fm;
    k.DPhiIntTemp = k.C2Int + (k.bet[0] + k.bet[2] / (fm * fm * fm * fm) + k.bet[1] / fm) / eta;
    const D one(1.0);
    const D u = (fm - k.alp[4] * fring) / fdamp;
    const D dmrd = (k.alp[0] + k.alp[1] / (fm * fm) + k.alp[2] / dsqrt(dsqrt(fm)) + k.alp[3] / (fdamp * (1.0 + u * u))) / eta;
    k.C2MRD = k.DPhiIntTemp - dmrd;
    k.C1MRD = k.PhiIntTemp - mrd_phase_raw<D>(k, fm, one, one) - k.C2MRD * fm;
  }
  // amplitude (gwfast/waveforms.py:1189-1245)
  {
    const D sp1 = 1.0 + seta;
    const D e2 = eta * eta;
    const D c12 = chi1 * chi1, c22 = chi2 * chi2;
    k.a23 = (-969. + 1804. * eta) * (pow(kPi, 2.0 / 3.0) / 672.);
    k.a1 = (chi1 * (81. * sp1 - 44. * eta) + chi2 * (81. - 81. * seta - 44. * eta)) * (kPi / 48.);
    k.a43 = (-27312085.0 - 10287648. * c22 - 10287648. * c12 * sp1 + 10287648. * c22 * seta
             + 24. * (-1975055. + 857304. * c12 - 994896. * chi1 * chi2 + 857304. * c22) * eta + 35371056. * e2)
            * (pow(kPi, 4.0 / 3.0) / 8.128512e6);
    k.a53 = (chi2 * (-285197. * (seta - 1.0) + 4. * (-91902. + 1579. * seta) * eta - 35632. * e2)
             + chi1 * (285197. * sp1 - 4. * (91902. + 1579. * seta) * eta - 35632. * e2) + 42840. * kPi * (4. * eta - 1.0))
            * (pow(kPi, 5.0 / 3.0) / 32256.);
    k.a2 = -(kPi * kPi / 6.0085960704e10) *
           (-336. * (-3248849057.0 + 2943675504. * c12 - 3339284256. * chi1 * chi2 + 2943675504. * c22) * e2
            - 324322727232. * e2 * eta
            - 7. * (-177520268561. + 107414046432. * c22 + 107414046432. * c12 * sp1 - 107414046432. * c22 * seta
                    + 11087290368. * kPi * (chi1 + chi2 + chi1 * seta - chi2 * seta))
            + 12. * eta * (-545384828789. - 176491177632. * chi1 * chi2 + 202603761360. * c22
                           + 77616. * c12 * (2610335. + 995766. * seta) - 77287373856. * c22 * seta
                           + 5841690624. * kPi * (chi1 + chi2) + 21384760320. * kPi * kPi));
    k.r1 = fit11(FIT_RHO1, eta, xi);
    k.r2 = fit11(FIT_RHO2, eta, xi);
    k.r3 = fit11(FIT_RHO3, eta, xi);
    const D& g1 = k.gam[0];
    const D& g2 = k.gam[1];
    const D& g3 = k.gam[2];
    k.fpA = (g2.v >= 1.0) ? dabs(fring - fdamp * g3 / g2)
                          : fring + fdamp * (dsqrt(1.0 - g2 * g2) - 1.0) * g3 / g2;
    // collocation data: value and slope of the inspiral at f1, value v2 at f2, value and slope of the ringdown at f3
    const double f1 = kAmpFJoin;
    const D f3 = k.fpA;
    const D f2 = f1 + 0.5 * (f3 - f1);
    k.f2 = f2;
    const D v1 = ins_amp<D>(k, D(f1));
    const double f113 = cbrt(f1);
    const D d1 = (2. / 3.) * k.a23 / f113 + k.a1 + (4. / 3.) * k.a43 * f113 + (5. / 3.) * k.a53 * f113 * f113 + 2. * k.a2 * f1
                  + (7. / 3.) * k.r1 * f1 * f113 + (8. / 3.) * k.r2 * f1 * f113 * f113 + 3. * k.r3 * f1 * f1;
    const D v2 = fit11(FIT_V2, eta, xi);
    const D v3 = mrd_amp<D>(k, f3);
    const D fdg3 = fdamp * g3;
    const D dx3 = f3 - fring;
    const D den3 = dx3 * dx3 + fdg3 * fdg3;
    const D d2 = (-2.0 * fdamp * dx3 * g3 * g1 / den3 - g2 * g1) / (dexp(dx3 * g2 / fdg3) * den3);
    // divided differences over the nodes (f1, f1, f2, f3, f3)
    const D q12 = (v2 - v1) / (f2 - f1);
    const D q23 = (v3 - v2) / (f3 - f2);
    const D q012 = (q12 - d1) / (f2 - f1);
    const D q123 = (q23 - q12) / (f3 - f1);
    const D q234 = (d2 - q23) / (f3 - f2);
    const D q0123 = (q123 - q012) / (f3 - f1);
    const D q1234 = (q234 - q123) / (f3 - f1);
    k.h0 = v1;
    k.h1 = d1;
    k.h2 = q012;
    k.h3 = q0123;
    k.h4 = (q1234 - q0123) / (f3 - f1);
  }
}

// t0 and phiRef (detector-dependent through fRef = M G fmin); gwfast/waveforms.py:1131-1147
template <class D>
__device__ inline void phenom_ref_setup(PhdCoreT<D>& k, const D& fpeak, double fmin_hz, const D& C1, const D& C2) {
  const D u = (fpeak - k.alp[4] * k.fring) / k.fdamp;
  k.t0 = (k.alp[0] + k.alp[1] / (fpeak * fpeak) + k.alp[2] / dsqrt(dsqrt(fpeak)) + k.alp[3] / (k.fdamp * (1.0 + u * u))) / k.eta;
  k.fRef = k.MG * fmin_hz;
  const D one(1.0);
  k.phiRef = complete_phase<D>(k, k.fRef, C1, C2, one, one);
}

struct PhdEv {
  PhdCore k;
};

template <class D>
__device__ inline void qnm_lookup(const double* qa, const double* qr, const double* qd, int n, const D& a,
                                  D& fr, D& fd) {
  // jnp.interp semantics: segment [j, j+1] with qa[j] <= a < qa[j+1]; slope carries the tangent
  int lo = 0, hi = n - 1;
  const double x = a.v;
  if (x < qa[0]) { lo = 0; }
  else if (x >= qa[n - 1]) { lo = n - 2; }
  else {
    while (hi - lo > 1) { const int mid = (lo + hi) >> 1; if (qa[mid] <= x) lo = mid; else hi = mid; }
  }
  const double x0 = qa[lo], x1 = qa[lo + 1];
  fr = qr[lo] + (a - x0) * ((qr[lo + 1] - qr[lo]) / (x1 - x0));
  fd = qd[lo] + (a - x0) * ((qd[lo + 1] - qd[lo]) / (x1 - x0));
}

// the detector-dependent part of the IMRPhenomD record: fRef = M G fmin and the phase there
// (the rest of the record depends on the source alone)
__device__ inline void phd_ref(PhdEv& e, double fmin_hz) {
  PhdCore& k = e.k;
  const D4& g2 = k.gam[1];
  const D4& g3 = k.gam[2];
  const D4& fr = k.fring;
  const D4& fd = k.fdamp;
  // phase peak frequency keeps the modulus in both branches (gwfast/waveforms.py:1134)
  const D4 fpP = (g2.v >= 1.0) ? dabs(fr - fd * g3 / g2) : dabs(fr + fd * (dsqrt(1.0 - g2 * g2) - 1.0) * g3 / g2);
  phenom_ref_setup(k, fpP, fmin_hz, k.C1MRD, k.C2MRD);
}

// IMRPhenomD per event (gwfast/waveforms.py:992-1254); fmin_hz sets fRef = min of the grid
__device__ inline void phd_setup(PhdEv& e, const D4& Mc, const D4& eta, const D4& chi1, const D4& chi2, double dL,
                                 double fmin_hz, const double* qa, const double* qr, const double* qd, int nq) {
  PhdCore& k = e.k;
  const D4 af = final_spin(eta, chi1, chi2);
  const D4 er = radiated_energy(eta, chi1, chi2);
  D4 fr, fd;
  qnm_lookup(qa, qr, qd, nq, af, fr, fd);
  fr = fr / (1.0 - er);
  fd = fd / (1.0 - er);
  phenom_core_setup(k, Mc, eta, chi1, chi2, fr, fd);
  phd_ref(e, fmin_hz);
  // 2 sqrt(5/(64 pi)) M G/c^2[Gpc] M G/c^3 / dL * sqrt(2 eta/3) pi^(-1/6)  (gwfast/waveforms.py:1204, :1248)
  const D4 M = k.MG * (1.0 / kG3);   // total mass Mc / eta^(3/5) (MG = M G/c^3)
  k.ampPref = (2.0 * sqrt(5.0 / (64.0 * kPi)) * kG2Gpc * kG3 / dL * pow(kPi, -1.0 / 6.0)) * M * M * dsqrt(eta * (2.0 / 3.0));
}

// amplitude A(f) and phase Phi(f) of IMRPhenomD at physical frequency f (Hz)
template <class S, class C>
__device__ __forceinline__ void phd_point(const PhdCoreT<C>& k, typename Real<S>::T f, S& amp, S& phase) {
  typedef typename Real<S>::T T;
  const S x = co<S>(k.MG) * f;
  const T xv = val(x);
  const S one(T(1));
  const S shape = complete_amp_shape(k, x);
  // x^(-7/6)
  const S xm76 = T(1) / (x * dsqrt(dcbrt(x)));
  amp = co<S>(k.ampPref) * xm76 * shape;
  const S ph = complete_phase(k, x, co<S>(k.C1MRD), co<S>(k.C2MRD), one, one);
  phase = (xv < T(kMfCut)) ? ph - co<S>(k.t0) * (x - co<S>(k.fRef)) - co<S>(k.phiRef) : ph;
}

// IMRPhenomD amplitude only
template <class S, class C>
__device__ __forceinline__ S phd_amp_point(const PhdCoreT<C>& k, typename Real<S>::T f) {
  typedef typename Real<S>::T T;
  const S x = co<S>(k.MG) * f;
  return co<S>(k.ampPref) * (T(1) / (x * dsqrt(dcbrt(x)))) * complete_amp_shape(k, x);
}

// IMRPhenomD amplitude with its tangent in FP64 (the FP64 Fisher kernels). In the inspiral region
// A = ampPref x^(-7/6) S(x), S = 1 + sum_k c_k x^(k/3) (k = 2..9; c_k = a23, a1, a43, a53, a2, r1, r2,
// r3), x = MG f with tangent x d ln MG, so
//   d ln A = d ln ampPref + (-7/6 + x S'(x) / S) d ln MG + (sum_k d c_k x^(k/3)) / S
// (t: the event's log-derivatives of ampPref and MG); elsewhere the dual evaluation.
__device__ __forceinline__ D4 phd_amp_d(const PhdCore& k, const TauD& t, double f) {
  const double xv = k.MG.v * f;
  if (!(xv < kAmpFJoin)) return phd_amp_point<D4>(k, f);
  const double x13 = cbrt(xv), x23 = x13 * x13, x2 = xv * xv;
  const double bas[8] = {x23, xv, xv * x13, xv * x23, x2, x2 * x13, x2 * x23, x2 * xv};
  const D4* c[8] = {&k.a23, &k.a1, &k.a43, &k.a53, &k.a2, &k.r1, &k.r2, &k.r3};
  double S = 1.0, xS = 0.0, T[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const double cb = c[j]->v * bas[j];
    S += cb;
    xS = fma((double)(j + 2) * (1.0 / 3.0), cb, xS);
#pragma unroll
    for (int q = 0; q < 4; ++q) T[q] = fma(c[j]->d[q], bas[j], T[q]);
  }
  const double iS = 1.0 / S;
  D4 A;
  A.v = k.ampPref.v * S / (xv * sqrt(x13));
  const double gx = -7.0 / 6.0 + xS * iS;
#pragma unroll
  for (int q = 0; q < 4; ++q) A.d[q] = A.v * (t.dlnP[q] + gx * t.dlnMG[q] + T[q] * iS);
  return A;
}

// ------------------------------------------------------------------ phase tangent in a frequency basis
// Within each region the phase is a fixed linear combination of basis functions of the physical
// frequency f with parameter-dependent coefficients:
//   inspiral (Mf < 0.018), 13 terms: f^-5/3 f^-1 f^-2/3 f^-1/3 1 ln f f^1/3 f^1/3 ln f f^2/3 f f^4/3 f^5/3 f^2
//   intermediate (Mf < fring/2), 4 terms: f f^-3 ln f 1
//   merger-ringdown (Mf < 0.2), 5 terms: f^-1 f^3/4 f 1 atan((U1 f - U0))
// (expanding (pi M f)^q = (pi M)^q f^q and folding -t0 (Mf - MfRef) - phiRef into the f and 1
// coefficients).  Their d/d(Mc, eta, chi1z, chi2z) are formed here in FP64; large terms that
// cancel in the tangent (the eta-independence of the Newtonian term at fixed Mc, the t0 shift
// against the merger slope, the reference-phase subtraction) therefore cancel in FP64, once
// per event, and the per-point FP32 work is a short, well-conditioned sum.
struct PhaseBasis {
  D4 ins[13];
  D4 itm[4];
  D4 mrd[5];
  D4 U1, U0;
  D4 MG;          // region boundaries are tested on MG f
  double fMRD;    // intermediate/merger join in Mf
  double pad;
};

__device__ inline void tf2_phase_basis(const TF2Ev& e, PhaseBasis& b) {
  // Phi = A (pi Ms f)^(-5/3) [1 + c2 v^2 + ... ] with v = (pi Ms f)^(1/3)  (gwfast/waveforms.py:860)
  const D4 lpm = dlog(kPi * e.Ms);
  const D4 pm13 = dexp(lpm * (1.0 / 3.0));
  const D4 pm_53 = dexp(lpm * (-5.0 / 3.0));
  const D4 pm13_2 = pm13 * pm13;
  const PNC& c = e.pn;
  for (int i = 0; i < 13; ++i) b.ins[i] = D4(0.0);
  b.ins[0] = c.A * pm_53;
  b.ins[1] = c.A * c.c2 * pm_53 * pm13_2;
  b.ins[2] = c.A * c.c3 * pm_53 * pm13_2 * pm13;
  b.ins[3] = c.A * c.c4 * pm_53 * pm13_2 * pm13_2;
  b.ins[4] = c.A * (c.c5 + c.c5l * lpm * (1.0 / 3.0));
  b.ins[5] = c.A * c.c5l * (1.0 / 3.0);
  b.ins[6] = c.A * (c.c6 + c.c6l * lpm * (1.0 / 3.0)) * pm13;
  b.ins[7] = c.A * c.c6l * (1.0 / 3.0) * pm13;
  b.ins[8] = c.A * c.c7 * pm13_2;
  for (int i = 0; i < 4; ++i) b.itm[i] = D4(0.0);
  for (int i = 0; i < 5; ++i) b.mrd[i] = D4(0.0);
  b.U1 = D4(0.0); b.U0 = D4(0.0);
  b.MG = D4(0.0);  // every point is in the inspiral form
  b.fMRD = 1e30;
  b.pad = 0.0;
}

__device__ inline void phd_phase_basis(const PhdCore& k, PhaseBasis& b) {
  const D4& MG = k.MG;
  const D4 eta = k.eta;
  const D4 lpm = dlog(kPi * MG);
  const D4 pm13 = dexp(lpm * (1.0 / 3.0));
  const D4 pm_53 = dexp(lpm * (-5.0 / 3.0));
  const D4 pm13_2 = pm13 * pm13;
  const PNC& c = k.pn;
  const D4 lin = k.t0 * k.fRef - k.phiRef;           // constant part of -t0 (Mf - MfRef) - phiRef
  const D4 m13 = pm13 * 0.68278406325529573;          // MG^(1/3) = (pi MG)^(1/3) / pi^(1/3)
  const D4 lmg = lpm - 1.1447298858494002;            // ln MG = ln(pi MG) - ln pi
  // inspiral (gwfast/waveforms.py:1145)
  b.ins[0] = c.A * pm_53;
  b.ins[1] = c.A * c.c2 * pm_53 * pm13_2;
  b.ins[2] = c.A * c.c3 * pm_53 * pm13_2 * pm13;
  b.ins[3] = c.A * c.c4 * pm_53 * pm13_2 * pm13_2;
  b.ins[4] = c.A * (c.c5 + c.c5l * lpm * (1.0 / 3.0)) + lin;
  b.ins[5] = c.A * c.c5l * (1.0 / 3.0);
  b.ins[6] = c.A * (c.c6 + c.c6l * lpm * (1.0 / 3.0)) * pm13;
  b.ins[7] = c.A * c.c6l * (1.0 / 3.0) * pm13;
  b.ins[8] = c.A * c.c7 * pm13_2;
  b.ins[9] = (k.sig[0] / eta - k.t0) * MG;
  b.ins[10] = (0.75 * k.sig[1] / eta) * MG * m13;
  b.ins[11] = (0.6 * k.sig[2] / eta) * MG * m13 * m13;
  b.ins[12] = (0.5 * k.sig[3] / eta) * MG * MG;
  // intermediate: (b1 x - b3/(3 x^3) + b2 ln x)/eta + C1Int + C2Int x
  b.itm[0] = (k.bet[0] / eta + k.C2Int - k.t0) * MG;
  b.itm[1] = -k.bet[2] / (3.0 * eta * MG * MG * MG);
  b.itm[2] = k.bet[1] / eta;
  b.itm[3] = k.bet[1] / eta * lmg + k.C1Int + lin;
  // merger-ringdown: (-a2/x + 4/3 a3 x^3/4 + a1 x + a4 atan((x - a5 fring)/fdamp))/eta + C1MRD + C2MRD x
  const D4 m14 = dsqrt(dsqrt(MG));
  b.mrd[0] = -k.alp[1] / (eta * MG);
  b.mrd[1] = (4.0 / 3.0) * k.alp[2] / eta * m14 * m14 * m14;
  b.mrd[2] = (k.alp[0] / eta + k.C2MRD - k.t0) * MG;
  b.mrd[3] = k.C1MRD + lin;
  b.mrd[4] = k.alp[3] / eta;
  b.U1 = MG / k.fdamp;
  b.U0 = k.alp[4] * k.fring / k.fdamp;
  b.MG = MG;
  b.fMRD = k.fMRD.v;
  b.pad = 0.0;
}

// d Phi / d(Mc, eta, chi1z, chi2z) at physical frequency f (Hz) from the basis, in FP64: the FP64
// Fisher kernels' phase tangent for TaylorF2 and IMRPhenomD (a basis sum of at most 13 terms per
// direction in place of the dual evaluation of the phase at every point). The region tests are those
// of complete_phase, on MG f; beyond Mf = 0.2 the phase and its tangent are zero. In the
// merger-ringdown term k4 atan(U1 f - U0) the argument depends on the parameters as well.
__device__ __forceinline__ void phase_tangent_d(const PhaseBasis& b, double f, double lnf, double (&dphi)[4]) {
  const double x = b.MG.v * f;
#pragma unroll
  for (int q = 0; q < 4; ++q) dphi[q] = 0.0;
  if (x < kPhiFJoin) {
    const double f13 = cbrt(f), i13 = 1.0 / f13, i23 = i13 * i13;
    // f^-5/3 f^-1 f^-2/3 f^-1/3 1 ln f f^1/3 f^1/3 ln f f^2/3 f f^4/3 f^5/3 f^2
    const double bas[13] = {i23 * i23 * i13, i23 * i13, i23, i13, 1.0, lnf, f13, f13 * lnf, f13 * f13,
                            f, f * f13, f * f13 * f13, f * f};
#pragma unroll
    for (int j = 0; j < 13; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) dphi[q] = fma(b.ins[j].d[q], bas[j], dphi[q]);
  } else if (x < b.fMRD) {
    const double i1 = 1.0 / f;
    const double bas[4] = {f, i1 * i1 * i1, lnf, 1.0};
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) dphi[q] = fma(b.itm[j].d[q], bas[j], dphi[q]);
  } else if (x < kMfCut) {
    const double u = b.U1.v * f - b.U0.v;
    const double f14 = sqrt(sqrt(f));
    const double bas[5] = {1.0 / f, f14 * f14 * f14, f, 1.0, atan(u)};
#pragma unroll
    for (int j = 0; j < 5; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) dphi[q] = fma(b.mrd[j].d[q], bas[j], dphi[q]);
    const double kd = b.mrd[4].v / (1.0 + u * u);
#pragma unroll
    for (int q = 0; q < 4; ++q) dphi[q] = fma(kd, fma(b.U1.d[q], f, -b.U0.d[q]), dphi[q]);
  }
}

// ------------------------------------------------------------------ IMRPhenomD_NRTidalv2 (gwfast/waveforms.py:1339-1836)
// IMRPhenomD with the spin-induced quadrupole (from the tidal deformabilities) in its 2PN and 3PN
// spin-spin phase terms, the NRTidalv2 tidal phase (Pade approximant, arXiv:1905.06011 eq. 17), the
// 3.5PN spin-squared and spin-cubed terms (eq. 27), the tidal amplitude (eq. 24) and a Planck taper
// ending the waveform at 1.2 times the merger frequency. The tidal deformabilities enter the phase
// connection constants through the quadrupole moments, so the per-event set-up carries six
// tangent directions (Mc, eta, chi1z, chi2z, LambdaTilde, deltaLambda).
template <class C> struct NRTEvT {
  PhdCoreT<C> k;
  C tidP;   // -kappa2T c_Newt / (m1 m2): coefficient of the tidal phase
  C ssA;    // (SS_3p5PN + SSS_3p5PN) 3 / (128 eta): coefficient of (pi M f)^(2/3)
  C tidA;   // 2 sqrt(pi/5) (-9 kappa2T) / amp0: the tidal amplitude relative to the prefactor
  C fmer;   // Planck-taper merger frequency in M f
};
using NRTEv = NRTEvT<D6>;

// quadrupole moment from the tidal deformability, arXiv:1608.02582 eq. 15 (gwfast/waveforms.py:1402-1403)
template <class D>
__device__ inline D quad_mon(const D& lam) {
  if (lam.v < 1.0) return 1.0 + lam * (0.427688866723244 + lam * (-0.324336526985068 + lam * 0.1107439432180572));
  const D l = dlog(lam);
  return dexp(0.1940 + l * (0.09163 + l * (0.04812 + l * (-4.283e-3 + l * 1.245e-4))));
}
// octupole moment minus 1 from the quadrupole moment (gwfast/waveforms.py:1564-1565)
template <class D>
__device__ inline D oct_mon_m1(const D& q) {
  const D l = dlog(q);
  return dexp(0.003131 + l * (2.071 + l * (-0.7152 + l * (0.2458 + l * -0.03309)))) - 1.0;
}

// Lambda1, Lambda2 from (LambdaTilde, deltaLambda): the inverse of the linear map of
// gwfast/gwfastUtils.py:398-417 (its inverse, :419-446)
template <class D>
__device__ inline void lam12_of(const D& lt, const D& dlt, const D& eta, D& l1, D& l2) {
  const D e2 = eta * eta;
  const D seta = seta_of(eta);
  const D ap = (8. / 13.) * (1. + 7. * eta - 31. * e2), am = (8. / 13.) * seta * (1. + 9. * eta - 11. * e2);
  const D bp = 0.5 * seta * (1. - 13272. / 1319. * eta + 8944. / 1319. * e2);
  const D bm = 0.5 * (1. - 15910. / 1319. * eta + 32850. / 1319. * e2 + 3380. / 1319. * e2 * eta);
  const D det = ap * bm - am * bp;
  const D lp = (bm * lt - am * dlt) / det, lm = (ap * dlt - bp * lt) / det;
  l1 = 0.5 * (lp + lm);
  l2 = 0.5 * (lp - lm);
}

// merger frequency of the Planck taper in M f (gwfast/waveforms.py:1681-1694, :1813-1832)
template <class D>
__device__ inline D nrt_fmerger(const D& eta, const D& kap) {
  const D seta = seta_of(eta);
  const D q = 0.5 * (1.0 + seta - 2.0 * eta) / eta;
  const D num = 1.0 + kap * (3.35411203e-2 + kap * 4.31460284e-5);
  const D den = 1.0 + kap * (7.54224145e-2 + kap * 2.23626859e-4);
  return (0.3586 / dsqrt(q)) * (num / den) / (2.0 * kPi);
}

template <class D>
__device__ inline D nrt_kappa2t(const D& eta, const D& l1, const D& l2) {
  const D seta = seta_of(eta);
  const D xa = 0.5 * (1.0 + seta), xb = 0.5 * (1.0 - seta);
  const D xa2 = xa * xa, xb2 = xb * xb;
  return (3.0 / 13.0) * ((1.0 + 12.0 * xb / xa) * (xa2 * xa2 * xa) * l1 + (1.0 + 12.0 * xa / xb) * (xb2 * xb2 * xb) * l2);
}

// upper grid frequency in Hz: 1.2 times the merger frequency (gwfast/waveforms.py:1798-1832)
__device__ inline double nrt_fcut(double Mc, double eta, double lt, double dlt) {
  typedef Dual<double, 1> D1;   // value-only use of the dual helpers
  D1 l1, l2;
  lam12_of(D1(lt), D1(dlt), D1(eta), l1, l2);
  const D1 kap = nrt_kappa2t(D1(eta), l1, l2);
  return 1.2 * nrt_fmerger(D1(eta), kap).v / (Mc / pow(eta, 0.6) * kG3);
}

__device__ inline void nrt_ref(NRTEv& e, double fmin_hz) {
  PhdCoreT<D6>& k = e.k;
  const D6& g2 = k.gam[1];
  const D6& g3 = k.gam[2];
  const D6 fpP = (g2.v >= 1.0) ? dabs(k.fring - k.fdamp * g3 / g2) : dabs(k.fring + k.fdamp * (dsqrt(1.0 - g2 * g2) - 1.0) * g3 / g2);
  phenom_ref_setup(k, fpP, fmin_hz, k.C1MRD, k.C2MRD);
}

__device__ inline void nrt_setup(NRTEv& e, const D6& Mc, const D6& eta, const D6& chi1, const D6& chi2, double dL,
                                 double fmin_hz, const double* qa, const double* qr, const double* qd, int nq,
                                 const D6& lt, const D6& dlt) {
  PhdCoreT<D6>& k = e.k;
  D6 l1, l2;
  lam12_of(lt, dlt, eta, l1, l2);
  const D6 q1 = quad_mon(l1), q2 = quad_mon(l2);
  const D6 af = final_spin(eta, chi1, chi2);
  const D6 er = radiated_energy(eta, chi1, chi2);
  D6 fr, fd;
  qnm_lookup(qa, qr, qd, nq, af, fr, fd);
  fr = fr / (1.0 - er);
  fd = fd / (1.0 - er);
  phenom_core_setup(k, Mc, eta, chi1, chi2, fr, fd, q1 - 1.0, q2 - 1.0);
  nrt_ref(e, fmin_hz);
  const D6 M = Mc / dpowc(eta, 0.6);
  const D6 amp0 = dsqrt(eta * (2.0 / 3.0)) * pow(kPi, -1.0 / 6.0);
  k.ampPref = (2.0 * sqrt(5.0 / (64.0 * kPi)) * kG2Gpc * kG3 / dL) * M * M * amp0;
  const D6 seta = seta_of(eta);
  const D6 m1 = 0.5 * (1.0 + seta), m2 = 0.5 * (1.0 - seta);
  const D6 kap = nrt_kappa2t(eta, l1, l2);
  e.tidP = (-2.4375) * kap / (m1 * m2);
  e.tidA = (2.0 * sqrt(kPi / 5.0) * -9.0) * kap / amp0;
  e.fmer = nrt_fmerger(eta, kap);
  // 3.5PN spin-squared and spin-cubed terms (gwfast/waveforms.py:1567-1568)
  const D6 c12 = chi1 * chi1, c22 = chi2 * chi2, m12 = m1 * m1, m22 = m2 * m2;
  const D6 dq1 = q1 - 1.0, dq2 = q2 - 1.0;
  const D6 ss = -400. * kPi * dq1 * c12 * m12 - 400. * kPi * dq2 * c22 * m22;
  const D6 sss = 10. * ((m12 + 308. / 3. * m1) * chi1 + (m22 - 89. / 3. * m2) * chi2) * dq1 * m12 * c12
                 + 10. * ((m22 + 308. / 3. * m2) * chi2 + (m12 - 89. / 3. * m1) * chi1) * dq2 * m22 * c22
                 - 440. * oct_mon_m1(q1) * m12 * m1 * c12 * chi1 - 440. * oct_mon_m1(q2) * m22 * m2 * c22 * chi2;
  e.ssA = (ss + sss) * (3.0 / (128.0 * eta));
}

__device__ __forceinline__ double taper_make(double, double t, double) { return t; }
template <class U, int N>
__device__ __forceinline__ Dual<U, N> taper_make(const Dual<U, N>& y, U t, U dy) { return chain(y, t, dy); }

// Planck taper (gwfast/waveforms.py:1696-1716) at x = M f for merger frequency y: its tangent is
// carried only through y, as gwfast's custom derivative of the taper does (the x dependence is
// left out there)
template <class S, class C>
__device__ __forceinline__ S planck_taper(typename Real<S>::T x, const C& y_) {
  typedef typename Real<S>::T T;
  const S y = co<S>(y_);
  const T yv = val(y), a = T(1.2), yp = a * yv;
  if (x < yv) return S(T(1));
  if (x > yp) return S(T(0));
  const T u = (yp - yv) / (x - yv) + (yp - yv) / (x - yp);
  const T E = exp(u);
  T t = T(1) - T(1) / (E + T(1));
  if (!(t == t)) t = T(0);   // nan_to_num
  T dy = E * ((a - T(1)) / (x - yv) + (a - T(1)) / (x - yp) + (yp - yv) / ((x - yv) * (x - yv))
              + a * (yp - yv) / ((x - yp) * (x - yp))) / ((E + T(1)) * (E + T(1)));
  if (!(dy == dy) || isinf(dy)) dy = T(0);
  return taper_make(y, t, dy);
}

// amplitude and phase of IMRPhenomD_NRTidalv2 at physical frequency f (Hz)
template <class S, class C>
__device__ __forceinline__ void nrt_point(const NRTEvT<C>& e, typename Real<S>::T f, S& amp, S& phase) {
  typedef typename Real<S>::T T;
  const PhdCoreT<C>& k = e.k;
  const S x = co<S>(k.MG) * f;
  const T xv = val(x);
  const S one(T(1));
  const S xm76 = T(1) / (x * dsqrt(dcbrt(x)));
  const S px = T(kPi) * x;
  const S xt = dcbrt(px) * dcbrt(px);   // (pi M f)^(2/3)
  const S xt2 = xt * xt;
  const S poly = (T(1) + T(4.157407407407407) * xt + T(2519.111111111111) * dexp(T(2.89) * dlog(xt)))
                 / (T(1) + T(13477.8073677) * xt2 * xt2);
  const S tidal_amp = co<S>(e.tidA) * dexp(T(3.25) * dlog(xt)) * poly;
  const S taper = planck_taper<S, C>(xv, e.fmer);
  amp = co<S>(k.ampPref) * (xm76 * complete_amp_shape(k, x) + tidal_amp) * taper;
  S ph = complete_phase(k, x, co<S>(k.C1MRD), co<S>(k.C2MRD), one, one);
  if (xv < T(kMfCut)) {
    const S x13 = dcbrt(px);
    const S num = T(1) + x13 * x13 * T(-12.615214237993088) + px * T(19.0537346970349)
                  + x13 * px * T(-21.166863146081035) + x13 * x13 * px * T(90.55082156324926) + px * px * T(-60.25357801943598);
    const S den = T(1) + x13 * x13 * T(-15.11120782773667) + px * T(22.195327350624694) + x13 * px * T(8.064109635305156);
    const S tidal_ph = co<S>(e.tidP) * (x13 * x13 * px) * num / den;   // (pi M f)^(5/3) num / den
    ph = ph - co<S>(k.t0) * (x - co<S>(k.fRef)) - co<S>(k.phiRef) + tidal_ph + co<S>(e.ssA) * xt;
  }
  phase = ph;
}

// ------------------------------------------------------------------ IMRPhenomNSBH (gwfast/waveforms.py:2752-3284)
// Object 1 is the black hole, object 2 the neutron star; only Lambda2 enters (the BH deformability
// recovered from LambdaTilde, deltaLambda is discarded).

// xi_tide grid (gwfast/waveforms.py:3306-3308): numpy linspace values, k * step + start with the last
// node set to the end point, so that the cell search matches numpy's searchsorted exactly
constexpr int kXiN = 200;
__host__ __device__ inline double xi_grid(int dim, int k) {
  const double lo = dim == 0 ? 0.1 : (dim == 1 ? 1.0 : -1.0), hi = dim == 0 ? 0.5 : (dim == 1 ? 100.0 : 1.0);
  if (k == kXiN - 1) return hi;
#ifdef __CUDA_ARCH__
  return __dadd_rn(__dmul_rn((double)k, (hi - lo) / (kXiN - 1)), lo);
#else
  const volatile double t = (double)k * ((hi - lo) / (kXiN - 1));
  return t + lo;
#endif
}

// trilinear interpolation of the table tab[i][j][k] as gwfast's RegularGridInterpolator_JAX
// (gwfast/gwfastUtils.py:1113-1200): cell from searchsorted - 1 clamped to the grid (linear
// extrapolation outside), edge sum in itertools.product order, NaN where that code's out-of-bounds
// test (as written: (oob + x) < lo, then (oob + x) > hi, per dimension in turn) is set
template <class D>
__device__ inline D xitide_interp(const double* tab, const D& C, const D& q, const D& chi) {
  const D* x[3] = {&C, &q, &chi};
  int idx[3];
  D y[3];
  bool oob = false;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const double xv = val(*x[d]);
    // searchsorted(grid, x, 'left') - 1: the last node below x (a guess from the spacing, then exact)
    double t = (xv - xi_grid(d, 0)) / ((xi_grid(d, kXiN - 1) - xi_grid(d, 0)) / (kXiN - 1));
    t = t == t ? fmin(fmax(t, -2.0), (double)kXiN) : 0.0;
    int i = (int)floor(t);
    i = i < -1 ? -1 : (i > kXiN - 1 ? kXiN - 1 : i);
    while (i >= 0 && !(xi_grid(d, i) < xv)) --i;
    while (i + 1 <= kXiN - 1 && xi_grid(d, i + 1) < xv) ++i;
    i = i < 0 ? 0 : (i > kXiN - 2 ? kXiN - 2 : i);
    idx[d] = i;
    const double g0 = xi_grid(d, i), g1 = xi_grid(d, i + 1);
    y[d] = (*x[d] - g0) / (g1 - g0);
    oob = ((double)oob + xv) < xi_grid(d, 0);
    oob = ((double)oob + xv) > xi_grid(d, kXiN - 1);
  }
  D out(0.0);
#pragma unroll
  for (int e0 = 0; e0 < 2; ++e0)
#pragma unroll
    for (int e1 = 0; e1 < 2; ++e1)
#pragma unroll
      for (int e2 = 0; e2 < 2; ++e2) {
        const double v = tab[((size_t)(idx[0] + e0) * kXiN + (idx[1] + e1)) * kXiN + (idx[2] + e2)];
        const D w = (e0 ? y[0] : 1.0 - y[0]) * (e1 ? y[1] : 1.0 - y[1]) * (e2 ? y[2] : 1.0 - y[2]);
        out = out + v * w;
      }
  if (oob) out = D(nan(""));
  return out;
}

// remnant fits (gwfast/waveforms.py:2854-2874, :3124-3151): remnant-spin and remnant-mass models of
// arXiv:1903.11622, the orbital angular momentum fit of arXiv:1611.00332 eq. 16 and its radiated energy
// eq. 27
template <class D>
__device__ inline D nsbh_rem_model(const double* c, const D& eta, const D& chi1, const D& lam) {
  const D p1 = ((c[0] * chi1 + c[1]) + (c[2] * chi1 + c[3]) * eta) * eta;
  const D p2 = ((c[4] * chi1 + c[5]) + (c[6] * chi1 + c[7]) * eta) * eta;
  const D p3 = ((c[8] * chi1 + c[9]) + (c[10] * chi1 + c[11]) * eta) * eta;
  const D den = 1.0 + lam * p3 * p3;
  const D m = (1.0 + lam * p1 + lam * lam * p2) / (den * den);
  if ((chi1.v < 0.0 && eta.v < 0.188) || chi1.v < -0.5 || m.v > 1.0) return D(1.0);
  return m;
}

template <class D>
__device__ inline void nsbh_remnant(const D& eta, const D& chi1, const D& lam, D& chif, D& mfin) {
  const double csp[12] = {-5.44187381e-03, 7.91165608e-03, 2.33362046e-02, 2.47764497e-02, -8.56844797e-07,
                          -2.81727682e-06, 6.61290966e-06, 4.28979016e-05, -3.04174272e-02, 2.54889050e-01,
                          1.47549350e-01, -4.27905832e-01};
  const double cm[12] = {-1.83417425e-03, 2.39226041e-03, 4.29407902e-03, 9.79775571e-03, 2.33868869e-07,
                         -8.28090025e-07, -1.64315549e-06, 8.08340931e-06, -2.00726981e-02, 1.31986011e-01,
                         6.50754064e-02, -1.42749961e-01};
  const D rsp = nsbh_rem_model(csp, eta, chi1, lam), rm = nsbh_rem_model(cm, eta, chi1, lam);
  const D seta = seta_of(eta);
  const D m1 = 0.5 * (1.0 + seta), m2 = 0.5 * (1.0 - seta);
  const D e2 = eta * eta, e3 = e2 * eta;
  const D S1 = chi1 * m1 * m1;
  const D Sh = S1 / (m1 * m1 + m2 * m2);
  const D Sh2 = Sh * Sh, Sh3 = Sh2 * Sh;
  const D lorb = (2.0 * sqrt(3.0) * eta + 5.24 * 3.8326341618708577 * e2 + 1.3 * (-9.487364155598392) * e3)
                     / (1.0 + 2.88 * 2.5134875145648374 * eta)
                 + ((-0.194) * 1.0009563702914628 * Sh * (4.409160174224525 * eta + 0.5118334706832706 * e2
                                                         + (64. - 16. * 4.409160174224525 - 4. * 0.5118334706832706) * e3)
                    + 0.0851 * 0.7877509372255369 * Sh2 * (8.77367320110712 * eta + (-32.060648277652994) * e2
                                                           + (64. - 16. * 8.77367320110712 - 4. * (-32.060648277652994)) * e3)
                    + 0.00954 * 0.6540138407185817 * Sh3 * (22.830033250479833 * eta + (-153.83722669033995) * e2
                                                            + (64. - 16. * 22.830033250479833 - 4. * (-153.83722669033995)) * e3))
                       / (1.0 + (-0.579) * 0.8396665722805308 * Sh
                                    * (1.8804718791591157 + (-4.770246856212403) * eta
                                       + (64. - 64. * 1.8804718791591157 - 16. * (-4.770246856212403)) * e3))
                 + 0.3223660562764661 * seta * e2 * (1.0 + 9.332575956437443 * eta) * chi1
                 + 2.3170397514509933 * Sh * seta * e3 * (1.0 + (-3.2624649875884852) * eta) * chi1
                 + (-0.059808322561702126) * e3 * chi1 * chi1;
  chif = (lorb + S1) * rsp;
  const D erad = ((1.0 - 2.0 / 3.0 * sqrt(2.0)) * eta + 0.5609904135313374 * e2 + (-0.84667563764404) * e3
                  + 3.145145224278187 * e2 * e2)
                     * (1.0 + 0.346 * (-0.2091189048177395) * Sh
                                  * (1.8083565298668276 + 15.738082204419655 * eta
                                     + (16. - 16. * 1.8083565298668276 - 4. * 15.738082204419655) * e2)
                        + 0.211 * (-0.19709136361080587) * Sh2 * (4.271313308472851 + (16. - 16. * 4.271313308472851) * e2)
                        + 0.128 * (-0.1588185739358418) * Sh3
                              * (31.08987570280556 + (-243.6299258830685) * eta
                                 + (16. - 16. * 31.08987570280556 - 4. * (-243.6299258830685)) * e2))
                     / (1.0 + (-0.212) * 2.9852925538232014 * Sh
                                  * (1.5673498395263061 + (-0.5808669012986468) * eta
                                     + (16. - 16. * 1.5673498395263061 - 4. * (-0.5808669012986468)) * e2))
                 + (-0.09803730445895877) * seta * e2 * (1.0 + (-3.2283713377939134) * eta) * chi1
                 + (-0.01978238971523653) * Sh * seta * eta * (1.0 + (-4.91667749015812) * eta) * chi1
                 + 0.01118530335431078 * e3 * chi1 * chi1;
  mfin = (1.0 - erad) * rm;
}

// NS spin-induced quadrupole moment, arXiv:1303.1528 eq. 54 (gwfast/waveforms.py:2832)
template <class D>
__device__ inline D nsbh_quad_mon(const D& lam) {
  if (lam.v < 1e-5) return D(1.0);
  const D l = dlog(lam);
  return dexp(0.194 + l * (0.0936 + l * (0.0474 + l * (-0.00421 + l * 0.000123))));
}

template <class C> struct NSBHEvT {
  PhdCoreT<C> k;   // phase: IMRPhenomD with the NSBH ringdown
  C tidP;          // -kappa2T c_Newt / (m1 m2)
  C xd[7];         // xdotaN, xdota2, xdota3, xdota4, xdota5, xdota6, xdota7 (gwfast/waveforms.py:3047-3054)
  C an[8];         // AN, A2, A3, A4, A5, A5imag, A6, A6imag (:3056-3065)
  C aPM;           // gamma_correction g1
  C aRD;           // epsilon_tide del1
  C frA, sig;      // amplitude ringdown frequency (M f) and Lorentzian width
  C c0pn, c0pm, c0rd;   // window centres in M f (epsilon_ins f0_PN, f0_PM, f0_RD)
  C wsc;           // 4 / (d0 + sigma_tide)
};
using NSBHEv = NSBHEvT<D6>;

// the detector-dependent part: fRef = M G fmin and t0 at the highest grid frequency (:2991-2993)
__device__ inline void nsbh_ref(NSBHEv& e, double fmin_hz, double fmax_grid_hz) {
  PhdCoreT<D6>& k = e.k;
  phenom_ref_setup(k, k.MG * fmax_grid_hz, fmin_hz, k.C1MRD, k.C2MRD);
}

__device__ inline void nsbh_setup(NSBHEv& e, const D6& Mc, const D6& eta, const D6& chi1, const D6& chi2, double dL,
                                  double fmin_hz, double fmax_grid_hz, const double* qa, const double* qr,
                                  const double* qd, int nq, const D6& lt, const D6& dlt, const double* xit) {
  PhdCoreT<D6>& k = e.k;
  D6 l1, lam;
  lam12_of(lt, dlt, eta, l1, lam);
  D6 chif, mfin;
  nsbh_remnant(eta, chi1, lam, chif, mfin);
  // phase (gwfast/waveforms.py:2874-3015): ringdown from the remnant spin, IMRPhenomD radiated energy
  const D6 er = radiated_energy(eta, chi1, chi2);
  D6 fr, fd;
  qnm_lookup(qa, qr, qd, nq, chif, fr, fd);
  fr = fr / (1.0 - er);
  fd = fd / (1.0 - er);
  phenom_core_setup(k, Mc, eta, chi1, chi2, fr, fd, D6(0.0), nsbh_quad_mon(lam) - 1.0);
  nsbh_ref(e, fmin_hz, fmax_grid_hz);
  const D6 seta = seta_of(eta);
  const D6 m1 = 0.5 * (1.0 + seta), m2 = 0.5 * (1.0 - seta);
  const D6 m22 = m2 * m2;
  const D6 kap = (3.0 / 13.0) * ((1.0 + 12.0 * m1 / m2) * (m22 * m22 * m2) * lam);
  e.tidP = (-2.4375) * kap / (m1 * m2);
  // amplitude (gwfast/waveforms.py:3017-3226)
  const D6 M = Mc / dpowc(eta, 0.6);
  k.ampPref = (2.0 * sqrt(5.0 / (64.0 * kPi)) * kG2Gpc * kG3 / dL) * M * M;
  const D6 q = 0.5 * (1.0 + seta - 2.0 * eta) / eta;
  const D6 e2 = eta * eta;
  const D6 ce = m1 * chi1 + m2 * chi2, cs = 2.0 * ce, cp = ce * ce;
  const double pi2 = kPi * kPi, eg = kEulerGamma;
  e.xd[0] = 64.0 * eta / 5.0;
  e.xd[1] = -7.43 / 3.36 - 11.0 * eta / 4.0;
  e.xd[2] = 4.0 * kPi - 11.3 * ce / 1.2 + 19.0 * eta * cs / 6.0;
  e.xd[3] = 3.4103 / 1.8144 + 5.0 * cp + eta * (13.661 / 2.016 - cp / 8.0) + 5.9 * e2 / 1.8;
  e.xd[4] = -kPi * (41.59 / 6.72 + 189.0 * eta / 8.0) - ce * (31.571 / 1.008 - 116.5 * eta / 2.4)
            + cs * (21.863 * eta / 1.008 - 79.0 * e2 / 6.0) - 3.0 * ce * cp / 4.0 + 9.0 * eta * ce * cp / 4.0;
  e.xd[5] = 164.47322263 / 1.39708800 - 17.12 * eg / 1.05 + 16.0 * pi2 / 3.0 - 8.56 * log(16.0) / 1.05
            + eta * (45.1 * pi2 / 4.8 - 561.98689 / 2.17728) + 5.41 * e2 / 8.96 - 5.605 * eta * e2 / 2.592
            - 80.0 * kPi * ce / 3.0 + eta * cs * (20.0 * kPi / 3.0 - 113.5 * ce / 3.6)
            + cp * (64.153 / 1.008 - 45.7 * eta / 3.6) - cp * (7.87 * eta / 1.44 - 30.37 * e2 / 1.44);
  e.xd[6] = -kPi * (4.415 / 4.032 - 358.675 * eta / 6.048 - 91.495 * e2 / 1.512)
            - ce * (252.9407 / 2.7216 - 845.827 * eta / 6.048 + 415.51 * e2 / 8.64)
            + cs * (158.0239 * eta / 5.4432 - 451.597 * e2 / 6.048 + 20.45 * e2 * eta / 4.32 + 107.0 * eta * cp / 6.0
                    - 5.0 * e2 * cp / 24.0)
            + 12.0 * kPi * cp - cp * ce * (150.5 / 2.4 + eta / 8.0) + ce * cp * (10.1 * eta / 2.4 + 3.0 * e2 / 8.0);
  e.an[0] = 8.0 * sqrt(kPi / 5.0) * eta;
  e.an[1] = (-107.0 + 55.0 * eta) / 42.0;
  e.an[2] = 2.0 * kPi - 4.0 * ce / 3.0 + 2.0 * eta * cs / 3.0;
  e.an[3] = -2.173 / 1.512 - eta * (10.69 / 2.16 - 2.0 * cp) + 2.047 * e2 / 1.512;
  e.an[4] = -10.7 * kPi / 2.1 + eta * (3.4 * kPi / 2.1);
  e.an[5] = -24.0 * eta;
  e.an[6] = 270.27409 / 6.46800 - 8.56 * eg / 1.05 + 2.0 * pi2 / 3.0 + eta * (4.1 * pi2 / 9.6 - 27.8185 / 3.3264)
            - 20.261 * e2 / 2.772 + 11.4635 * eta * e2 / 9.9792 - 4.28 * log(16.0) / 1.05;
  e.an[7] = D6(4.28 * kPi / 1.05);
  D6 g1 = 4.149e+00 * ce + (-4.070e+00) * cp + (-8.752e+01) * eta * ce + (-4.897e+01) * eta + 6.665e+02 * e2;
  if (g1.v < 0.0) g1 = D6(0.0);
  D6 del1 = (-5.472e-02) * ce + 2.094e-02 * cp + 3.554e-01 * eta * ce + 1.151e-01 * eta + 9.640e-01 * e2;
  D6 del2 = (-1.235e+00) * ce + 3.423e-01 * cp + 6.062e+00 * eta * ce + 5.949e+00 * eta + (-1.069e+01) * e2;
  if (del1.v < 0.0) del1 = D6(0.0);
  if (del2.v < 1.0e-4) del2 = D6(1.0e-4);
  // NS compactness (arXiv:1608.02582 eq. 78) and torus mass (arXiv:1509.00512 eq. 11)
  D6 Comp;
  if (lam.v > 1.0) {
    const D6 ll = dlog(lam);
    Comp = 0.360 + (-0.0355) * ll + 0.000705 * ll * ll;
  } else {
    Comp = 0.5 + (3.0 * 0.360 + 0.0355 - 1.5) * lam * lam + (-2.0 * 0.360 - 0.0355 + 1.0) * lam * lam * lam;
  }
  const D6 xi = xitide_interp(xit, Comp, q, chi1);
  const D6 z1 = 1.0 + dcbrt(1.0 - chi1 * chi1) * (dcbrt(1.0 + chi1) + dcbrt(1.0 - chi1));
  const D6 z2 = dsqrt(3.0 * chi1 * chi1 + z1 * z1);
  const D6 rr = dsqrt((3.0 - z1) * (3.0 + z1 + 2.0 * z2));
  const D6 r_isco = chi1.v > 0.0 ? 3.0 + z2 - rr : 3.0 + z2 + rr;
  D6 Mtor = 0.296 * xi * (1.0 - 2.0 * Comp) - 0.171 * q * Comp * r_isco;
  if (!(Mtor.v > 0.0)) Mtor = D6(0.0);
  // 22 quasi-normal mode of the remnant (complex fit in kappa)
  const D6 kp = dsqrt(dlog(2.0 - chif) / log(3.0));
  const double ca[5] = {1.5578, 1.9510, 2.0997, 1.4109, 0.4106}, cb[5] = {2.9031, 5.9210, 2.7606, 5.9143, 2.7952};
  D6 sre(0.0), sim(0.0);
  for (int n = 4; n >= 0; --n) {
    sre = sre * kp + ca[n] * cos(cb[n]);
    sim = sim * kp + ca[n] * sin(cb[n]);
  }
  const D6 om_re = 1.0 + kp * sre, om_im = kp * sim;
  const D6 frA = 0.5 * om_re / kPi / mfin;
  const D6 rt = xi * (1.0 - 2.0 * Comp) / (q * Comp);
  const D6 qf = 0.5 * om_re / om_im;
  const D6 ftide = dabs(1.0 / (kPi * (chi1 + dsqrt(rt * rt * rt))) * (1.0 + 1.0 / q));
  const D6 frt = (0.99 * 0.98) * frA;
  const D6 gcorr = lam.v > 1.0 ? D6(1.25) : 1.0 + 0.5 * lam - 0.25 * lam * lam;
  const D6 u = ftide / frt - 1.0;
  const D6 d2p = lam.v > 1.0 ? 1.62496 * 0.25 * (1.0 + dtanh(4.0 * (u - 0.0188092) / 0.338737))
                             : del2 - 2.0 * (del2 - 0.81248) * lam + (del2 - 0.81248) * lam * lam;
  const D6 sig = d2p * frA / qf;
  const bool low = ftide.v < frA.v;
  const D6 eps_tide = low ? D6(0.0) : 0.5 * (1.0 + dtanh(4.0 * ((u * u - 0.571505 * Comp - 0.00508451 * chi1) + 0.0796251) / 0.0801192));
  const D6 X = 1.29971 - 1.61724 * (Mtor + 0.424912 * Comp + 0.363604 * dsqrt(eta) - 0.0605591 * chi1);
  const D6 eps_ins = low ? (X.v > 1.0 ? D6(1.0) : X) : (Mtor.v > 0.0 ? X : D6(1.0));
  const D6 Y = 0.137722 - 0.293237 * (Mtor - 0.132754 * Comp + 0.576669 * dsqrt(eta) - 0.0603749 * chi1
                                      - 0.0601185 * chi1 * chi1 - 0.0729134 * chi1 * chi1 * chi1);
  const D6 W = 0.5 * (1.0 - dtanh(4.0 * ((u * u - 0.657424 * Comp - 0.0259977 * chi1) + 0.206465) / 0.226844));
  const D6 sig_tide = low ? (Mtor.v > 0.0 ? Y : 0.5 * Y + W) : W;
  // window centres, in M f (gwfast writes them in Hz and multiplies back by M G)
  const D6& MG = k.MG;
  const D6 ring_end = lam.v > 1.0 ? frt : (1.0 - 0.02 * lam + 0.01 * lam * lam) * 0.98 * frA;
  const D6 f0pn = low ? (Mtor.v > 0.0 ? ftide : (1.0 - 1.0 / q) * frt + eps_ins * ftide / q) : ring_end;
  const D6 f0pm = low ? (Mtor.v > 0.0 ? ftide : (1.0 - 1.0 / q) * frt + ftide / q) : ring_end;
  e.c0pn = eps_ins * ((f0pn / MG) * MG);
  e.c0pm = (f0pm / MG) * MG;
  e.c0rd = low ? D6(0.0) : (ring_end / MG) * MG;
  e.wsc = 4.0 / (0.015 + sig_tide);
  e.aPM = gcorr * g1;
  e.aRD = eps_tide * del1;
  e.frA = frA;
  e.sig = sig;
}

// amplitude and phase of IMRPhenomNSBH at physical frequency f (Hz)
template <class S, class C>
__device__ __forceinline__ void nsbh_point(const NSBHEvT<C>& e, typename Real<S>::T f, S& amp, S& phase) {
  typedef typename Real<S>::T T;
  const PhdCoreT<C>& k = e.k;
  const S x = co<S>(k.MG) * f;
  const T xv = val(x);
  const S one(T(1));
  const S px = T(kPi) * x;
  const S v = dcbrt(px), v2 = v * v;
  const S lv2 = T(2) * dlog(v);
  const S px2 = px * px;
  const S xdot = co<S>(e.xd[0]) * (v2 * v2 * v2 * v2 * v2)
                 * (T(1) + co<S>(e.xd[1]) * v2 + co<S>(e.xd[2]) * px + co<S>(e.xd[3]) * px * v + co<S>(e.xd[4]) * v2 * px
                    + (co<S>(e.xd[5]) + T(-856. / 105.) * lv2) * px2 + co<S>(e.xd[6]) * v * px2);
  const S aft = dsqrt(dabs(T(kPi) / (T(1.5) * v * xdot)));
  const S base = aft * co<S>(e.an[0]) * v2;
  const S re = base * (T(1) + co<S>(e.an[1]) * v2 + co<S>(e.an[2]) * px + co<S>(e.an[3]) * v * px + co<S>(e.an[4]) * v2 * px
                       + (co<S>(e.an[6]) + T(-428. / 105.) * lv2) * px2);
  const S im = base * (co<S>(e.an[5]) * v2 * px + co<S>(e.an[7]) * px2);
  const S aPN = dsqrt(re * re + im * im);
  const S x56 = dexp(T(5.0 / 6.0) * dlog(x));
  const S aPM = co<S>(e.aPM) * x56;
  const S sg = co<S>(e.sig);
  const S dr = x - co<S>(e.frA);
  const S LRD = sg * sg / (dr * dr + sg * sg * T(0.25));
  const S aRD = co<S>(e.aRD) * LRD / (x * dsqrt(dcbrt(x)));
  const S wsc = co<S>(e.wsc);
  const S wpn = T(0.5) * (T(1) - dtanh(wsc * (x - co<S>(e.c0pn))));
  const S wpm = T(0.5) * (T(1) - dtanh(wsc * (x - co<S>(e.c0pm))));
  const S wrd = T(0.5) * (T(1) + dtanh(wsc * (x - co<S>(e.c0rd))));
  amp = xv < T(kMfCut) ? co<S>(k.ampPref) * (aPN * wpn + aPM * wpm + aRD * wrd) : S(T(0));
  S ph = complete_phase(k, x, co<S>(k.C1MRD), co<S>(k.C2MRD), one, one);
  if (xv < T(kMfCut)) {
    const S x13 = v;
    const S num = T(1) + x13 * x13 * T(-12.615214237993088) + px * T(19.0537346970349)
                  + x13 * px * T(-21.166863146081035) + x13 * x13 * px * T(90.55082156324926) + px * px * T(-60.25357801943598);
    const S den = T(1) + x13 * x13 * T(-15.11120782773667) + px * T(22.195327350624694) + x13 * px * T(8.064109635305156);
    const S tidal_ph = co<S>(e.tidP) * (x13 * x13 * px) * num / den;
    ph = ph - co<S>(k.t0) * (x - co<S>(k.fRef)) - co<S>(k.phiRef) + T(kPi) + tidal_ph;
  }
  phase = ph;
}

// ------------------------------------------------------------------ IMRPhenomHM (gwfast/waveforms.py:2256-2616)
template <class C> struct HMModeT {
  C rho, tau, C1, C2, frlm;
  C fip, amp_, bmp, PhDB, PhDC, PhDBA, phC;  // phase frequency map and offsets
  C fia, ama, bma;                          // amplitude frequency map
  C hr1, hr2, hr3, hr4, hi4;                // PN amplitude polynomial H(v) = v (hr1 + v (hr2 + v (hr3 + v (hr4 + i hi4))))
  double yp, yc, dyp, dyc;                  // 0.5(Y +- (-1)^l Y_{l-m}) and d/diota
  double ysp, ysm;                          // yp - yc = (-1)^l Y_{l-m} and yp + yc = Y, formed directly
  double shift;
  int l, m;
};
using HMMode = HMModeT<D4>;

template <class C> struct HMEvT {
  PhdCoreT<C> k;
  C phi0;
  HMModeT<C> md[6];
};
using HMEv = HMEvT<D4>;

__device__ inline void rd_fit(int mode, const D4& finmass, const D4& finspin, D4& fr, D4& fd) {
  const int l = kModeL[mode], m = kModeM[mode];
  const D4 alpha = dlog(2.0 - finspin) / log(3.0);
  const double beta = 1.0 / (2.0 + l - (m < 0 ? -m : m));
  const D4 kap = dpowc(alpha, beta);
  D4 re(0.0), im(0.0), kp(1.0);
  for (int j = 0; j < 7; ++j) {
    double s, c;
    sincos(kRDPhase[mode][j], &s, &c);
    re = re + (kRDMod[mode][j] * c) * kp;
    im = im + (kRDMod[mode][j] * s) * kp;
    kp = kp * kap;
  }
  const D4 den = (2.0 * kPi) * finmass;
  fr = re / den;
  fd = im / den;
}

// spin-weighted harmonics Y_lm, Y_l-m (s = -2, phi = 0) and their iota derivatives, gwfast/waveforms.py:2517-2524
__device__ inline void sw_harm(int mode, double iota, double& Y, double& Ym, double& dY, double& dYm) {
  typedef Dual<double, 1> D1;
  const D1 io = D1::seed(iota, 0);
  D1 c, s, ch, sh;
  dsincos(io, &s, &c);
  dsincos(io * 0.5, &sh, &ch);
  D1 y, ym;
  switch (mode) {
    case 0: y = sqrt(5.0 / (16.0 * kPi)) * s * (1.0 + c); ym = sqrt(5.0 / (16.0 * kPi)) * s * (1.0 - c); break;
    case 1: y = sqrt(5.0 / (64.0 * kPi)) * (1.0 + c) * (1.0 + c); ym = sqrt(5.0 / (64.0 * kPi)) * (1.0 - c) * (1.0 - c); break;
    case 2: { const D1 c2 = ch * ch; y = sqrt(7.0 / kPi) * c2 * c2 * (3.0 * c - 2.0) * 0.5;
              const D1 s2 = sh * sh; ym = sqrt(7.0 / (4.0 * kPi)) * (2.0 + 3.0 * c) * s2 * s2; break; }
    case 3: { const D1 c2 = ch * ch; const D1 s2 = sh * sh;
              y = -sqrt(21.0 / (2.0 * kPi)) * c2 * c2 * ch * sh; ym = sqrt(21.0 / (2.0 * kPi)) * ch * s2 * s2 * sh; break; }
    case 4: { const D1 c2 = ch * ch; const D1 s2 = sh * sh;
              y = -3.0 * sqrt(7.0 / (2.0 * kPi)) * c2 * c2 * ch * (2.0 * c - 1.0) * sh;
              ym = 3.0 * sqrt(7.0 / (2.0 * kPi)) * ch * (1.0 + 2.0 * c) * s2 * s2 * sh; break; }
    default: { const D1 c2 = ch * ch; const D1 s2 = sh * sh;
               y = 3.0 * sqrt(7.0 / kPi) * c2 * c2 * c2 * s2; ym = 3.0 * sqrt(7.0 / kPi) * c2 * s2 * s2 * s2; break; }
  }
  Y = y.v; Ym = ym.v; dY = y.d[0]; dYm = ym.d[0];
}

// the detector-dependent part of the IMRPhenomHM record (the modes depend on the source alone);
// hphc uses the amplitude peak (no modulus in the second branch) for t0 as well (gwfast/waveforms.py:2433, :2527)
__device__ inline void hm_ref(HMEv& e, double fmin_hz) {
  phenom_ref_setup(e.k, e.k.fpA, fmin_hz, e.k.C1MRD, e.k.C2MRD);
  e.phi0 = 0.5 * e.k.phiRef;
}

__device__ inline void hm_setup_core(HMEv& e, const D4& Mc, const D4& eta, const D4& chi1, const D4& chi2, double dL,
                                     double fmin_hz) {
  PhdCore& k = e.k;
  const D4 af = final_spin(eta, chi1, chi2);
  const D4 finmass = 1.0 - radiated_energy(eta, chi1, chi2);
  D4 fr, fd;
  rd_fit(1, finmass, af, fr, fd);
  phenom_core_setup(k, Mc, eta, chi1, chi2, fr, fd);
  hm_ref(e, fmin_hz);
  const D4 M = k.MG * (1.0 / kG3);   // total mass Mc / eta^(3/5) (MG = M G/c^3)
  // M G/c^2[Gpc] M G/c^3 / dL * sqrt(2 eta/3) pi^(-1/6)   (gwfast/waveforms.py:2444, :2489)
  k.ampPref = (kG2Gpc * kG3 / dL * pow(kPi, -1.0 / 6.0)) * M * M * dsqrt(eta * (2.0 / 3.0));
}

// af, finmass: the remnant's spin and mass (final_spin, 1 - radiated_energy), the same for every mode
__device__ inline void hm_setup_mode(HMEv& e, int mode, const D4& eta, const D4& chi1, const D4& chi2, double iota,
                                     const D4& af, const D4& finmass) {
  PhdCore& k = e.k;
  HMMode& md = e.md[mode];
  const int l = kModeL[mode], m = kModeM[mode];
  md.l = l; md.m = m;
  const double shifts[5] = {0.0, 0.5 * kPi, 0.0, -0.5 * kPi, kPi};
  md.shift = shifts[m];
  D4 frlm, fdlm;
  rd_fit(mode, finmass, af, frlm, fdlm);
  md.frlm = frlm;
  md.rho = k.fring / frlm;
  md.tau = fdlm / k.fdamp;
  const D4& rho = md.rho;
  const D4& tau = md.tau;
  const D4& fm = k.fMRD;
  const D4 u = (fm - k.alp[4] * k.fring) / (k.fdamp * rho * tau);
  const D4 dmrd = (k.alp[0] + k.alp[1] / (fm * fm) + k.alp[2] / dsqrt(dsqrt(fm)) + k.alp[3] / (k.fdamp * tau * (1.0 + u * u))) / k.eta;
  md.C2 = k.DPhiIntTemp - dmrd;
  md.C1 = k.PhiIntTemp - mrd_phase_raw<D4>(k, fm, rho, tau) - md.C2 * fm;
  // phase map (gwfast/waveforms.py:2544-2563, :2587-2597)
  const double ai = 2.0 / m;
  md.fip = kPhiFJoin / rho;
  const D4 Ti = md.fip * ai;
  md.amp_ = (frlm * rho - Ti) / (frlm - md.fip);
  md.bmp = Ti - md.fip * md.amp_;
  md.PhDB = complete_phase<D4>(k, md.amp_ * md.fip + md.bmp, md.C1, md.C2, rho, tau) / md.amp_;
  md.PhDC = complete_phase<D4>(k, rho * frlm, md.C1, md.C2, rho, tau) / rho;
  md.PhDBA = complete_phase<D4>(k, md.fip * ai, md.C1, md.C2, rho, tau) / ai;
  md.phC = md.PhDBA - md.PhDB + complete_phase<D4>(k, md.amp_ * frlm + md.bmp, md.C1, md.C2, rho, tau) / md.amp_;
  // amplitude map (gwfast/waveforms.py:2546-2568)
  md.fia = kAmpFJoin / rho;
  const D4 Tia = md.fia * ai;
  md.ama = (k.fring - Tia) / (frlm - md.fia);
  md.bma = Tia - md.fia * md.ama;
  // PN amplitude H_lm(v) = v (hr1 + v (hr2 + v (hr3 + v (hr4 + i hi4))))  (gwfast/waveforms.py:2511)
  const D4 seta = seta_of(eta);
  const D4 chis = 0.5 * (chi1 + chi2), chia = 0.5 * (chi1 - chi2);
  const D4 z(0.0);
  md.hr1 = z; md.hr2 = z; md.hr3 = z; md.hr4 = z; md.hi4 = z;
  switch (mode) {
    case 0: {
      const double s = sqrt(2.0) / 3.0;
      md.hr1 = s * seta;
      md.hr2 = -1.5 * s * (chia + seta * chis);
      md.hr3 = s * seta * (335.0 / 672.0 + 117.0 / 56.0 * eta);
      md.hr4 = s * (chia * (3427.0 / 1344. - 2101.0 / 336. * eta) + seta * chis * (3427.0 / 1344. - 965.0 / 336. * eta) - kPi * seta);
      md.hi4 = s * seta * (-0.5 - 2.0 * 0.69314718056);
      break;
    }
    case 1: md.hr1 = D4(1.0); break;  // H22 = 1 handled as a constant below
    case 2: md.hr2 = (sqrt(5.0 / 7.0) / 3.0) * (1.0 - 3.0 * eta); break;
    case 3: md.hr1 = (0.75 * sqrt(5.0 / 7.0)) * seta; break;
    case 4: md.hr3 = (0.75 * sqrt(3.0 / 35.0)) * seta * (1.0 - 2.0 * eta); break;
    default: md.hr2 = (4.0 / 9.0 * sqrt(10.0 / 7.0)) * (1.0 - 3.0 * eta); break;
  }
  double Y, Ym, dY, dYm;
  sw_harm(mode, iota, Y, Ym, dY, dYm);
  const double sg = (l % 2 == 0) ? 1.0 : -1.0;
  md.yp = 0.5 * (Y + sg * Ym);
  md.yc = 0.5 * (Y - sg * Ym);
  md.dyp = 0.5 * (dY + sg * dYm);
  md.dyc = 0.5 * (dY - sg * dYm);
  md.ysp = sg * Ym;
  md.ysm = Y;
}

// |H_lm(v)| for v = (2 pi x / m)^(1/3)
template <class S, class C>
__device__ __forceinline__ S hm_absH(const HMModeT<C>& md, int mode, const S& x) {
  typedef typename Real<S>::T T;
  if (mode == 1) return S(T(1));
  const S v = dcbrt(x * T(kTwoPi / md.m));
  const S re = v * (co<S>(md.hr1) + v * (co<S>(md.hr2) + v * (co<S>(md.hr3) + v * co<S>(md.hr4))));
  if (mode == 0) {
    const S v2 = v * v;
    const S im = v2 * v2 * co<S>(md.hi4);
    return dsqrt(re * re + im * im);
  }
  return dabs(re);
}

template <class S> struct Cplx { S re, im; };

// hp, hc of IMRPhenomHM without the common factor; returns P, C with hp = P, hc = i C, plus the iota derivatives
// (dP, dC, value-only).  Point at physical frequency f (Hz).
template <class S, class K>
__device__ __forceinline__ void hm_point(const HMEvT<K>& e, typename Real<S>::T f, Cplx<S>& P, Cplx<S>& C,
                                         Cplx<typename Real<S>::T>& dP, Cplx<typename Real<S>::T>& dC) {
  typedef typename Real<S>::T T;
  const PhdCoreT<K>& k = e.k;
  const S x = co<S>(k.MG) * f;
  const T xv = val(x);
  const S zero(T(0));
  P.re = zero; P.im = zero; C.re = zero; C.im = zero;
  dP.re = T(0); dP.im = T(0); dC.re = T(0); dC.im = T(0);
  const S lin = co<S>(k.t0) * (x - co<S>(k.fRef));
#pragma unroll 1
  for (int mode = 0; mode < 6; ++mode) {
    const HMModeT<K>& md = e.md[mode];
    const T ai = T(2.0) / T(md.m);
    // amplitude
    S fs;
    if (xv < T(val(md.fia))) fs = x * ai;
    else if (xv < T(val(md.frlm))) fs = x * co<S>(md.ama) + co<S>(md.bma);
    else fs = x - co<S>(md.frlm) + co<S>(k.fring);
    S amp = co<S>(k.ampPref) * (T(1) / (fs * dsqrt(dcbrt(fs)))) * complete_amp_shape(k, fs);
    if (mode != 1) {
      const S h1 = hm_absH(md, mode, x);
      const S h2 = hm_absH(md, mode, x * ai);
      const S h3 = hm_absH(md, mode, fs);
      amp = amp * h1 * h3 / h2;
      if (!(val(amp) == val(amp))) amp = zero;  // nan_to_num at equal mass (gwfast/waveforms.py:2582)
    }
    // phase
    S ph;
    const S rho = co<S>(md.rho), tau = co<S>(md.tau), C1 = co<S>(md.C1), C2 = co<S>(md.C2);
    if (xv < T(val(md.fip))) ph = complete_phase(k, x * ai, C1, C2, rho, tau) / ai;
    else if (xv < T(val(md.frlm)))
      ph = co<S>(md.PhDBA) - co<S>(md.PhDB) + complete_phase(k, x * co<S>(md.amp_) + co<S>(md.bmp), C1, C2, rho, tau) / co<S>(md.amp_);
    else ph = co<S>(md.phC) - co<S>(md.PhDC) + complete_phase(k, x * rho, C1, C2, rho, tau) / rho;
    ph = ph - lin - T(md.m) * co<S>(e.phi0) + T(md.shift);
    S sn, cs;
    dsincos(ph, &sn, &cs);
    // M = amp e^{-i ph}
    const S mre = amp * cs, mim = -(amp * sn);
    const T yp = T(md.yp), yc = T(md.yc);
    P.re = P.re + yp * mre; P.im = P.im + yp * mim;
    C.re = C.re + yc * mre; C.im = C.im + yc * mim;
    dP.re += T(md.dyp) * val(mre); dP.im += T(md.dyp) * val(mim);
    dC.re += T(md.dyc) * val(mre); dC.im += T(md.dyc) * val(mim);
  }
}

}  // namespace gwf
