// Fused SNR and Fisher kernels: one CTA per (event, detector).
//
// Per frequency point a thread evaluates the waveform and its analytic tangent, the
// detector projection (with Earth rotation when enabled) and the 11 complex
// derivatives of the strain; the overall factor exp(i(2 pi f tcoal + phiL - Phicoal))
// is common to every derivative and cancels in Re<d_a h|d_b h>, so it is never formed.
// Each warp stages its 32 points' weighted derivatives in shared memory and the lanes
// accumulate the upper triangle of the 11x11 Gram matrix; the four warps are summed at
// the end.  Reference: gwfast/signal.py:658-777 (SNR), :782-1098 (Fisher),
// :1303-1584 (closed-form extrinsic derivatives, which are exact derivatives).
#pragma once
#include "gwf_model.cuh"

namespace gwf {

constexpr int kThreads = 128;
constexpr int kWarps = kThreads / 32;

// Per-event kernels (set-up records, projections, condition numbers) run one thread per event,
// epw events per warp (lanes >= epw idle), kEvBlock threads per block. Their FP64 chains are long
// and latency-bound: a batch too small to give every SM sub-partition a few warps runs faster
// spread over more, partly filled warps than packed into full ones (ev_lanes on the host).
constexpr int kEvBlock = 64;
__device__ __forceinline__ long long ev_thread(int epw) {
  const int lane = threadIdx.x & 31;
  if (lane >= epw) return -1;
  return ((long long)blockIdx.x * (kEvBlock / 32) + (threadIdx.x >> 5)) * epw + lane;
}
constexpr int NP = 11;    // Fisher parameters
constexpr int NE = 66;    // upper-triangle entries
// Fisher order: Mc, eta, dL, theta, phi, iota, psi, tcoal, Phicoal, chi1z, chi2z
// (the tidal TaylorF2, model 3, appends LambdaTilde, deltaLambda)
enum { I_MC = 0, I_ETA, I_DL, I_TH, I_PH, I_IO, I_PS, I_TC, I_PC, I_C1, I_C2, I_LT, I_DLT };

// Fisher parameters of a model, upper-triangle entries, entries plus strain products, entry index
// Fisher parameters: 11; the tidal models (3, 4) add LambdaTilde, deltaLambda; the eccentric
// TaylorF2 adds ecc after them (5: 12 parameters, 6: with the tidal terms, 14)
template <int MODEL> __host__ __device__ constexpr int np_of() {
  return MODEL == 5 ? 12 : (MODEL == 6 ? 14 : (MODEL >= 3 ? 13 : 11));
}
template <int MODEL> __host__ __device__ constexpr bool is_tf2() { return MODEL == 0 || MODEL == 3 || MODEL == 5 || MODEL == 6; }
template <int MODEL> __host__ __device__ constexpr bool has_tidal() { return MODEL == 3 || MODEL == 4 || MODEL == 6 || MODEL == 7; }
template <int MODEL> __host__ __device__ constexpr bool has_ecc() { return MODEL == 5 || MODEL == 6; }
template <int MODEL> __host__ __device__ constexpr int ecc_col() { return MODEL == 6 ? 13 : 11; }
// intrinsic tangent directions of the per-event duals: Mc, eta, chi1z, chi2z (+ LambdaTilde,
// deltaLambda for IMRPhenomD_NRTidalv2, model 4, whose set-up depends on them non-linearly)
template <int MODEL> __host__ __device__ constexpr int ndir_of() { return (MODEL == 4 || MODEL == 7) ? 6 : 4; }
template <int MODEL> using DualOf = Dual<double, ndir_of<MODEL>()>;
__host__ __device__ constexpr int ne_of(int npr) { return npr * (npr + 1) / 2; }
__host__ __device__ constexpr int nex_of(int npr) { return ne_of(npr) + npr; }
__host__ __device__ constexpr int pidx_n(int npr, int a, int b) { return a * npr - a * (a - 1) / 2 + (b - a); }
// (a, b), a <= b, of upper-triangle entry e
__host__ __device__ inline void pair_n(int npr, int e, int& a, int& b) {
  a = 0;
  while (e >= npr - a) { e -= npr - a; ++a; }
  b = a + e;
}

struct DetDev {
  double lat, lon, xax;  // radians
  double sin_zeta;       // sine of the angle between the arms
  double fmin, fmax;     // fmax <= 0 means none
  int shape;             // 0 = L, 1 = triangle
  int earth;             // Earth rotation
  const double* psd_f;
  const double* psd_S;
  int npsd;
  const int* acc;        // log-frequency bin -> table index (accelerates the PSD lookup)
  int nacc;
  double acc_l0, acc_idl;
  // FP32 copy for the split-precision kernels, as linear segments (one 16-byte load per step):
  // segment j is (f_j, f_j+1, S_j / psd_scale, slope), the slope formed in FP64 and rounded once
  const float4* psd_seg;
  float psd_f32_lo, psd_f32_hi;   // first and last table frequency (FP32)
  double psd_scale;
  // sines and cosines of the latitude, twice the latitude and twice the angle of each arm (the arms
  // at xax and xax + 60 degrees), set on the host by det_trig: constants of the detector, which the
  // per-event projection set-up would otherwise evaluate for every event
  double sl, cl, s2l, c2l;
  double s2g[2], c2g[2];
};

__host__ inline void det_trig(DetDev& d) {
  d.sl = sin(d.lat);
  d.cl = cos(d.lat);
  d.s2l = sin(2.0 * d.lat);
  d.c2l = cos(2.0 * d.lat);
  for (int a = 0; a < 2; ++a) {
    const double g = d.xax + a * (3.14159265358979323846 / 3.0);
    d.s2g[a] = sin(2.0 * g);
    d.c2g[a] = cos(2.0 * g);
  }
}

struct EvBatch {
  const double* p;       // parameters, [11][ld] (Fisher order)
  long long ld;
  long long N;
  long long n0;          // first event of this launch
  int res;
  const int* res_ev;     // optional per-event grid length
  int spacing;           // 0 = geometric, 1 = linear
  const double* fcut_ev = nullptr;   // optional per-event upper grid frequency (replaces the model cut and fmax)
  const double* fmin_ev = nullptr;   // optional per-event lower frequency (replaces the detector's fmin in the
                                     // set-up: the models' reference frequency is the lowest of the event's points)
};

struct WfDesc {
  int model;             // 0 = TaylorF2, 1 = IMRPhenomD, 2 = IMRPhenomHM, 3 = tidal TaylorF2,
                         // 4 = IMRPhenomD_NRTidalv2, 5 = eccentric TaylorF2, 6 = tidal eccentric TaylorF2
  int spin_ho;
  double fcut_par;       // TaylorF2: fHigh in Hz; IMR: cut in Mf
  int flags;             // TaylorF2 options: kTF2Vlso | kTF2KerrIsco | kTF2QuadMon
  int pad_;
  double fref_ecc;       // eccentric TaylorF2: reference frequency of ecc in Hz (<= 0: lowest grid frequency)
  const double* xitide = nullptr;   // IMRPhenomNSBH: the xi_tide table on the device (200^3)
};

static __constant__ unsigned char kPairA[NE] = {0,0,0,0,0,0,0,0,0,0,0,1,1,1,1,1,1,1,1,1,1,2,2,2,2,2,2,2,2,2,3,3,3,3,3,3,3,3,4,4,4,4,4,4,4,5,5,5,5,5,5,6,6,6,6,6,7,7,7,7,8,8,8,9,9,10};
static __constant__ unsigned char kPairB[NE] = {0,1,2,3,4,5,6,7,8,9,10,1,2,3,4,5,6,7,8,9,10,2,3,4,5,6,7,8,9,10,3,4,5,6,7,8,9,10,4,5,6,7,8,9,10,5,6,7,8,9,10,6,7,8,9,10,7,8,9,10,8,9,10,9,10,10};

struct cd { double re, im; };
__device__ __forceinline__ cd cmul(cd a, cd b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__device__ __forceinline__ cd cadd(cd a, cd b) { return {a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ cd cscale(cd a, double s) { return {a.re * s, a.im * s}; }
__device__ __forceinline__ cd cmuli(cd a) { return {-a.im, a.re}; }  // i * a

// np.interp(f, psd_f, psd_S, left=1, right=1) (gwfast/signal.py:723, :901)
__device__ __forceinline__ double psd_at(const DetDev& d, double f, double lnf) {
  const double* xf = d.psd_f;
  const int n = d.npsd;
  if (!(f >= xf[0]) || f > xf[n - 1]) return 1.0;
  int b = (int)((lnf - d.acc_l0) * d.acc_idl);
  b = b < 0 ? 0 : (b >= d.nacc ? d.nacc - 1 : b);
  int j = d.acc[b];
  while (j > 0 && xf[j] > f) --j;
  while (j < n - 2 && xf[j + 1] <= f) ++j;
  const double x0 = xf[j], x1 = xf[j + 1];
  const double y0 = d.psd_S[j], y1 = d.psd_S[j + 1];
  return y0 + (f - x0) * ((y1 - y0) / (x1 - x0));
}

// ------------------------------------------------------------------ per-event shared state
struct GridEv {
  double fmin, fcut, lnfmin, delta, fac_w, w0, wl;  // geometric: delta = ln step
  double df;                                         // linear
  int R;
  int ok;
};

// pattern-function constants of one event seen by one detector (gwfast/signal.py:342-387)
struct ProjEv {
  double c2p, s2p;               // cos/sin 2 psi
  double cp, ci, dcp, dci;       // (1+cos^2 i)/2, cos i and d/diota
  double KA1[3], KA2[2], KB1[2], KB2[2];     // x-harmonic coefficients
  double dKA1[3], dKA2[2], dKB1[2], dKB2[2]; // their d/d(dec)
  double s2g[2], c2g[2];         // per computed arm
  double Rc, cdcl, sdsl, sdcl, cdsl;  // Earth-centre delay pieces
  double u0;                     // lon - ra (plus 2 pi t added per point)
  double tc, dL;
};

// pattern functions and their partial derivatives for one arm
struct ArmPat {
  double Fp, Fc;
  double Fp_x, Fc_x;   // d/dx, x = ra - lon - 2 pi t
  double Fp_d, Fc_d;   // d/d(dec) at fixed x
  double Fp_s, Fc_s;   // d/dpsi
};

struct TimeState {
  double D, D_th, D_ph, D_t;  // Earth-centre delay (s) and its derivatives (t in days)
  double x;
};

__device__ __forceinline__ void proj_setup(ProjEv& pj, const DetDev& d, double theta, double phi, double iota,
                                           double psi, double tc, double dL) {
  const double dec = 0.5 * kPi - theta;
  double sd, cdd, s2ps, c2ps, si, ci;
  sincos(dec, &sd, &cdd);
  const double s2d = 2.0 * sd * cdd, c2d = (cdd - sd) * (cdd + sd);   // (double angle)
  sincos(2.0 * psi, &s2ps, &c2ps);
  sincos(iota, &si, &ci);
  pj.c2p = c2ps; pj.s2p = s2ps;
  pj.cp = 0.5 * (1.0 + ci * ci); pj.ci = ci;
  pj.dcp = -ci * si; pj.dci = -si;
  const double sl = d.sl, cl = d.cl, s2l = d.s2l, c2l = d.c2l;
  // a = s2g*A1 + c2g*A2 ; b = c2g*B1 + s2g*B2 with
  // A1 = KA1[0] cos2x + KA1[1] cos x + KA1[2];  A2 = KA2[0] sin2x + KA2[1] sin x
  // B1 = KB1[0] cos2x + KB1[1] cos x;           B2 = KB2[0] sin2x + KB2[1] sin x
  pj.KA1[0] = 0.0625 * (3.0 - c2l) * (3.0 - c2d);  pj.dKA1[0] = 0.0625 * (3.0 - c2l) * 2.0 * s2d;
  pj.KA1[1] = 0.25 * s2l * s2d;                    pj.dKA1[1] = 0.25 * s2l * 2.0 * c2d;
  pj.KA1[2] = 0.75 * cl * cl * cdd * cdd;          pj.dKA1[2] = -0.75 * cl * cl * s2d;
  pj.KA2[0] = -0.25 * sl * (3.0 - c2d);            pj.dKA2[0] = -0.25 * sl * 2.0 * s2d;
  pj.KA2[1] = -0.5 * cl * s2d;                     pj.dKA2[1] = -0.5 * cl * 2.0 * c2d;
  pj.KB1[0] = sl * sd;                             pj.dKB1[0] = sl * cdd;
  pj.KB1[1] = cl * cdd;                            pj.dKB1[1] = -cl * sd;
  pj.KB2[0] = 0.25 * (3.0 - c2l) * sd;             pj.dKB2[0] = 0.25 * (3.0 - c2l) * cdd;
  pj.KB2[1] = 0.5 * s2l * cdd;                     pj.dKB2[1] = -0.5 * s2l * sd;
  for (int a = 0; a < 2; ++a) {   // arms rotated by 0 and 60 degrees
    pj.s2g[a] = d.s2g[a];
    pj.c2g[a] = d.c2g[a];
  }
  pj.Rc = kREarth / kClight;
  pj.cdcl = cdd * cl; pj.sdsl = sd * sl; pj.sdcl = sd * cl; pj.cdsl = cdd * sl;
  pj.u0 = d.lon - phi;
  pj.tc = tc;
  pj.dL = dL;
}

// Earth-centre delay at time tn (days) and x at the detector time (gwfast/signal.py:401-423, :444-453)
__device__ __forceinline__ void time_state(const ProjEv& pj, double tn, TimeState& ts) {
  double su, cu;
  sincos(pj.u0 + kTwoPi * tn, &su, &cu);  // u = lon + 2 pi t - ra
  ts.D = -pj.Rc * (pj.cdcl * cu + pj.sdsl);
  ts.D_th = pj.Rc * (pj.cdsl - pj.sdcl * cu);
  ts.D_ph = -pj.Rc * pj.cdcl * su;
  ts.D_t = kTwoPi * pj.Rc * pj.cdcl * su;
  ts.x = -(pj.u0 + kTwoPi * tn) - kTwoPi * ts.D / kDay;
}

__device__ __forceinline__ void arm_pattern(const ProjEv& pj, double sz, double x, int arm, ArmPat& ap) {
  double sx, cx;
  sincos(x, &sx, &cx);
  const double s2x = 2.0 * sx * cx, c2x = cx * cx - sx * sx;
  const double A1 = pj.KA1[0] * c2x + pj.KA1[1] * cx + pj.KA1[2];
  const double A2 = pj.KA2[0] * s2x + pj.KA2[1] * sx;
  const double B1 = pj.KB1[0] * c2x + pj.KB1[1] * cx;
  const double B2 = pj.KB2[0] * s2x + pj.KB2[1] * sx;
  const double A1x = -2.0 * pj.KA1[0] * s2x - pj.KA1[1] * sx;
  const double A2x = 2.0 * pj.KA2[0] * c2x + pj.KA2[1] * cx;
  const double B1x = -2.0 * pj.KB1[0] * s2x - pj.KB1[1] * sx;
  const double B2x = 2.0 * pj.KB2[0] * c2x + pj.KB2[1] * cx;
  const double A1d = pj.dKA1[0] * c2x + pj.dKA1[1] * cx + pj.dKA1[2];
  const double A2d = pj.dKA2[0] * s2x + pj.dKA2[1] * sx;
  const double B1d = pj.dKB1[0] * c2x + pj.dKB1[1] * cx;
  const double B2d = pj.dKB2[0] * s2x + pj.dKB2[1] * sx;
  const double s2g = pj.s2g[arm], c2g = pj.c2g[arm];
  const double a = s2g * A1 + c2g * A2, b = c2g * B1 + s2g * B2;
  const double ax = s2g * A1x + c2g * A2x, bx = c2g * B1x + s2g * B2x;
  const double ad = s2g * A1d + c2g * A2d, bd = c2g * B1d + s2g * B2d;
  const double c2p = pj.c2p, s2p = pj.s2p;
  ap.Fp = sz * (a * c2p + b * s2p);    ap.Fc = sz * (b * c2p - a * s2p);
  ap.Fp_x = sz * (ax * c2p + bx * s2p); ap.Fc_x = sz * (bx * c2p - ax * s2p);
  ap.Fp_d = sz * (ad * c2p + bd * s2p); ap.Fc_d = sz * (bd * c2p - ad * s2p);
  ap.Fp_s = 2.0 * sz * (b * c2p - a * s2p); ap.Fc_s = 2.0 * sz * (-b * s2p - a * c2p);
}

// strain derivatives of one arm, without the common phase factor.
// hp = P, hc = i C; dP[k], dC[k] are the intrinsic tangents (k = Mc, eta, chi1, chi2),
// dPi/dCi the iota derivatives; dtn[k] = d t_noloc / d theta_k (days).
template <int NI = 4>
__device__ __forceinline__ void arm_derivs(const ProjEv& pj, const ArmPat& ap, const TimeState& ts, double f,
                                           cd P, cd C, const cd* dP, const cd* dC, cd dPi, cd dCi,
                                           const double* dtn, cd* out) {
  const cd hp = P, hc = cmuli(C);
  const cd H = cadd(cscale(hp, ap.Fp), cscale(hc, ap.Fc));
  const cd iH = cmuli(H);
  const double tpf = kTwoPi * f;
  const double G = 1.0 + ts.D_t / kDay;                        // d t / d t_noloc
  // chain through x = ra - lon - 2 pi t and dec = pi/2 - theta
  const double x_th = -kTwoPi * ts.D_th / kDay;
  const double x_ph = 1.0 - kTwoPi * ts.D_ph / kDay;
  const double x_tc = -kTwoPi * G;
  const cd hx = cadd(cscale(hp, ap.Fp_x), cscale(hc, ap.Fc_x)); // d(h)/dx at fixed waveform
  const cd hd = cadd(cscale(hp, ap.Fp_d), cscale(hc, ap.Fc_d)); // d(h)/d(dec)
  const int map[6] = {I_MC, I_ETA, I_C1, I_C2, I_LT, I_DLT};
#pragma unroll
  for (int k = 0; k < NI; ++k) {
    cd v = cadd(cscale(cmuli(dC[k]), ap.Fc), cscale(dP[k], ap.Fp));
    if (dtn[k] != 0.0) {
      v = cadd(v, cscale(hx, -kTwoPi * G * dtn[k]));
      v = cadd(v, cscale(iH, tpf * ts.D_t * dtn[k]));
    }
    out[map[k]] = v;
  }
  out[I_IO] = cadd(cscale(dPi, ap.Fp), cscale(cmuli(dCi), ap.Fc));
  out[I_DL] = cscale(H, -1.0 / pj.dL);
  out[I_TH] = cadd(cadd(cscale(hx, x_th), cscale(hd, -1.0)), cscale(iH, tpf * ts.D_th));
  out[I_PH] = cadd(cscale(hx, x_ph), cscale(iH, tpf * ts.D_ph));
  out[I_PS] = cadd(cscale(hp, ap.Fp_s), cscale(hc, ap.Fc_s));
  out[I_TC] = cscale(cadd(cscale(hx, x_tc), cscale(iH, tpf * (kDay + ts.D_t))), 1.0 / kDay);
  out[I_PC] = cscale(iH, -1.0);
}

// ------------------------------------------------------------------ event setup (one thread)
union EvUnion {
  TF2Ev tf2;
  PhdEv phd;
  HMEv hm;
  TF2TEv tf2t;
  NRTEv nrt;
  TF2EEv tf2e;
  NSBHEv nsbh;
};

// Kerr ISCO radius (prograde for chi > 0), gwfast/waveforms.py:934-937
__host__ __device__ inline double r_isco_kerr(double chi) {
  const double z1 = 1.0 + cbrt(1.0 - chi * chi) * (cbrt(1.0 + chi) + cbrt(1.0 - chi));
  const double z2 = sqrt(3.0 * chi * chi + z1 * z1);
  const double r = sqrt((3.0 - z1) * (3.0 + z1 + 2.0 * z2));
  return chi > 0.0 ? 3.0 + z2 - r : 3.0 + z2 + r;
}

// twice the ISCO frequency of the Kerr remnant (gwfast/waveforms.py:921-951: final spin and mass from
// the fits of arXiv:1605.01938, arXiv:2108.05861 App. C), in Hz
__host__ __device__ inline double tf2_kerr_fcut(double Mc, double eta, double chi1, double chi2) {
  const double eta2 = eta * eta;
  const double Mtot = Mc / pow(eta, 0.6);
  const double sv = eta < 0.25 ? sqrt(1.0 - 4.0 * eta) : 0.0;
  const double m1 = 0.5 * (1.0 + sv), m2 = 0.5 * (1.0 - sv);
  const double s = (m1 * m1 * chi1 + m2 * m2 * chi2) / (m1 * m1 + m2 * m2);
  const double q = m2 / m1;
  const double atot = (chi1 + chi2 * q * q) / ((1.0 + q) * (1.0 + q));
  const double aeff = atot + 0.41616 * eta * (chi1 + chi2);
  const double r_isco = r_isco_kerr(aeff);
  const double ens = eta * (0.055974469826360077 + 0.5809510763115132 * eta - 0.9606726679372312 * eta2
                            + 3.352411249771192 * eta2 * eta);
  const double erad = ens * (1.0 + (-0.0030302335878845507 - 2.0066110851351073 * eta + 7.7050567802399215 * eta2) * s)
                      / (1.0 + (-0.6714403054720589 - 1.4756929437702908 * eta + 7.304676214885011 * eta2) * s);
  const double Mfin = Mtot * (1.0 - erad);
  const double L = 2.0 / (3.0 * sqrt(3.0)) * (1.0 + 2.0 * sqrt(3.0 * r_isco - 2.0));
  const double E = sqrt(1.0 - 2.0 / (3.0 * r_isco));
  const double chif = atot + eta * (L - 2.0 * atot * (E - 1.0)) + (-3.821158961 - 1.2019 * aeff - 1.20764 * aeff * aeff) * eta2
                      + (3.79245 + 1.18385 * aeff + 4.90494 * aeff * aeff) * eta2 * eta;
  const double rf = r_isco_kerr(chif);
  const double om = 1.0 / (rf * sqrt(rf) + chif);
  return om / (kPi * Mfin * kG3);
}

// upper grid frequency of the model (gwfast/waveforms.py:903-951, :1324-1333, :2737-2750)
__host__ __device__ inline double model_fcut(const WfDesc& wf, double Mc, double eta, double chi1 = 0.0,
                                             double chi2 = 0.0) {
  // TaylorF2 (models 0, 3, 5, 6): fcut_par is fHigh in Hz Msun, or the Kerr ISCO; the IMR models: a cut in M f
  const bool tf2 = wf.model == 0 || wf.model == 3 || wf.model == 5 || wf.model == 6;
  if (tf2 && (wf.flags & kTF2KerrIsco)) return tf2_kerr_fcut(Mc, eta, chi1, chi2);
  return tf2 ? wf.fcut_par / (Mc / pow(eta, 0.6)) : wf.fcut_par / (Mc * kG3 / pow(eta, 0.6));
}

__device__ inline bool grid_setup(GridEv& g, const DetDev& d, const EvBatch& ev, const WfDesc& wf, long long n,
                                  double Mc, double eta, double fcut_model = -1.0, double chi1 = 0.0, double chi2 = 0.0) {
  double fcut = fcut_model >= 0.0 ? fcut_model : model_fcut(wf, Mc, eta, chi1, chi2);
  if (d.fmax > 0.0 && fcut > d.fmax) fcut = d.fmax;
  if (ev.fcut_ev) fcut = ev.fcut_ev[n];
  const int R = ev.res_ev ? ev.res_ev[n] : ev.res;
  g.R = R;
  g.fmin = d.fmin;
  g.fcut = fcut;
  g.lnfmin = log(d.fmin);
  if (R < 2 || !(fcut > 0.0)) { g.ok = 0; return false; }
  g.ok = 1;
  if (ev.spacing == 0) {
    g.delta = (log(fcut) - g.lnfmin) / (R - 1);
    g.fac_w = sinh(g.delta);
    g.w0 = 0.5 * expm1(g.delta);
    g.wl = -0.5 * expm1(-g.delta);
  } else {
    g.df = (fcut - d.fmin) / (R - 1);
  }
  return true;
}

// frequency, log-frequency and trapezoid weight of point k (numpy geomspace/linspace + trapz)
__device__ __forceinline__ void grid_point(const GridEv& g, int spacing, int k, double& f, double& lnf, double& w) {
  if (spacing == 0) {
    if (k == g.R - 1) { f = g.fcut; lnf = log(f); w = f * g.wl; }
    else {
      lnf = g.lnfmin + k * g.delta;
      f = (k == 0) ? g.fmin : exp(lnf);
      w = (k == 0) ? f * g.w0 : f * g.fac_w;
    }
  } else {
    f = (k == g.R - 1) ? g.fcut : g.fmin + k * g.df;
    lnf = log(f);
    w = (k == 0 || k == g.R - 1) ? 0.5 * g.df : g.df;
  }
}

template <int MODEL>
__device__ inline void event_setup(EvUnion& E, const DetDev& d, const WfDesc& wf, const double* q, int nq,
                                   double Mc, double eta, double chi1, double chi2, double dL, double lam_t,
                                   double del_lam, double ecc = 0.0, double fgrid_max = 0.0) {
  const D4 mc = D4::seed(Mc, P_MC), et = D4::seed(eta, P_ETA), c1 = D4::seed(chi1, P_CHI1), c2 = D4::seed(chi2, P_CHI2);
  if (MODEL == 7) {
    nsbh_setup(E.nsbh, D6::seed(Mc, P_MC), D6::seed(eta, P_ETA), D6::seed(chi1, P_CHI1), D6::seed(chi2, P_CHI2), dL,
               d.fmin, fgrid_max, q, q + nq, q + 2 * nq, nq, D6::seed(lam_t, P_LT), D6::seed(del_lam, P_DLT), wf.xitide);
    return;
  }
  if (MODEL == 4) {
    nrt_setup(E.nrt, D6::seed(Mc, P_MC), D6::seed(eta, P_ETA), D6::seed(chi1, P_CHI1), D6::seed(chi2, P_CHI2), dL,
              d.fmin, q, q + nq, q + 2 * nq, nq, D6::seed(lam_t, P_LT), D6::seed(del_lam, P_DLT));
    return;
  }
  if (MODEL == 5 || MODEL == 6)
    tf2e_setup(E.tf2e, mc, et, c1, c2, dL, wf.spin_ho != 0, lam_t, del_lam, wf.flags, ecc, d.fmin, wf.fref_ecc);
  else if (MODEL == 3) tf2t_setup(E.tf2t, mc, et, c1, c2, dL, wf.spin_ho != 0, lam_t, del_lam, wf.flags);
  else if (MODEL == 0) tf2_setup(E.tf2, mc, et, c1, c2, dL, wf.spin_ho != 0, wf.flags);
  else if (MODEL == 1) phd_setup(E.phd, mc, et, c1, c2, dL, d.fmin, q, q + nq, q + 2 * nq, nq);
  else hm_setup_core(E.hm, mc, et, c1, c2, dL, d.fmin);
}

// constant pi - pi/4 of the TaylorF2 phase (gwfast/waveforms.py:802, :862), left out of tf2_point
// (with phiref_vlso the pi is absent: the strain outputs subtract it)
constexpr double kTF2PhaseConst = 0.75 * kPi;

// the TaylorF2 record of the TaylorF2 models (0, 3, 5, 6)
template <int MODEL> __device__ __forceinline__ const TF2Ev& tf2_base(const EvUnion& E) {
  return MODEL == 3 ? E.tf2t.b : (MODEL == 5 || MODEL == 6 ? E.tf2e.t.b : E.tf2);
}
template <int MODEL> __device__ __forceinline__ const TF2TEv& tf2_tidal(const EvUnion& E) {
  return MODEL == 5 || MODEL == 6 ? E.tf2e.t : E.tf2t;
}

// TaylorF2 phase and amplitude of models 0, 3, 5, 6 at one point (tidal and eccentric parts added)
template <int MODEL, class S>
__device__ __forceinline__ void tf2_any_point(const EvUnion& E, double f, double f13, double lnf, S& A, S& Phi) {
  const TF2Ev& t = tf2_base<MODEL>(E);
  tf2_point<S>(t, f, f13, lnf, exp(lnf * (-7.0 / 6.0)), A, Phi);
  if constexpr (has_tidal<MODEL>()) Phi = Phi + tf2_tidal_phase<S>(tf2_tidal<MODEL>(E), co<S>(t.vM) * f13);
  if constexpr (has_ecc<MODEL>()) {
    const S v = co<S>(t.vM) * f13;
    const S lnv = co<S>(t.lnvM) + lnf * (1.0 / 3.0);
    Phi = Phi + tf2_ecc_phase<S>(E.tf2e, v, lnv, lnf);
  }
}

// waveform at one point: P, C (hp = P, hc = i C) with tangents, iota derivatives, and tau_star tangent.
// phi0: the waveform phase left out of P and C (22-mode models: Phi(f); HM: 0, the mode phases are in P, C)
// pb (TaylorF2 and IMRPhenomD, Fisher kernels): the event's phase basis; the phase tangent is then
// the basis sum (phase_tangent_d) instead of the dual evaluation of the phase, and phi0 is not formed
template <int MODEL, bool EARTH>
__device__ __forceinline__ void wave_point_dual(const EvUnion& E, const ProjEv& pj, double f, double lnf,
                                                cd& P, cd& C, cd* dP, cd* dC, cd& dPi, cd& dCi, DualOf<MODEL>& tau,
                                                double& phi0, const PhaseBasis* pb = nullptr, const TauD* td = nullptr) {
  constexpr int NI = ndir_of<MODEL>();
  phi0 = 0.0;
  if constexpr (MODEL == 2) {
    Cplx<D4> Pd, Cd;
    Cplx<double> dPv, dCv;
    hm_point<D4>(E.hm, f, Pd, Cd, dPv, dCv);
    P = {Pd.re.v, Pd.im.v}; C = {Cd.re.v, Cd.im.v};
#pragma unroll
    for (int k = 0; k < 4; ++k) { dP[k] = {Pd.re.d[k], Pd.im.d[k]}; dC[k] = {Cd.re.d[k], Cd.im.d[k]}; }
    dPi = {dPv.re, dPv.im}; dCi = {dCv.re, dCv.im};
    if (EARTH) tau = tau_star_point<D4>(E.hm.k.Ms, E.hm.k.vM, E.hm.k.eta, exp(lnf / 3.0));
  } else if constexpr (MODEL == 4 || MODEL == 7) {
    D6 A, Phi;
    const PhdCoreT<D6>& kc = MODEL == 4 ? E.nrt.k : E.nsbh.k;
    if constexpr (MODEL == 4) nrt_point<D6>(E.nrt, f, A, Phi);
    else nsbh_point<D6>(E.nsbh, f, A, Phi);
    if (EARTH) tau = tau_star_point<D6>(kc.Ms, kc.vM, kc.eta, exp(lnf / 3.0));
    phi0 = Phi.v;
    P = {pj.cp * A.v, 0.0};
    C = {pj.ci * A.v, 0.0};
#pragma unroll
    for (int k = 0; k < NI; ++k) {
      const cd dW = {A.d[k], -A.v * Phi.d[k]};
      dP[k] = cscale(dW, pj.cp);
      dC[k] = cscale(dW, pj.ci);
    }
    dPi = {pj.dcp * A.v, 0.0};
    dCi = {pj.dci * A.v, 0.0};
  } else {
    D4 A, Phi;
    double dphi[4];
    bool basis = false;
    if constexpr (MODEL == 0 || MODEL == 1) basis = pb != nullptr;
    if (basis) {
      if constexpr (MODEL == 0) {
        const TF2Ev& t = E.tf2;
        A = t.ampK * exp(lnf * (-7.0 / 6.0));
        if (EARTH) tau = td ? tau_point_d(*td, exp(lnf / 3.0), lnf) : tau_star_point<D4>(t.Ms, t.vM, t.eta, exp(lnf / 3.0));
      } else if constexpr (MODEL == 1) {
        A = td ? phd_amp_d(E.phd.k, *td, f) : phd_amp_point<D4>(E.phd.k, f);
        if (EARTH)
          tau = td ? tau_point_d(*td, exp(lnf / 3.0), lnf)
                   : tau_star_point<D4>(E.phd.k.Ms, E.phd.k.vM, E.phd.k.eta, exp(lnf / 3.0));
      }
      phase_tangent_d(*pb, f, lnf, dphi);
      phi0 = 0.0;
    } else {
      if (is_tf2<MODEL>()) {
        const TF2Ev& t = tf2_base<MODEL>(E);
        const double f13 = exp(lnf / 3.0);
        tf2_any_point<MODEL, D4>(E, f, f13, lnf, A, Phi);
        if (EARTH) tau = tau_star_point<D4>(t.Ms, t.vM, t.eta, f13);
      } else {
        phd_point<D4>(E.phd.k, f, A, Phi);
        if (EARTH) tau = tau_star_point<D4>(E.phd.k.Ms, E.phd.k.vM, E.phd.k.eta, exp(lnf / 3.0));
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) dphi[k] = Phi.d[k];
      phi0 = Phi.v + (is_tf2<MODEL>() ? kTF2PhaseConst : 0.0);
    }
    // W = A e^{-i Phi} with the common phase dropped: value A, tangent dA - i A dPhi
    P = {pj.cp * A.v, 0.0};
    C = {pj.ci * A.v, 0.0};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const cd dW = {A.d[k], -A.v * dphi[k]};
      dP[k] = cscale(dW, pj.cp);
      dC[k] = cscale(dW, pj.ci);
    }
    dPi = {pj.dcp * A.v, 0.0};
    dCi = {pj.dci * A.v, 0.0};
  }
}

// Fisher columns formed analytically per point (their parameters enter the phase only):
// tidal TaylorF2 d Phi / d LambdaTilde, d Phi / d deltaLambda (with use_QuadMonTid also through c4 v^-1
// and c6 v of the series); eccentric TaylorF2 d Phi / d ecc = 2 Phi_ecc / ecc (the eccentric phase is
// proportional to ecc^2). Written as d h = -i h d Phi into D.
template <int MODEL>
__device__ __forceinline__ void analytic_tangents(const EvUnion& E, double lnf, double& dphl, double& dphd, double& dphe) {
  dphl = dphd = dphe = 0.0;
  if constexpr (MODEL == 3 || MODEL == 6) {
    const TF2TEv& t = tf2_tidal<MODEL>(E);
    const double v = t.b.vM.v * exp(lnf / 3.0), v2 = v * v, v5 = v2 * v2 * v;
    const double A = t.b.pn.A.v;
    dphl = A * (v5 * (-19.5 - (3115.0 / 64.0) * v2) + t.q4l / v + t.q6l * v);
    dphd = A * (v5 * v2 * t.s12.v + t.q4d / v + t.q6d * v);
  }
  if constexpr (has_ecc<MODEL>()) {
    const TF2EEv& e = E.tf2e;
    if (e.ecc != 0.0) {
      const double v = e.t.b.vM.v * exp(lnf / 3.0), lnv = e.t.b.lnvM.v + lnf / 3.0;
      dphe = 2.0 * tf2_ecc_phase<double>(e, v, lnv, lnf) / e.ecc;
    }
  }
}
template <int MODEL>
__device__ __forceinline__ void analytic_columns(const cd& H, double dphl, double dphd, double dphe, cd* D) {
  if constexpr (MODEL == 3 || MODEL == 6) {
    D[I_LT] = cscale(cmuli(H), -dphl);
    D[I_DLT] = cscale(cmuli(H), -dphd);
  }
  if constexpr (has_ecc<MODEL>()) D[ecc_col<MODEL>()] = cscale(cmuli(H), -dphe);
}

// value-only waveform with its phase: P, C (hp = P, hc = i C) and phi0 as in wave_point_dual
template <int MODEL, bool EARTH>
__device__ __forceinline__ void wave_point_full(const EvUnion& E, const ProjEv& pj, double f, double lnf,
                                                cd& P, cd& C, double& phi0, double& tau) {
  if (MODEL == 2) {
    Cplx<double> Pd, Cd, dPv, dCv;
    hm_point<double>(E.hm, f, Pd, Cd, dPv, dCv);
    P = {Pd.re, Pd.im};
    C = {Cd.re, Cd.im};
    phi0 = 0.0;
    if (EARTH) tau = tau_star_point<double>(E.hm.k.Ms, E.hm.k.vM, E.hm.k.eta, exp(lnf / 3.0));
  } else {
    double A, Phi;
    if (MODEL == 4 || MODEL == 7) {
      const PhdCoreT<D6>& kc = MODEL == 4 ? E.nrt.k : E.nsbh.k;
      if (MODEL == 4) nrt_point<double>(E.nrt, f, A, Phi);
      else nsbh_point<double>(E.nsbh, f, A, Phi);
      if (EARTH) tau = tau_star_point<double>(kc.Ms, kc.vM, kc.eta, exp(lnf / 3.0));
    } else if (is_tf2<MODEL>()) {
      const TF2Ev& t = tf2_base<MODEL>(E);
      const double f13 = exp(lnf / 3.0);
      tf2_any_point<MODEL, double>(E, f, f13, lnf, A, Phi);
      if (EARTH) tau = tau_star_point<double>(t.Ms, t.vM, t.eta, f13);
    } else {
      phd_point<double>(E.phd.k, f, A, Phi);
      if (EARTH) tau = tau_star_point<double>(E.phd.k.Ms, E.phd.k.vM, E.phd.k.eta, exp(lnf / 3.0));
    }
    P = {pj.cp * A, 0.0};
    C = {pj.ci * A, 0.0};
    phi0 = Phi + (is_tf2<MODEL>() ? kTF2PhaseConst : 0.0);
  }
}

// value-only waveform for the SNR: |hp|, |hc| (HM) or A (22-mode)
template <int MODEL, bool EARTH>
__device__ __forceinline__ void wave_point_val(const EvUnion& E, const ProjEv& pj, double f, double lnf,
                                               double& ap, double& ac, double& tau) {
  if (MODEL == 2) {
    Cplx<double> Pd, Cd, dPv, dCv;
    hm_point<double>(E.hm, f, Pd, Cd, dPv, dCv);
    ap = sqrt(Pd.re * Pd.re + Pd.im * Pd.im);
    ac = sqrt(Cd.re * Cd.re + Cd.im * Cd.im);
    if (EARTH) tau = tau_star_point<double>(E.hm.k.Ms, E.hm.k.vM, E.hm.k.eta, exp(lnf / 3.0));
  } else {
    double A, Phi;
    if (MODEL == 4 || MODEL == 7) {
      const PhdCoreT<D6>& kc = MODEL == 4 ? E.nrt.k : E.nsbh.k;
      if (MODEL == 4) nrt_point<double>(E.nrt, f, A, Phi);
      else nsbh_point<double>(E.nsbh, f, A, Phi);
      if (EARTH) tau = tau_star_point<double>(kc.Ms, kc.vM, kc.eta, exp(lnf / 3.0));
    } else if (is_tf2<MODEL>()) {   // (the phase does not enter |h|: amplitudes only)
      const TF2Ev& t = tf2_base<MODEL>(E);
      A = t.ampK.v * exp(lnf * (-7.0 / 6.0));
      if (EARTH) tau = tau_star_point<double>(t.Ms, t.vM, t.eta, exp(lnf / 3.0));
    } else {
      A = phd_amp_point<double>(E.phd.k, f);
      if (EARTH) tau = tau_star_point<double>(E.phd.k.Ms, E.phd.k.vM, E.phd.k.eta, exp(lnf / 3.0));
    }
    (void)Phi;
    ap = A * pj.cp;
    ac = A * pj.ci;
  }
}

// ------------------------------------------------------------------ per-event set-up records
// The per-event set-up (FP64 duals) runs in its own kernel, one thread per event, and writes a
// record per event into a scratch buffer: [GridEv | ProjEv | model coefficients].  The SNR and
// Fisher kernels copy their event's record into shared memory.
struct SetupHdr {
  GridEv g;
  ProjEv pj;
};

template <int MODEL>
__host__ __device__ constexpr size_t wave_bytes() {
  return MODEL == 0 ? sizeof(TF2Ev)
                    : (MODEL == 1 ? sizeof(PhdEv)
                                  : (MODEL == 2 ? sizeof(HMEv)
                                                : (MODEL == 3 ? sizeof(TF2TEv)
                                                              : (MODEL == 4 ? sizeof(NRTEv) : (MODEL == 7 ? sizeof(NSBHEv) : sizeof(TF2EEv))))));
}
// the 22-mode models also carry the phase-tangent basis used by the FP32 kernel
template <int MODEL>
__host__ __device__ constexpr size_t basis_bytes() {
  return MODEL < 2 ? sizeof(PhaseBasis) : 0;
}
template <int MODEL>
__host__ __device__ constexpr size_t rec_stride() {
  return ((sizeof(SetupHdr) + wave_bytes<MODEL>() + basis_bytes<MODEL>() + 15) / 16) * 16;
}
template <int MODEL>
__device__ __forceinline__ const PhaseBasis* rec_basis(const unsigned char* scratch, long long i) {
  return reinterpret_cast<const PhaseBasis*>(scratch + i * rec_stride<MODEL>() + sizeof(SetupHdr) + wave_bytes<MODEL>());
}

// copy N 8-byte words, 32 at a time: every load of a batch is issued before any of its stores. The
// source and destination are different records, but the compiler cannot tell, so a plain loop
// waits for each load in turn (one L2 round trip per word).
template <int N>
__device__ __forceinline__ void copy_words(unsigned long long* dst, const unsigned long long* src) {
  constexpr int B = 32;
#pragma unroll 1
  for (int w0 = 0; w0 < N; w0 += B) {
    unsigned long long v[B];
#pragma unroll
    for (int k = 0; k < B; ++k)
      if (w0 + k < N) v[k] = src[w0 + k];
#pragma unroll
    for (int k = 0; k < B; ++k)
      if (w0 + k < N) dst[w0 + k] = v[k];
  }
}

// core: optional per-call cache of the source-dependent model record, indexed by event (or by
// core_idx[event] for a gathered batch); core_mode 1 computes the record and stores it there, 2 loads
// it and recomputes only the detector-dependent part (the per-event set-up is FP64-bound, and a
// network evaluates it once per detector)
template <int MODEL>
__global__ void __launch_bounds__(kEvBlock) setup_kernel(EvBatch ev, DetDev det_in, WfDesc wf, const double* qnm, int nq,
                                                          unsigned char* scratch, long long count, unsigned char* core,
                                                          int core_mode, const long long* core_idx, int epw) {
  const long long i = ev_thread(epw);
  const long long n = ev.n0 + i;
  if (i < 0 || i >= count || n >= ev.N) return;
  DetDev det = det_in;
  if (ev.fmin_ev) det.fmin = ev.fmin_ev[n];
  unsigned char* rec = scratch + i * rec_stride<MODEL>();
  SetupHdr& h = *reinterpret_cast<SetupHdr*>(rec);
  EvUnion& E = *reinterpret_cast<EvUnion*>(rec + sizeof(SetupHdr));
  const double* p = ev.p;
  const long long ld = ev.ld;
  const double Mc = p[0 * ld + n], eta = p[1 * ld + n], dL = p[2 * ld + n];
  const double th = p[3 * ld + n], ph = p[4 * ld + n], io = p[5 * ld + n], ps = p[6 * ld + n];
  const double tc = p[7 * ld + n], c1 = p[9 * ld + n], c2 = p[10 * ld + n];
  const double lt = has_tidal<MODEL>() ? p[11 * ld + n] : 0.0, dlt = has_tidal<MODEL>() ? p[12 * ld + n] : 0.0;
  const double ecc = has_ecc<MODEL>() ? p[ecc_col<MODEL>() * ld + n] : 0.0;
  // IMRPhenomD_NRTidalv2 ends at 1.2 times its merger frequency, which depends on the deformabilities
  if (grid_setup(h.g, det, ev, wf, n, Mc, eta, MODEL == 4 ? nrt_fcut(Mc, eta, lt, dlt) : -1.0, c1, c2)) {
    constexpr int nw = (int)(wave_bytes<MODEL>() / 8);
    const long long crow = core_idx ? core_idx[n] : n;   // a gathered batch reads the rows of its events
    unsigned long long* cw = core ? reinterpret_cast<unsigned long long*>(core + (size_t)crow * wave_bytes<MODEL>()) : nullptr;
    unsigned long long* ew = reinterpret_cast<unsigned long long*>(&E);
    if (core_mode == 2 && cw) {
      copy_words<nw>(ew, cw);
      if (MODEL == 1) phd_ref(E.phd, det.fmin);
      if (MODEL == 2) hm_ref(E.hm, det.fmin);
      if (MODEL == 4) nrt_ref(E.nrt, det.fmin);
      if (MODEL == 5 || MODEL == 6) tf2e_ref(E.tf2e, det.fmin, wf.fref_ecc);
      if (MODEL == 7) nsbh_ref(E.nsbh, det.fmin, h.g.fcut);
    } else {
      event_setup<MODEL>(E, det, wf, qnm, nq, Mc, eta, c1, c2, dL, lt, dlt, ecc, h.g.fcut);
      if (MODEL == 2) {
        const D4 et = D4::seed(eta, P_ETA), k1 = D4::seed(c1, P_CHI1), k2 = D4::seed(c2, P_CHI2);
        const D4 af = final_spin(et, k1, k2);
        const D4 finmass = 1.0 - radiated_energy(et, k1, k2);
        for (int mode = 0; mode < 6; ++mode) hm_setup_mode(E.hm, mode, et, k1, k2, io, af, finmass);
      }
      if (core_mode == 1 && cw)
        copy_words<nw>(cw, ew);
    }
    PhaseBasis* pb = reinterpret_cast<PhaseBasis*>(rec + sizeof(SetupHdr) + wave_bytes<MODEL>());
    if (MODEL == 0) tf2_phase_basis(E.tf2, *pb);
    if (MODEL == 1) phd_phase_basis(E.phd.k, *pb);
  }
  proj_setup(h.pj, det, th, ph, io, ps, tc, dL);
}

// cooperative copy of one event record into shared memory (all pieces are multiples of 8 bytes)
// (pb: also the phase basis that follows the model record, for TaylorF2 and IMRPhenomD)
template <int MODEL>
__device__ inline void block_load(EvUnion& E, ProjEv& pj, GridEv& g, const unsigned char* scratch, long long i,
                                  PhaseBasis* pb = nullptr) {
  const unsigned char* rec = scratch + i * rec_stride<MODEL>();
  const unsigned long long* src = reinterpret_cast<const unsigned long long*>(rec);
  unsigned long long* dg = reinterpret_cast<unsigned long long*>(&g);
  unsigned long long* dp = reinterpret_cast<unsigned long long*>(&pj);
  unsigned long long* de = reinterpret_cast<unsigned long long*>(&E);
  unsigned long long* db = reinterpret_cast<unsigned long long*>(pb);
  constexpr int ng = sizeof(GridEv) / 8, np = sizeof(ProjEv) / 8, ne = wave_bytes<MODEL>() / 8;
  constexpr int nb = basis_bytes<MODEL>() / 8;
  static_assert(sizeof(SetupHdr) == sizeof(GridEv) + sizeof(ProjEv), "packed header");
  static_assert(basis_bytes<MODEL>() % 8 == 0, "basis in 8-byte words");
  const int nw = ng + np + ne + (pb ? nb : 0);
  for (int w = threadIdx.x; w < nw; w += blockDim.x) {
    const unsigned long long v = src[w];
    if (w < ng) dg[w] = v;
    else if (w < ng + np) dp[w - ng] = v;
    else if (w < ng + np + ne) de[w - ng - np] = v;
    else db[w - ng - np - ne] = v;
  }
  __syncthreads();
}

// ------------------------------------------------------------------ Fisher kernels
// Work unit: an item = (event, frequency segment [k0, k1)). The classic kernels run one item per
// event (k0 = 0, k1 = R) and write the event's matrices; the segmented kernels are persistent,
// take items from an atomic counter (work stealing), and write one partial Gram per item, which
// gram_reduce_kernel sums per event in segment order (deterministic).
//
// Gram layout in shared memory and in the partials: [set][upper-triangle entry], entry index
// pidx(a, b) for a <= b (kPairA / kPairB order).
__host__ __device__ constexpr int pidx(int a, int b) { return a * NP - a * (a - 1) / 2 + (b - a); }
// per Gram set: the NE upper-triangle entries, then the NP products Re<dh/dtheta_a | h> with the
// strain itself (for the SNR derivatives; zero unless asked for)
constexpr int NEX = NE + NP;

// Column changes of the FP32 form, undone here in FP64. The FP32 kernel accumulates the Gram G of
// modified columns D' and the original columns are D_a = D'_a + k_a D'_{c(a)}:
//   psi:    D_psi  = Delta + 2 s D_Phicoal   (psi_sgn = s = +-1; 0: no change)
//   chi1z:  D_chi1 = D'_chi1 + alpha D_chi2  (chi_alpha = alpha; 0: no change)
// so F_ab = G_ab + k_a G_{c(a) b} + k_b G_{a c(b)} + k_a k_b G_{c(a) c(b)}.
struct ColMix {
  double psi2, alpha;
  __device__ __forceinline__ int partner(int a, double& k) const {
    if (a == I_PS && psi2 != 0.0) { k = psi2; return I_PC; }
    if (a == I_C1 && alpha != 0.0) { k = alpha; return I_C2; }
    k = 0.0;
    return -1;
  }
};

// write the event's matrices from gsum[NG][nex_of(NPR)] (upper triangles, then the strain
// products): column changes undone, scaled; outputs are NPR x NPR per event
template <int NG, int NPR = NP>
__device__ void write_gram(const double* gsum, double scale, ColMix mix, long long n, long long N, double* out_arm,
                           double* out_det, double* out_sd_arm, double* out_sd_det, int accum) {
  constexpr int NEP = ne_of(NPR), NEXP = nex_of(NPR);
  for (int e = threadIdx.x; e < NEP; e += blockDim.x) {
    int a, b;
    pair_n(NPR, e, a, b);
    double ka, kb;
    const int ca = mix.partner(a, ka), cb = mix.partner(b, kb);
    double sdet = 0.0;
#pragma unroll
    for (int gs = 0; gs < NG; ++gs) {
      const double* G = gsum + gs * NEXP;
      auto at = [&](int x, int y) { return x <= y ? G[pidx_n(NPR, x, y)] : G[pidx_n(NPR, y, x)]; };
      double v = G[e];
      if (ca >= 0) v += ka * at(ca, b);
      if (cb >= 0) v += kb * at(a, cb);
      if (ca >= 0 && cb >= 0) v += ka * kb * at(ca, cb);
      v *= scale;
      sdet += v;
      if (out_arm && (NG == 1 || NG == 3)) {
        double* o = out_arm + ((size_t)gs * N + n) * (NPR * NPR);
        o[a * NPR + b] = v;
        o[b * NPR + a] = v;
      }
    }
    if (out_det) {
      double* o = out_det + (size_t)n * (NPR * NPR);
      if (accum) { o[a * NPR + b] += sdet; if (a != b) o[b * NPR + a] += sdet; }
      else { o[a * NPR + b] = sdet; o[b * NPR + a] = sdet; }
    }
  }
  if (out_sd_arm || out_sd_det) {   // Re<dh/dtheta_a | h>, the same column changes undone
    for (int a = threadIdx.x; a < NPR; a += blockDim.x) {
      double k;
      const int c = mix.partner(a, k);
      double sdet = 0.0;
#pragma unroll
      for (int gs = 0; gs < NG; ++gs) {
        const double* H = gsum + gs * NEXP + NEP;
        double v = H[a];
        if (c >= 0) v += k * H[c];
        v *= scale;
        sdet += v;
        if (out_sd_arm && (NG == 1 || NG == 3)) out_sd_arm[((size_t)gs * N + n) * NPR + a] = v;
      }
      if (out_sd_det) {
        double* o = out_sd_det + (size_t)n * NPR + a;
        *o = accum ? *o + sdet : sdet;
      }
    }
  }
}

// per-event state of the FP64 kernels (shared memory)
template <int NARM, int NG, int NPR = NP>
struct F64State {
  EvUnion E;
  PhaseBasis pb;   // TaylorF2 and IMRPhenomD: the phase tangent's basis
  TauD td;         // and the coefficients of tau_star (Earth rotation)
  ProjEv pj;
  GridEv g;
  ArmPat apc[NARM];
  TimeState tsc;
  double gsum[NG * nex_of(NPR)];
  long long rec;
};

template <int MODEL, bool EARTH, int NARM, int NG>
__device__ inline void f64_prepare(const DetDev& det, const unsigned char* scratch, long long rec,
                                   F64State<NARM, NG, np_of<MODEL>()>& S) {
  block_load<MODEL>(S.E, S.pj, S.g, scratch, rec, (MODEL == 0 || MODEL == 1) ? &S.pb : nullptr);
  if (!EARTH) {
    if (threadIdx.x == 0) {
      time_state(S.pj, S.pj.tc, S.tsc);
      for (int a = 0; a < NARM; ++a) arm_pattern(S.pj, det.sin_zeta, S.tsc.x, a, S.apc[a]);
    }
  }
  if constexpr (MODEL == 0 || MODEL == 1) {
    if (threadIdx.x == 32 && S.g.ok) {
      if constexpr (MODEL == 0) tau_setup_d(S.td, S.E.tf2.Ms, S.E.tf2.vM, S.E.tf2.eta);
      else {
        tau_setup_d(S.td, S.E.phd.k.Ms, S.E.phd.k.vM, S.E.phd.k.eta);
        amp_setup_d(S.td, S.E.phd.k.ampPref, S.E.phd.k.MG);
      }
    }
  }
  if (threadIdx.x == 0) S.rec = rec;
  __syncthreads();
}

// staging row stride (complex values): lanes of a quarter-warp read different rows at the same
// point; with an odd stride those rows fall in different banks (32 gives 8-way conflicts)
constexpr int kSR64 = 33;

// Gram of points [k0, k1) into S.gsum (summed over warps); stage: [warp][NG][NPM + 1][kSR64] complex,
// column NPM holding the strain itself when sd (SNR derivatives) is set (NPM = np_of<MODEL>())
template <int MODEL, bool EARTH, int NARM, int NG>
__device__ inline void f64_item(const EvBatch& ev, const DetDev& det, F64State<NARM, NG, np_of<MODEL>()>& S, cd* stage,
                                int k0, int k1, bool sd) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int NPM = np_of<MODEL>();
  constexpr int NEM = ne_of(NPM), NEXM = nex_of(NPM);
  constexpr int NPS = NPM + 1;
  constexpr int NENT = NEXM * NG;
  constexpr int EPT = (NENT + 31) / 32;
  double acc[EPT];
  int ea[EPT], eb[EPT], eg[EPT];   // this lane's entries: rows, set (-1: none)
#pragma unroll
  for (int i = 0; i < EPT; ++i) {
    acc[i] = 0.0;
    const int e = lane + 32 * i;
    eg[i] = -1;
    ea[i] = eb[i] = 0;
    if (e < NENT) {
      const int gs = e / NEXM, pe = e - gs * NEXM;
      if (pe < NEM) { pair_n(NPM, pe, ea[i], eb[i]); eg[i] = gs; }
      else if (sd) { ea[i] = pe - NEM; eb[i] = NPM; eg[i] = gs; }   // (a, NPM): strain products
    }
  }
  cd* my = stage + (size_t)warp * NG * NPS * kSR64;
  for (int base = k0; base < k1; base += kThreads) {
    const int k = base + tid;
    cd D[NARM][NPS];
    double sw = 0.0;
    if (k < k1) {
      double f, lnf, w;
      grid_point(S.g, ev.spacing, k, f, lnf, w);
      const double Sn = psd_at(det, f, lnf);
      sw = sqrt(4.0 * w / Sn);
      constexpr int NI = ndir_of<MODEL>();
      cd P, C, dP[NI], dC[NI], dPi, dCi;
      DualOf<MODEL> tau(0.0);
      double phi0;
      wave_point_dual<MODEL, EARTH>(S.E, S.pj, f, lnf, P, C, dP, dC, dPi, dCi, tau, phi0,
                                    (MODEL == 0 || MODEL == 1) ? &S.pb : nullptr,
                                    (MODEL == 0 || MODEL == 1) ? &S.td : nullptr);
      double dtn[NI];
#pragma unroll
      for (int q = 0; q < NI; ++q) dtn[q] = 0.0;
      TimeState ts;
      if (EARTH) {
        const double tn = S.pj.tc - tau.v / kDay;
#pragma unroll
        for (int q = 0; q < NI; ++q) dtn[q] = -tau.d[q] / kDay;
        time_state(S.pj, tn, ts);
      } else {
        ts = S.tsc;
      }
      double dphl, dphd, dphe;
      analytic_tangents<MODEL>(S.E, lnf, dphl, dphd, dphe);
#pragma unroll
      for (int a = 0; a < NARM; ++a) {
        ArmPat ap;
        if (EARTH) arm_pattern(S.pj, det.sin_zeta, ts.x, a, ap);
        else ap = S.apc[a];
        arm_derivs<NI>(S.pj, ap, ts, f, P, C, dP, dC, dPi, dCi, dtn, D[a]);
        const cd H = cadd(cscale(P, ap.Fp), cscale(cmuli(C), ap.Fc));
        analytic_columns<MODEL>(H, dphl, dphd, dphe, D[a]);
        D[a][NPM] = sd ? H : cd{0.0, 0.0};
      }
    } else {
#pragma unroll
      for (int a = 0; a < NARM; ++a)
#pragma unroll
        for (int q = 0; q < NPS; ++q) D[a][q] = {0.0, 0.0};
    }
    // stage weighted derivative vectors of this warp's 32 points
#pragma unroll
    for (int q = 0; q < NPS; ++q) {
      if (NG == 1) {
        my[(0 * NPS + q) * kSR64 + lane] = cscale(D[0][q], sw);
      } else if (NG == 2) {
        const cd u = D[0][q], v = D[1][q];
        my[(0 * NPS + q) * kSR64 + lane] = cscale(cadd(u, v), sw * 1.2247448713915890);   // sqrt(3/2)
        my[(1 * NPS + q) * kSR64 + lane] = cscale(cadd(u, cscale(v, -1.0)), sw * 0.70710678118654752);
      } else {
        const cd u = D[0][q], v = D[1][q];
        my[(0 * NPS + q) * kSR64 + lane] = cscale(u, sw);
        my[(1 * NPS + q) * kSR64 + lane] = cscale(v, sw);
        my[(2 * NPS + q) * kSR64 + lane] = cscale(cadd(u, v), -sw);
      }
    }
    __syncwarp();
#pragma unroll
    for (int i = 0; i < EPT; ++i) {
      if (eg[i] >= 0) {
        const cd* ra = my + (eg[i] * NPS + ea[i]) * kSR64;
        const cd* rb = my + (eg[i] * NPS + eb[i]) * kSR64;
        double s2 = 0.0;
#pragma unroll 8
        for (int j = 0; j < 32; ++j) s2 += ra[j].re * rb[j].re + ra[j].im * rb[j].im;
        acc[i] += s2;
      }
    }
    __syncwarp();
  }
  // cross-warp reduction through the staging area
  __syncthreads();
  double* red = reinterpret_cast<double*>(stage);  // [kWarps][NENT]
#pragma unroll
  for (int i = 0; i < EPT; ++i) {
    const int e = lane + 32 * i;
    if (e < NENT) red[warp * NENT + e] = acc[i];
  }
  __syncthreads();
  for (int e = tid; e < NENT; e += kThreads) {
    double s2 = 0.0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) s2 += red[w * NENT + e];
    S.gsum[e] = s2;
  }
  __syncthreads();
}

// NG: Gram sets per point. L: 1. Triangle, per arm: 3 (arm1, arm2, -(arm1+arm2)).
// Triangle, detector total: 2, using G(U)+G(V)+G(U+V) = G(sqrt(3/2)(U+V)) + G(sqrt(1/2)(U-V)).
template <int MODEL, bool EARTH, int NARM, int NG>
__global__ void __launch_bounds__(kThreads) fisher_kernel(EvBatch ev, DetDev det, const unsigned char* scratch,
                                                          double* out_arm, double* out_det, double* out_sd_arm,
                                                          double* out_sd_det, int accum) {
  extern __shared__ __align__(16) unsigned char stage_raw[];
  __shared__ F64State<NARM, NG, np_of<MODEL>()> S;
  const long long n = ev.n0 + blockIdx.x;
  if (n >= ev.N) return;
  f64_prepare<MODEL, EARTH, NARM, NG>(det, scratch, blockIdx.x, S);
  f64_item<MODEL, EARTH, NARM, NG>(ev, det, S, reinterpret_cast<cd*>(stage_raw), 0, S.g.ok ? S.g.R : 0,
                                   out_sd_arm || out_sd_det);
  write_gram<NG, np_of<MODEL>()>(S.gsum, 1.0, ColMix{0.0, 0.0}, n, ev.N, out_arm, out_det, out_sd_arm, out_sd_det,
                                 accum);
}

// ------------------------------------------------------------------ segmented (persistent) launches
// Segment bookkeeping of one chunk: off[i] = first item of record i, off[count] = total items.
struct SegInfo {
  const long long* off;
  unsigned long long* counter;   // next item to take
  double* partial;               // [item][NG * NEX]
  long long cap;                 // items the partial buffer holds
  int seg;                       // points per segment (multiple of kThreads)
  int* overflow;                 // set when the items exceed cap (never expected: cap is an upper bound)
};

// items per record: ceil(R / seg); exclusive scan over the chunk in one block of 1024 threads
template <int MODEL>
__global__ void __launch_bounds__(1024) seg_scan_kernel(const unsigned char* scratch, long long count, int seg,
                                                        long long* off) {
  __shared__ long long part[1024];
  const int t = threadIdx.x;
  const long long per = (count + 1023) / 1024;
  const long long lo = t * per, hi = lo + per < count ? lo + per : count;
  long long s = 0;
  for (long long i = lo; i < hi; ++i) {
    const GridEv& g = reinterpret_cast<const SetupHdr*>(scratch + i * rec_stride<MODEL>())->g;
    const long long R = g.ok ? g.R : 0;
    s += (R + seg - 1) / seg;
  }
  part[t] = s;
  __syncthreads();
  for (int d = 1; d < 1024; d <<= 1) {   // inclusive scan (Hillis-Steele)
    const long long v = t >= d ? part[t - d] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  long long run = t ? part[t - 1] : 0;
  for (long long i = lo; i < hi; ++i) {
    off[i] = run;
    const GridEv& g = reinterpret_cast<const SetupHdr*>(scratch + i * rec_stride<MODEL>())->g;
    const long long R = g.ok ? g.R : 0;
    run += (R + seg - 1) / seg;
  }
  if (t == 1023) off[count] = part[1023];
}

// take the next item; returns false when none is left. Thread 0 takes it and finds its record by
// binary search in off[]; everything is broadcast through shared memory.
__device__ inline bool next_item(const SegInfo& si, long long count, long long& item, long long& rec, int& k0) {
  __shared__ long long sh_item, sh_rec;
  if (threadIdx.x == 0) {
    const long long total = si.off[count];
    long long it = (long long)atomicAdd(si.counter, 1ull);
    if (it >= total) it = -1;
    else if (it >= si.cap) { atomicExch(si.overflow, 1); it = -1; }
    long long r = -1;
    if (it >= 0) {
      long long a = 0, b = count;   // largest r with off[r] <= it
      while (b - a > 1) {
        const long long m = (a + b) >> 1;
        if (si.off[m] <= it) a = m; else b = m;
      }
      r = a;
    }
    sh_item = it;
    sh_rec = r;
  }
  __syncthreads();
  item = sh_item;
  rec = sh_rec;
  __syncthreads();
  if (item < 0) return false;
  k0 = (int)((item - si.off[rec]) * si.seg);
  return true;
}

template <int MODEL, bool EARTH, int NARM, int NG>
__global__ void __launch_bounds__(kThreads) fisher_seg_kernel(EvBatch ev, DetDev det, const unsigned char* scratch,
                                                              long long count, SegInfo si, int sd) {
  static_assert(np_of<MODEL>() == NP, "segmented launches carry 11-parameter partial Grams");
  extern __shared__ __align__(16) unsigned char stage_raw[];
  __shared__ F64State<NARM, NG, np_of<MODEL>()> S;
  if (threadIdx.x == 0) S.rec = -1;
  __syncthreads();
  long long item, rec;
  int k0;
  while (next_item(si, count, item, rec, k0)) {
    if (S.rec != rec) f64_prepare<MODEL, EARTH, NARM, NG>(det, scratch, rec, S);
    const int R = S.g.ok ? S.g.R : 0;
    const int k1 = k0 + si.seg < R ? k0 + si.seg : R;
    f64_item<MODEL, EARTH, NARM, NG>(ev, det, S, reinterpret_cast<cd*>(stage_raw), k0, k1, sd != 0);
    double* o = si.partial + item * (NG * NEX);
    for (int e = threadIdx.x; e < NG * NEX; e += blockDim.x) o[e] = S.gsum[e];
  }
}

// per event: sum of its items' partial Grams in segment order, then the event's matrices.
// rec (FP32 form) points at the first record's [scale, psi_sgn, chi_alpha] (stride rec_stride_d
// doubles); null: scale 1, no column changes.
template <int NG>
__global__ void __launch_bounds__(kThreads) gram_reduce_kernel(long long n0, long long N, long long count, SegInfo si,
                                                               const double* rec, long long rec_stride_d,
                                                               double* out_arm, double* out_det, double* out_sd_arm,
                                                               double* out_sd_det, int accum) {
  __shared__ double gsum[NG * NEX];
  const long long i = blockIdx.x;
  if (i >= count) return;
  const long long a = si.off[i];
  long long b = si.off[i + 1];
  if (b > si.cap) b = si.cap;   // items beyond the buffer were never written (overflow is flagged)
  for (int e = threadIdx.x; e < NG * NEX; e += blockDim.x) {
    double s = 0.0;
    for (long long it = a; it < b; ++it) s += si.partial[it * (NG * NEX) + e];
    gsum[e] = s;
  }
  __syncthreads();
  const double* r = rec ? rec + i * rec_stride_d : nullptr;
  const double scale = r ? r[0] : 1.0;
  const ColMix mix{r ? 2.0 * r[1] : 0.0, r ? r[2] : 0.0};
  write_gram<NG>(gsum, scale, mix, n0 + i, N, out_arm, out_det, out_sd_arm, out_sd_det, accum);
}

// ------------------------------------------------------------------ SNR kernel
// out_arm[a][n] = trapz((Ap^2 + Ac^2)/S) per arm (SNR_arm = 2 sqrt), out_det[n] += 4 sum_arms.
template <int MODEL, bool EARTH, int NARM>
__global__ void __launch_bounds__(kThreads) snr_kernel(EvBatch ev, DetDev det, const unsigned char* scratch,
                                                       double* out_arm, double* out_det, int accum) {
  __shared__ EvUnion E;
  __shared__ ProjEv pj;
  __shared__ GridEv g;
  __shared__ ArmPat apc[NARM];
  __shared__ double red[kWarps][3];
  const long long n = ev.n0 + blockIdx.x;
  if (n >= ev.N) return;
  block_load<MODEL>(E, pj, g, scratch, blockIdx.x);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (!EARTH) {
    if (tid == 0) {
      TimeState ts;
      time_state(pj, pj.tc, ts);
      for (int a = 0; a < NARM; ++a) arm_pattern(pj, det.sin_zeta, ts.x, a, apc[a]);
    }
    __syncthreads();
  }
  double s[3] = {0.0, 0.0, 0.0};
  const int R = g.ok ? g.R : 0;
  for (int k = tid; k < R; k += kThreads) {
    double f, lnf, w;
    grid_point(g, ev.spacing, k, f, lnf, w);
    const double S = psd_at(det, f, lnf);
    double ap, ac, tau = 0.0;
    wave_point_val<MODEL, EARTH>(E, pj, f, lnf, ap, ac, tau);
    double Fp[2], Fc[2];
    if (EARTH) {
      TimeState ts;
      time_state(pj, pj.tc - tau / kDay, ts);
#pragma unroll
      for (int a = 0; a < NARM; ++a) { ArmPat p; arm_pattern(pj, det.sin_zeta, ts.x, a, p); Fp[a] = p.Fp; Fc[a] = p.Fc; }
    } else {
#pragma unroll
      for (int a = 0; a < NARM; ++a) { Fp[a] = apc[a].Fp; Fc[a] = apc[a].Fc; }
    }
    const double ws = w / S;
    const double p1 = ap * Fp[0], c1 = ac * Fc[0];
    s[0] += ws * (p1 * p1 + c1 * c1);
    if (NARM == 2) {
      const double p2 = ap * Fp[1], c2 = ac * Fc[1];
      s[1] += ws * (p2 * p2 + c2 * c2);
      const double p3 = p1 + p2, c3 = c1 + c2;
      s[2] += ws * (p3 * p3 + c3 * c3);
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    double v = s[a];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp][a] = v;
  }
  __syncthreads();
  if (tid == 0) {
    const int na = (NARM == 2) ? 3 : 1;
    double tot = 0.0;
    for (int a = 0; a < na; ++a) {
      double v = 0.0;
      for (int w = 0; w < kWarps; ++w) v += red[w][a];
      if (out_arm) out_arm[(size_t)a * ev.N + n] = v;
      tot += 4.0 * v;
    }
    if (out_det) out_det[n] = accum ? out_det[n] + tot : tot;
  }
}

}  // namespace gwf
