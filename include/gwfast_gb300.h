/*
 * gwfast_gb300 C ABI: SNR and Fisher matrices of gravitational-wave events on one GPU.
 *
 * This is the drop-in boundary for the Fisher-forecast hot path of gwfast 1.1.2.
 * gwfast itself is pure Python; the functions below are what its Python
 * classes would bind through ctypes to move the hot path onto a GB300.  Every
 * entry point names the reference interface it replaces.
 *
 * Conventions
 *  - All functions return 0 (GWF_OK) or a negative GWF_ERR_* code; the message of
 *    the last failure on the calling thread is returned by gwf_last_error().
 *  - Event parameters are a structure of arrays: params[k * ld + n] holds
 *    parameter k of event n, k in the Fisher order
 *      0 Mc [Msun, detector frame], 1 eta, 2 dL [Gpc], 3 theta, 4 phi, 5 iota,
 *      6 psi [rad], 7 tcoal [GMST days], 8 Phicoal [rad], 9 chi1z, 10 chi2z
 *    (gwfast/waveforms.py:78, :125-129); the tidal models (GWF_WF_TAYLORF2_TIDAL, GWF_WF_PHENOMD_NRTIDALV2,
 *    GWF_WF_TAYLORF2_TIDAL_ECC) add 11 LambdaTilde, 12 deltaLambda (gwfast/waveforms.py:106-109), and the
 *    eccentric TaylorF2 adds ecc after them (GWF_WF_TAYLORF2_ECC: row 11, 12 rows; GWF_WF_TAYLORF2_TIDAL_ECC:
 *    row 13, 14 rows; gwfast/waveforms.py:110-123).
 *  - mem = GWF_MEM_HOST: params, res_per_event and outputs are host pointers; the
 *    call copies in, runs, copies out and returns when the outputs are written.
 *    mem = GWF_MEM_DEVICE: all pointers are device pointers owned by the caller;
 *    the work is queued on `stream` (NULL = the context's stream) and the call
 *    returns without waiting.
 *  - Fisher matrices are written row-major, P x P per event (P = the number of parameter rows),
 *    tcoal in seconds (gwfast/signal.py:918-920).
 *  - One context per thread; calls on one context are serialised on its stream.
 */
#ifndef GWFAST_GB300_H
#define GWFAST_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GWF_NPARAMS 11
#define GWF_NPARAMS_TIDAL 13
#define GWF_NPARAMS_ECC 12
#define GWF_NPARAMS_TIDAL_ECC 14

enum {
  GWF_OK = 0,
  GWF_ERR_INVALID_ARG = -1,
  GWF_ERR_CUDA = -2,
  GWF_ERR_OOM = -3,
  GWF_ERR_TIMEOUT = -4,
  GWF_ERR_UNSUPPORTED = -5
};

/* GWF_WF_TAYLORF2_TIDAL: TaylorF2_RestrictedPN(is_tidal=True), gwfast/waveforms.py:849-855;
 * GWF_WF_PHENOMD_NRTIDALV2: IMRPhenomD_NRTidalv2, gwfast/waveforms.py:1339-1836 (its cut frequency
 * follows from the deformabilities; fcut_par is the M f cut 0.2 of the IMRPhenomD part). Both FP64,
 * 13 parameters.
 * GWF_WF_TAYLORF2_ECC, GWF_WF_TAYLORF2_TIDAL_ECC: TaylorF2_RestrictedPN(is_eccentric=True), without or with
 * is_tidal (gwfast/waveforms.py:814-845): FP64, 12 and 14 parameters. */
enum { GWF_WF_TAYLORF2 = 0, GWF_WF_PHENOMD = 1, GWF_WF_PHENOMHM = 2, GWF_WF_TAYLORF2_TIDAL = 3,
       GWF_WF_PHENOMD_NRTIDALV2 = 4, GWF_WF_TAYLORF2_ECC = 5, GWF_WF_TAYLORF2_TIDAL_ECC = 6, GWF_WF_PHENOMNSBH = 7 };
/* GWF_WF_PHENOMNSBH: IMRPhenomNSBH, gwfast/waveforms.py:2752-3374 (object 1 the black hole, object 2 the
 * neutron star; LambdaTilde, deltaLambda rows as for the tidal models, 13 parameters, FP64; needs the QNM
 * table). Its xi_tide table (gwfast ships it as WFfiles/xiTide_Table_200.h5 or tabulates it,
 * :3286-3373) is built on the device on first use: 200^3 nodes, 64 MiB per context. */
/* gwf_wf_desc.flags, TaylorF2 models only (gwfast/waveforms.py:726-741):
 * GWF_TF2_PHIREF_VLSO    phiref_vlso=True (2.5PN constant referenced at the last stable orbit, :796-798)
 * GWF_TF2_KERR_ISCO      which_ISCO='Kerr' (cut at twice the Kerr-remnant ISCO frequency, :921-951)
 * GWF_TF2_QUADMON_TIDAL  use_QuadMonTid=True (tidal models: spin-induced quadrupole moments, :780-788) */
enum { GWF_TF2_PHIREF_VLSO = 1, GWF_TF2_KERR_ISCO = 2, GWF_TF2_QUADMON_TIDAL = 4 };
enum { GWF_SHAPE_L = 0, GWF_SHAPE_T = 1 };
enum { GWF_SPACING_GEOM = 0, GWF_SPACING_LIN = 1 };
enum { GWF_MEM_HOST = 0, GWF_MEM_DEVICE = 1 };
enum { GWF_PREC_FP64 = 0, GWF_PREC_FP32 = 1, GWF_PREC_MIXED = 2 };

typedef struct gwf_ctx gwf_ctx;
typedef struct gwf_mlp gwf_mlp;

/* Detector geometry and band (gwfast/signal.py:68-160, GWSignal.__init__). */
typedef struct {
  double lat_rad;      /* latitude */
  double long_rad;     /* longitude */
  double xax_rad;      /* bisector of the (first) arms w.r.t. local East */
  int shape;           /* GWF_SHAPE_L or GWF_SHAPE_T */
  int earth_rotation;  /* useEarthMotion */
  double fmin;         /* Hz */
  double fmax;         /* Hz, <= 0 for none */
} gwf_det_desc;

/* Waveform model (gwfast/waveforms.py:49-199 WaveFormModel; :697 TaylorF2_RestrictedPN (is_tidal:
 * model 3), :959 IMRPhenomD, :1838 IMRPhenomHM). */
typedef struct {
  int model;           /* GWF_WF_* */
  int spin_ho;         /* TaylorF2 use_3p5PN_SpinHO */
  double fcut_par;     /* TaylorF2: fHigh [Hz] (default 2 f_ISCO); IMR models: Mf cut (0.2) */
  int flags;           /* GWF_TF2_* (0 for the defaults) */
  int reserved;        /* 0 */
  double fref_ecc;     /* eccentric TaylorF2: fRef_ecc [Hz]; <= 0: the lowest grid frequency (gwfast's None) */
} gwf_wf_desc;

/* Context: device selection, PSD tables, staging memory.
 * Replaces the per-process JAX/XLA set-up of gwfast/signal.py:162-214 (_init_jax). */
int gwf_ctx_create(int device, gwf_ctx** out);
int gwf_ctx_destroy(gwf_ctx* ctx);
const char* gwf_last_error(void);
int gwf_version(void);

/* IMRPhenomNSBH's xi_tide (arXiv:1509.00512 eq. 8) interpolated on its table at n points (NS compactness,
 * mass ratio m1/m2 >= 1, BH spin); host arrays. Replaces IMRPhenomNSBH.xiTide_interp
 * (gwfast/waveforms.py:3373, gwfast/gwfastUtils.py:1024-1200); builds the table if needed. */
int gwf_xitide(gwf_ctx* ctx, const double* comp, const double* q, const double* chi_bh, int64_t n, double* out);

/* IMRPhenomD quasi-normal-mode table (spin, fring, fdamp), gwfast/waveforms.py:988-990. */
int gwf_set_qnm_table(gwf_ctx* ctx, const double* spin, const double* fring, const double* fdamp, int64_t n);

/* Register one detector and its PSD (strictly increasing psd_f, PSD not ASD).
 * Replaces GWSignal.__init__ geometry and noise-curve loading, gwfast/signal.py:86-147. */
int gwf_detector_add(gwf_ctx* ctx, const gwf_det_desc* desc, const double* psd_f, const double* psd_S,
                     int64_t n, int* det_id);

/* Optimal SNR of N events in n_det detectors.
 * Replaces GWSignal.SNRInteg (gwfast/signal.py:658-777) and DetNet.SNR (gwfast/network.py:53-82).
 * out_arm (may be NULL): per arm slot (L: 1 slot, triangle: 3 slots, in det_ids order),
 *   [slots][N] of trapz((A+^2 + Ax^2)/S, f), i.e. (SNR_arm / 2)^2.
 * out_net (may be NULL): [N] network SNR^2 = sum over arms of 4 * out_arm.
 * precision: GWF_PREC_FP64, or GWF_PREC_FP32 (TaylorF2, IMRPhenomD and IMRPhenomHM: per-point
 * amplitude, pattern functions and Earth-rotation time in FP32, IMRPhenomHM's mode phases in FP64
 * reduced modulo 2 pi, per-thread compensated sums, FP64 block sums). */
int gwf_snr(gwf_ctx* ctx, int n_det, const int* det_ids, const gwf_wf_desc* wf, const double* params, int64_t ld,
            int64_t n_events, int32_t res, const int32_t* res_per_event, int spacing, int precision, int mem,
            double* out_arm, double* out_net, void* stream);

/* Fisher matrices of N events in n_det detectors.
 * Replaces GWSignal.FisherMatr (gwfast/signal.py:782-1098, default arguments
 * use_chi1chi2=True, computeAnalyticalDeriv=True) and DetNet.FisherMatr (gwfast/network.py:84-153).
 * per_arm != 0: out_arm receives [slots][N][11][11] per arm (return_all=True);
 * out_net (may be NULL): [N][11][11] network total.
 * precision: GWF_PREC_FP64 (the drop-in) or GWF_PREC_FP32 (split precision: per-event set-up in
 * FP64, per-point arithmetic in FP32, outputs in FP64; IMRPhenomHM with its mode phases in FP64), or
 * GWF_PREC_MIXED: GWF_PREC_FP32 for all events, then the events whose network Fisher has an
 * equilibrated condition number above the context's threshold (gwf_set_refine_cond, default
 * 1e13) or a non-finite one are recomputed in FP64 (all outputs), each detector's pass on its own
 * stream. With mem = GWF_MEM_DEVICE,
 * GWF_PREC_MIXED waits on the stream once, to read how many events need FP64. */
int gwf_fisher(gwf_ctx* ctx, int n_det, const int* det_ids, const gwf_wf_desc* wf, const double* params, int64_t ld,
               int64_t n_events, int32_t res, const int32_t* res_per_event, int spacing, int per_arm, int precision,
               int mem, double* out_arm, double* out_net, void* stream);

/* gwf_fisher plus the SNR derivatives (GWSignal.FisherMatr / DetNet.FisherMatr with
 * return_SNR_derivatives=True, gwfast/signal.py:938-945, :1016-1022, :1090-1094; gwfast/network.py:139-145):
 * out_snr_der_arm (may be NULL): [slots][N][11] per arm, 4 trapz(Re(h conj(dh/dtheta)) / S, f)
 * (tcoal in seconds); out_snr_der_net (may be NULL): [N][11] the same summed over all arms.
 * Divided by the network SNR, the sum is d SNR / d theta. Same precision forms; the column changes
 * of the FP32 form are undone as for the Fisher. out_arm / out_net may both be NULL. */
int gwf_fisher_ex(gwf_ctx* ctx, int n_det, const int* det_ids, const gwf_wf_desc* wf, const double* params, int64_t ld,
                  int64_t n_events, int32_t res, const int32_t* res_per_event, int spacing, int per_arm, int precision,
                  int mem, double* out_arm, double* out_net, double* out_snr_der_arm, double* out_snr_der_net,
                  void* stream);

/* Strain derivatives on the frequency grid of each event, one detector (GWSignal.FisherMatr with
 * return_derivatives=True, gwfast/signal.py:938-939, :974-975, :1014-1015, :1048-1049, :1078-1079;
 * gwfast/network.py:130-137). out: complex128 as interleaved (re, im) doubles,
 * [arms][11][N][res], arms = 1 (L) or 3 (triangle; the third arm is minus the sum of the first
 * two); d h / d theta in the Fisher parameter order with the tcoal row in 1/s. FP64, one res for
 * all events (as gwfast). With mem = GWF_MEM_HOST the output is staged through a device buffer of
 * about 1 GiB per launch. */
int gwf_strain_derivs(gwf_ctx* ctx, int det_id, const gwf_wf_desc* wf, const double* params, int64_t ld,
                      int64_t n_events, int32_t res, int spacing, int mem, double* out, void* stream);

/* The strain on caller-given frequencies, one detector: GWSignal.GWstrain, GWAmplitudes and GWPhase
 * (gwfast/signal.py:425-655). freqs (Hz, > 0, any order; mem as the other arrays): one row of n_freq
 * frequencies for every event (f_ld = 0) or a row per event ([N][f_ld], f_ld >= n_freq). Beyond the
 * model's cut the IMR amplitudes are zero, as in gwfast. Outputs, each may be NULL (not all):
 *   out_strain [arms][N][n_freq] complex as interleaved (re, im) doubles: h = (A+ + i Ax) e^{i Psi};
 *   out_amp    [arms][N][n_freq] (A+, Ax) pairs: A (1 + cos^2 iota) / 2 F+ and A cos iota Fx for the
 *              22-mode models, |h+| F+ and |hx| Fx for IMRPhenomHM (gwfast/signal.py:457-463);
 *   out_phase  [2][N][n_freq]: [0] GWPhase = 2 pi f tcoal - Phicoal - Phi(f) (tcoal in days of 86400 s),
 *              [1] Psi = GWPhase + 2 pi f Delta t_loc, the strain's phase at the detector (the
 *              22-mode models; IMRPhenomHM's phase is one per mode: GWF_ERR_UNSUPPORTED).
 * arms = 1 (L) or 3 (triangle: the arms of rot = 0, 60, 120 degrees in gwfast, the third minus the
 * sum of the first two). Parameters as in gwf_fisher (Fisher order). FP64. */
int gwf_strain(gwf_ctx* ctx, int det_id, const gwf_wf_desc* wf, const double* params, int64_t ld, int64_t n_events,
               const double* freqs, int64_t f_ld, int32_t n_freq, int mem, double* out_strain, double* out_amp,
               double* out_phase, void* stream);

/* Overlap integrals of two waveforms on two parameter sets (GWSignal.WFOverlap with
 * return_separate=True, gwfast/signal.py:1759-1921; DetNet.WFOverlap, gwfast/network.py:198-227).
 * Per detector i and event n, on the geometric grid from fmin to max(fcut_1, fcut_2) (with a
 * detector fmax: fmax where that maximum exceeds it, else fcut_1, as gwfast), summed over the
 * detector's arms: out_ov[i][n] = 4 trapz(Re(h1 conj h2) / S), out_n1[i][n] = 4 trapz(|h1|^2 / S),
 * out_n2[i][n] = 4 trapz(|h2|^2 / S). The overlap is out_ov / sqrt(out_n1 out_n2) after summing
 * each over detectors. FP64. */
int gwf_overlap(gwf_ctx* ctx, int n_det, const int* det_ids, const gwf_wf_desc* wf1, const double* params1,
                int64_t ld1, const gwf_wf_desc* wf2, const double* params2, int64_t ld2, int64_t n_events, int32_t res,
                int mem, double* out_ov, double* out_n1, double* out_n2, void* stream);

/* Detector groups for network totals (no counterpart in gwfast: a launch-shape choice). on != 0 (the
 * default): in gwf_fisher with per_arm = 0, no SNR derivatives and no segments, detectors with the
 * same fmin, fmax and Earth-rotation flag (up to four) are evaluated by one launch that computes the
 * waveform and its tangent once per frequency point and accumulates all their derivative vectors into
 * one Gram (TaylorF2, IMRPhenomD and IMRPhenomHM, every precision; in FP64 the same sums in another
 * order; the mixed form's FP64 recomputation groups the same way). Detectors with identical PSD
 * tables share the per-point weight. on = 0: one launch per detector. */
int gwf_set_detector_groups(gwf_ctx* ctx, int on);

/* Kernel timing (an extension for measurement; no counterpart in gwfast). on != 0: the following
 * gwf_snr / gwf_fisher calls record CUDA events around their main sections, each on the stream it
 * runs on, so that the time of a kernel is measured without the rest of the call: the per-event
 * set-up launches of a chunk (GWF_KT_SETUP), the FP32 launch of a detector group
 * (GWF_KT_GROUP_F32), a per-detector FP32 or FP64 Fisher launch (GWF_KT_FISHER_F32,
 * GWF_KT_FISHER_F64) and a segmented launch sequence (GWF_KT_SEGMENTED: scan, persistent kernel,
 * reduction). Nothing is recorded inside a CUDA-graph capture or a replay. Each call starts a new
 * list (at most 64 sections). gwf_kernel_times waits for the last call's events and writes up to
 * max_entries (kind, milliseconds) pairs and the number of sections taken. */
enum { GWF_KT_SETUP = 1, GWF_KT_GROUP_F32 = 2, GWF_KT_FISHER_F32 = 3, GWF_KT_FISHER_F64 = 4, GWF_KT_SEGMENTED = 5 };
int gwf_set_kernel_timing(gwf_ctx* ctx, int on);
int gwf_kernel_times(gwf_ctx* ctx, int max_entries, int* kind, double* ms, int* n_entries);

/* Condition-number threshold of GWF_PREC_MIXED (no counterpart in gwfast: a property of the
 * reduced-precision form). kappa > 0; events with equilibrated condition number above it get FP64. */
int gwf_set_refine_cond(gwf_ctx* ctx, double kappa);

/* Work decomposition of gwf_fisher (no counterpart in gwfast: a launch-shape choice).
 * points = 0: one CTA per (event, detector), the default. points > 0 (a multiple of 128): every
 * event is cut into frequency segments of that many points; persistent CTAs take segments from
 * an atomic counter (work stealing), and a second kernel sums each event's segment Grams in
 * order (deterministic). Catalogues whose events have very different grid lengths
 * (res_per_event) keep every SM busy this way. */
int gwf_set_segments(gwf_ctx* ctx, int points);

/* CUDA graphs for device-resident calls (no counterpart in gwfast). on != 0: a gwf_fisher call with
 * mem = GWF_MEM_DEVICE and precision FP64 or FP32 is captured into a CUDA graph the second time the
 * same call (same arguments, pointers and stream included) is made, and later identical calls
 * replay the graph: one launch instead of the per-chunk set-up, scan, persistent and reduction
 * launches of every detector. The inputs behind the pointers may change between calls. A graph
 * is dropped when the context's buffers are reallocated. GWF_PREC_MIXED calls read a count back
 * to the host and are never captured. */
int gwf_set_graphs(gwf_ctx* ctx, int on);

/* Autotuner for gwf_set_segments: runs the given workload (typically a sample of the catalogue)
 * as gwf_fisher would, with each candidate segment length (0 = per event, 256, 512, 1024, 2048),
 * times each with CUDA events (one warm-up and two timed runs), keeps the fastest in the context
 * and returns it in *best. Arguments as gwf_fisher. */
int gwf_autotune_segments(gwf_ctx* ctx, int n_det, const int* det_ids, const gwf_wf_desc* wf, const double* params,
                          int64_t ld, int64_t n_events, int32_t res, const int32_t* res_per_event, int spacing,
                          int precision, int mem, int* best);

/* Covariance by equilibrated Cholesky inversion, FP64, one 11x11 matrix per event.
 * Replaces fisherTools.CovMatr 'cho' path (gwfast/fisherTools.py:32-196) together with
 * compute_inversion_error (:199-212); cond receives the condition number of the
 * diagonally equilibrated matrix (:81-88).  F, cov: [N][11][11]; eps, cond: [N] (may be NULL).
 * Events whose equilibrated matrix is not positive definite get NaN covariances. */
int gwf_cov(gwf_ctx* ctx, const double* F, int64_t n_events, int mem, double* cov, double* eps, double* cond,
            void* stream);

/* gwf_cov for P x P matrices, P = n_params = 11, 13 (tidal models) or 14 (tidal eccentric TaylorF2; smaller
 * matrices, e.g. after fixParams, are embedded with an identity block by the caller); F, cov [N][P][P]. */
int gwf_cov_n(gwf_ctx* ctx, const double* F, int64_t N, int n_params, int mem, double* cov, double* eps, double* cond,
              void* stream);

/* Learned SNR screen (no counterpart in gwfast: a method-level addition). A multilayer perceptron,
 * 11 features -> `layers` hidden layers of `hidden` SiLU units -> ln(network SNR), trained on SNRs
 * from gwf_snr. Weights are stored in FP32 (the optimiser's copy) and used in BF16; arithmetic
 * accumulates in FP32. Features: ln Mc, eta, ln dL, cos theta, sin and cos of (phi - 2 pi tcoal),
 * cos iota, sin and cos of 2 psi, chi1z, chi2z, standardised by the mean and deviation of the
 * training events. params as in gwf_fisher ([11][ld], Fisher order); mem as in gwf_fisher. The MLP
 * lives on the context's device and runs on its own stream; calls are synchronous. With hidden a
 * multiple of 64 up to 256, the hidden-to-hidden products run on the tensor cores (tcgen05.mma, BF16
 * operands, FP32 accumulation in tensor memory): in training as one GEMM per layer and pass, in
 * gwf_mlp_predict as one fused kernel per 128 events with the activations kept on chip. A tensor-core
 * completion wait that runs out returns GWF_ERR_TIMEOUT (the GPU stays usable). */
int gwf_mlp_create(gwf_ctx* ctx, int hidden, int layers, uint64_t seed, gwf_mlp** out);
int gwf_mlp_destroy(gwf_mlp* mlp);
/* weights + biases in the flat layout [W_0 (11 x H), W_1 (H x H), ..., W_L (H x 1), b_0, ..., b_L],
 * each W row-major (input index major) */
int gwf_mlp_num_weights(gwf_mlp* mlp, int64_t* n);
/* FP32 weights (may be NULL) and the standardisation [mean[11], 1/deviation[11]] (may be NULL) */
int gwf_mlp_get_weights(gwf_mlp* mlp, float* weights, float* norm);
int gwf_mlp_set_weights(gwf_mlp* mlp, const float* weights, const float* norm);
/* Adam (beta 0.9, 0.999) on the mean squared error of the predicted ln SNR against target_ln_snr,
 * minibatches drawn with replacement, learning rate lr with cosine decay over the run; sets the
 * standardisation from these events. final_loss: mean batch loss of the last epoch. */
int gwf_mlp_train(gwf_mlp* mlp, const double* params, int64_t ld, int64_t n_events, const double* target_ln_snr,
                  int epochs, int batch, double lr, uint64_t seed, int mem, double* final_loss);
/* one forward and backward pass over all n events as one batch: loss and the gradient of the loss
 * with respect to every weight and bias (flat layout above), for checking against a CPU model */
int gwf_mlp_gradients(gwf_mlp* mlp, const double* params, int64_t ld, int64_t n_events, const double* target_ln_snr,
                      int mem, double* loss, float* grad);
/* predicted ln(network SNR) of n events */
int gwf_mlp_predict(gwf_mlp* mlp, const double* params, int64_t ld, int64_t n_events, int mem, double* out_ln_snr);

/* Limits of gwf_fisher_noalloc: its scratch is one fixed array of GWF_NOALLOC_SCRATCH_MIB MiB
 * per GPU that loads the library, held until the process exits. */
#define GWF_NOALLOC_SCRATCH_MIB 24
#define GWF_NOALLOC_MAX_PSD 16384 /* PSD table rows */
#define GWF_NOALLOC_MAX_QNM 2048  /* QNM table rows */

/* FP64 Fisher matrices of one detector, with no device memory allocated by the library.
 *
 * No counterpart in the reference: this entry point exists for callers that cannot call
 * cudaMalloc — programs whose device memory belongs to their own pool allocator (a framework
 * that reserves the GPU at start-up, where a library's cudaMalloc fails or fragments the
 * pool), or loops that cannot take the device synchronisation of cudaMalloc/cudaFree. It needs
 * no context. The caller passes the detector, its PSD table and (IMRPhenomD only) the QNM table
 * in host memory, as gwf_detector_add and gwf_set_qnm_table take them, and params ([11][ld],
 * Fisher order, float64) and out ([n_events][11][11], float64) in DEVICE memory. accumulate != 0
 * adds into out, so a network is the sum of calls over its detectors. Geometric frequency
 * grid with res points per event; detector total over the arms of a triangle.
 *
 * Scratch (the PSD table and its index, the QNM table and the per-event set-up records) lives
 * in a file-scope __device__ array of GWF_NOALLOC_SCRATCH_MIB MiB; events run in passes that fit
 * it. PSD tables longer than GWF_NOALLOC_MAX_PSD rows or QNM tables longer than
 * GWF_NOALLOC_MAX_QNM rows are rejected with GWF_ERR_INVALID_ARG. The array belongs to the CUDA
 * context that is current at the call: the first call in a context (with its device current)
 * looks the array's address up and caches it under the context's unique ID, so a context made
 * later (after cudaDeviceReset, say) does its own lookup; make that first call before any stream
 * capture in the context. Every call shares the array and rewrites what it reads; calls whose GPU
 * work overlaps (unordered streams) race on it. The host tables are copied with
 * cudaMemcpyAsync on the stream: from pageable memory the call returns after they have been
 * read, but page-locked tables are read when the stream reaches the copy, so keep them
 * unchanged until then. stream NULL = the default stream. */
int gwf_fisher_noalloc(const gwf_det_desc* det, const double* psd_f, const double* psd_S, int64_t n_psd,
                       const gwf_wf_desc* wf, const double* qnm_spin, const double* qnm_fring, const double* qnm_fdamp,
                       int64_t n_qnm, const double* params, int64_t ld, int64_t n_events, int32_t res, int accumulate,
                       double* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GWFAST_GB300_H */
