"""GWSignal: one detector, with gwfast's constructor and SNRInteg/FisherMatr signatures.

Replaces gwfast/signal.py:37-1098.  The frequency grid, PSD interpolation, waveform,
analytic tangent, projection and the PSD-weighted Gram integral all run in one
fused CUDA kernel per detector (libgwfast_gb300.so); this module only builds the
event arrays, applies gwfast's host-side conventions (dict mutation, ValueError
on missing parameters, duty-factor masks, parameter reparametrisations) and
reshapes the outputs.
"""
import numpy as np

from . import _lib
from . import gwfastUtils as utils
from .waveforms import PARAMS

DAY = 3600. * 24.


def event_array(evParams, params=PARAMS):
    """(P, N) float64 array in the Fisher order from the events dict (P = 11, or 13 with the tidal
    parameters)."""
    cols = [np.atleast_1d(np.asarray(evParams[k], dtype=np.float64)) for k in params]
    n = max(len(c) for c in cols)
    cols = [np.broadcast_to(c, (n,)) if len(c) != n else c for c in cols]
    return np.ascontiguousarray(np.stack(cols))


def _prep(evParams, wf=None):
    utils.check_evparams(evParams)
    utils.fill_spins(evParams)
    if wf is not None and wf.is_tidal:
        utils.fill_tidal(evParams)
    if wf is not None and wf.is_eccentric and 'ecc' not in evParams:
        raise ValueError('Eccentricity has to be provided.')   # gwfast/signal.py:876-880
    if wf is not None and (wf.is_tidal or wf.is_eccentric):
        return event_array(evParams, wf.params)
    return event_array(evParams)


def _arm_slots(signals):
    return [1 if s.detector_shape == 'L' else 3 for s in signals]


def snr_batch(signals, evParams, res=1000, device=0, precision='fp64', res_per_event=None):
    """Per-arm SNRs of all signals in one library call.  Returns a list (per signal) of (arms, N) arrays.

    precision: 'fp64' or 'fp32' (TaylorF2 and IMRPhenomD); res_per_event as in fisher_batch."""
    wf = signals[0].wf_model
    p = _prep(evParams, wf)
    if any(type(s.wf_model) is not type(wf) for s in signals):
        return [s._snr_arms(evParams, res, precision) for s in signals]
    N = p.shape[1]
    slots = _arm_slots(signals)
    out = np.empty((sum(slots), N))
    ctx = _lib.context(device)
    rev = None if res_per_event is None else np.ascontiguousarray(np.broadcast_to(res_per_event, (N,)), dtype=np.int32)
    ctx.snr([s.det_id for s in signals], wf.gpu_desc(), p, res, res_ev=rev, out_arm=out, precision=precision)
    res_l, i = [], 0
    for s, k in zip(signals, slots):
        arms = 2. * np.sqrt(out[i:i + k])
        arms = s._apply_duty(arms, seed=True)
        res_l.append(arms)
        i += k
    return res_l


def fisher_batch(signals, evParams, res=1000, per_arm=False, spacing='geom', device=0, precision='fp64',
                 refine_cond=None, res_per_event=None, snr_derivs=False):
    """Fisher matrices of all signals in one library call.

    per_arm: list (per signal) of (arms, N, P, P); otherwise the network total (N, P, P); P = 11, or 13
    for the tidal TaylorF2 (LambdaTilde, deltaLambda last).
    res_per_event: optional (N,) grid lengths, one per event (an extension: gwfast uses one res).
    snr_derivs: also return, per signal, (arms, N, 11) of 4 trapz(Re(h conj(dh/dtheta)) / S) (the
    per-arm SNR-derivative integrals of gwfast's return_SNR_derivatives); the Fisher part is then
    per arm.
    precision: 'fp64' (the drop-in), 'fp32' (split precision; IMRPhenomHM with FP64 mode phases), or
    'mixed' ('fp32', then FP64 for the events whose network Fisher has an equilibrated condition
    number above refine_cond, default 1e13).
    """
    wf = signals[0].wf_model
    p = _prep(evParams, wf)
    N = p.shape[1]
    P = wf.nParams
    slots = _arm_slots(signals)
    ctx = _lib.context(device)
    if precision == 'mixed':
        ctx.set_refine_cond(1e13 if refine_cond is None else refine_cond)
    sp = 0 if spacing == 'geom' else 1
    rev = None if res_per_event is None else np.ascontiguousarray(np.broadcast_to(res_per_event, (N,)), dtype=np.int32)
    duty = any(s.DutyFactor is not None for s in signals)
    if per_arm or duty or snr_derivs:
        out = np.empty((sum(slots), N, P, P))
        sd = np.empty((sum(slots), N, P)) if snr_derivs else None
        ctx.fisher([s.det_id for s in signals], wf.gpu_desc(), p, res, res_ev=rev, spacing=sp, per_arm=True,
                   out_arm=out, precision=precision, out_sd_arm=sd)
        res_l, sd_l, i = [], [], 0
        for s, k in zip(signals, slots):
            res_l.append(s._apply_duty(out[i:i + k], seed=True))
            if snr_derivs:
                sd_l.append(s._apply_duty(sd[i:i + k], seed=True))
            i += k
        if snr_derivs:
            return res_l, sd_l
        if per_arm:
            return res_l
        return sum(r.sum(axis=0) for r in res_l)
    out = np.empty((N, P, P))
    ctx.fisher([s.det_id for s in signals], wf.gpu_desc(), p, res, res_ev=rev, spacing=sp, per_arm=False,
               out_net=out, precision=precision)
    return out


def strain_derivs_batch(signal, evParams, res=1000, spacing='geom'):
    """d h / d theta on each event's grid for one detector: complex128 (arms, P, N, res), tcoal
    row in 1/s (the per-arm arrays of gwfast's return_derivatives, gwfast/signal.py:938-939)."""
    wf = signal.wf_model
    p = _prep(evParams, wf)
    N = p.shape[1]
    arms = 1 if signal.detector_shape == 'L' else 3
    out = np.empty((arms, wf.nParams, N, int(res)), dtype=np.complex128)
    _lib.context(signal.device).strain_derivs(signal.det_id, signal.wf_model.gpu_desc(), p, res,
                                              spacing=0 if spacing == 'geom' else 1, out=out)
    return out


def overlap_batch(signals, WF1, WF2, evParams1, evParams2, res=1000):
    """Per detector (n_det, N) arrays (4 trapz(Re(h1 conj h2)/S), 4 trapz(|h1|^2/S), 4 trapz(|h2|^2/S)),
    summed over each detector's arms (gwfast/signal.py:1759-1921)."""
    p1 = _prep(evParams1, WF1)
    p2 = _prep(evParams2, WF2)
    if p1.shape[1] != p2.shape[1]:
        raise ValueError('the two parameter sets must hold the same number of events')
    N = p1.shape[1]
    ov, n1, n2 = (np.empty((len(signals), N)) for _ in range(3))
    _lib.context(signals[0].device).overlap([s.det_id for s in signals], WF1.gpu_desc(), p1, WF2.gpu_desc(), p2, res,
                                            out_ov=ov, out_n1=n1, out_n2=n2)
    return ov, n1, n2


def _jacobian(evParams, N, use_m1m2, use_chi1chi2, P=11):
    J = np.broadcast_to(np.eye(P), (N, P, P)).copy()
    if use_m1m2:
        m1, m2 = utils.m1m2_from_Mceta(np.asarray(evParams['Mc']), np.asarray(evParams['eta']))
        Mc, eta = utils.Mceta_from_m1m2(m1, m2)
        M = m1 + m2
        J[:, 0, 0] = Mc * (3. / (5. * m1) - 1. / (5. * M))
        J[:, 0, 1] = Mc * (3. / (5. * m2) - 1. / (5. * M))
        J[:, 1, 0] = m2 * (m2 - m1) / M ** 3
        J[:, 1, 1] = m1 * (m1 - m2) / M ** 3
    if not use_chi1chi2:
        J[:, 9, 9] = 1.; J[:, 9, 10] = 1.
        J[:, 10, 9] = 1.; J[:, 10, 10] = -1.
    return J


def reparametrise(F, evParams, use_m1m2=False, use_chi1chi2=True):
    """Chain rule to (m1, m2) and/or (chiS, chiA), F: (..., N, 11, 11) (gwfast/signal.py:818-842)."""
    if not use_m1m2 and use_chi1chi2:
        return F
    J = _jacobian(evParams, F.shape[-3], use_m1m2, use_chi1chi2, F.shape[-1])
    return np.einsum('nai,...nab,nbj->...nij', J, F, J)


def reparametrise_derivs(D, evParams, use_m1m2=False, use_chi1chi2=True):
    """The chain rule for strain derivatives, D: (arms, 11, N, R)."""
    if not use_m1m2 and use_chi1chi2:
        return D
    J = _jacobian(evParams, D.shape[2], use_m1m2, use_chi1chi2, D.shape[1])
    return np.einsum('naj,xanr->xjnr', J, D)


def reparametrise_vec(v, evParams, use_m1m2=False, use_chi1chi2=True):
    """The same chain rule for derivative vectors, v: (..., N, 11)."""
    if not use_m1m2 and use_chi1chi2:
        return v
    J = _jacobian(evParams, v.shape[-2], use_m1m2, use_chi1chi2, v.shape[-1])
    return np.einsum('nai,...na->...ni', J, v)


class GWSignal:
    """One interferometer (gwfast/signal.py:37-160).

    ``psd_path`` may be a two-column text file (as in gwfast) or a tuple ``(f, S)``
    of arrays.  ``device`` selects the CUDA device.
    """

    def __init__(self, wf_model, psd_path=None, detector_shape='T', det_lat=40.44, det_long=9.45, det_xax=0.,
                 verbose=True, is_ASD=True, useEarthMotion=False, noMotion=False, fmin=2., fmax=None,
                 IntTablePath=None, DutyFactor=None, compute2arms=True, jitCompileDerivs=False, device=0):
        if detector_shape not in ('L', 'T'):
            raise ValueError('Enter valid detector configuration')
        if psd_path is None:
            raise ValueError('Enter a valid PSD or ASD path')
        if noMotion:
            raise NotImplementedError('noMotion (a check-only mode of gwfast) is not implemented on the GPU path')
        self.wf_model = wf_model
        self.verbose = verbose
        self.detector_shape = detector_shape
        self.det_lat_rad = det_lat * np.pi / 180.
        self.det_long_rad = det_long * np.pi / 180.
        self.det_xax_rad = det_xax * np.pi / 180.
        self.DutyFactor = DutyFactor
        self.useEarthMotion = useEarthMotion
        self.noMotion = noMotion
        self.fmin = fmin
        self.fmax = fmax
        self.compute2arms = compute2arms
        self.angbtwArms = 0.5 * np.pi if detector_shape == 'L' else np.pi / 3.
        if isinstance(psd_path, (tuple, list)):
            f, S = (np.asarray(a, dtype=np.float64) for a in psd_path)
            self.psd_base_path, self.psd_file_name = '', '<array>'
        else:
            noise = np.loadtxt(psd_path, usecols=(0, 1))
            f, S = noise[:, 0], noise[:, 1]
            self.psd_base_path = '/'.join(psd_path.split('/')[:-1])
            self.psd_file_name = psd_path.split('/')[-1]
        if is_ASD:
            S = S ** 2
        self.strainFreq = f
        self.noiseCurve = S
        np.random.seed(None)
        self.seedUse = np.random.randint(2 ** 32 - 1, size=1)
        self.device = device
        self.det_id = _lib.context(device).add_detector(self.det_lat_rad, self.det_long_rad, self.det_xax_rad,
                                                        detector_shape, useEarthMotion, fmin, fmax, f, S)

    def _update_seed(self, seed=None):
        np.random.seed(None)
        self.seedUse = np.random.randint(2 ** 32 - 1, size=1) if seed is None else seed

    def _duty_masks(self, n_arms, n, seed=True):
        """Bernoulli duty-cycle masks, one per arm, drawn exactly as gwfast draws them
        (gwfast/signal.py:672-673, :729-765, :809-810, :932-937)."""
        if seed:
            np.random.seed(self.seedUse)
        return [np.random.choice([0, 1], n, p=[1. - self.DutyFactor, self.DutyFactor]) for _ in range(n_arms)]

    def _apply_duty(self, arms, seed=True, masks=None):
        """arms: (arms, N, ...) with the duty-cycle mask of each arm applied."""
        if self.DutyFactor is None:
            return arms
        out = np.array(arms, copy=True)
        n = out.shape[1]
        masks = self._duty_masks(out.shape[0], n, seed) if masks is None else masks
        for a in range(out.shape[0]):
            out[a] = out[a] * masks[a].reshape((n,) + (1,) * (out.ndim - 2))
        return out

    def _snr_arms(self, evParams, res, precision='fp64'):
        return snr_batch([self], evParams, res, self.device, precision=precision)[0]

    def SNRInteg(self, evParams, res=1000, return_all=False, precision='fp64'):
        """gwfast/signal.py:658-777; precision='fp32' selects the FP32 SNR kernel."""
        arms = self._snr_arms(evParams, res, precision)
        if self.detector_shape == 'T':
            return arms if return_all else np.sqrt((arms ** 2).sum(axis=0))
        return arms[0]

    def FisherMatr(self, evParams, res=1000, df=None, spacing='geom', use_m1m2=False, use_chi1chi2=True,
                   use_prec_ang=True, computeDerivFinDiff=False, computeAnalyticalDeriv=True, return_all=False,
                   return_derivatives=False, return_SNR_derivatives=False, precision='fp64', **kwargs):
        """gwfast/signal.py:782-1098; returns (P, P, N), or a list per arm with return_all (P = nParams).

        precision='fp32' selects the split-precision kernel (all three models), 'mixed' the
        split-precision kernel with FP64 recomputation of ill-conditioned events (refine_cond)."""
        if computeDerivFinDiff:
            raise NotImplementedError('finite-difference derivatives are not used on the GPU path')
        res = self._resolve_res(evParams, res, df)
        if return_derivatives and not return_SNR_derivatives:
            # as gwfast: per-arm Fisher matrices and per-arm (P, N, R) strain derivatives, the same
            # duty-cycle mask on both
            Fa = fisher_batch([self], evParams, res, per_arm=True, spacing=spacing, device=self.device,
                              precision=precision, refine_cond=kwargs.get('refine_cond'))
            Fa = np.asarray(Fa[0])
            D = strain_derivs_batch(self, evParams, res, spacing)
            if self.DutyFactor is not None:
                # fisher_batch applied the masks drawn from the seed; draw the same ones for D
                masks = self._duty_masks(D.shape[0], D.shape[2])
                D = D * np.stack(masks)[:, None, :, None]
            Fa = reparametrise(Fa, evParams, use_m1m2, use_chi1chi2)
            D = reparametrise_derivs(D, evParams, use_m1m2, use_chi1chi2)
            return [np.moveaxis(F, 0, -1) for F in Fa], [D[i] for i in range(D.shape[0])]
        if return_SNR_derivatives:
            # as gwfast: per-arm Fisher matrices and per-arm (P, N) SNR-derivative integrals
            Fa, Da = fisher_batch([self], evParams, res, per_arm=True, spacing=spacing, device=self.device,
                                  precision=precision, refine_cond=kwargs.get('refine_cond'), snr_derivs=True)
            Fa = reparametrise(Fa[0], evParams, use_m1m2, use_chi1chi2)
            Da = reparametrise_vec(Da[0], evParams, use_m1m2, use_chi1chi2)
            return [np.moveaxis(F, 0, -1) for F in Fa], [np.moveaxis(D, 0, -1) for D in Da]
        Fa = fisher_batch([self], evParams, res, per_arm=True, spacing=spacing, device=self.device,
                          precision=precision, refine_cond=kwargs.get('refine_cond'))[0]
        Fa = reparametrise(Fa, evParams, use_m1m2, use_chi1chi2)
        arms = [np.moveaxis(F, 0, -1) for F in Fa]
        if return_all:
            return arms
        return arms[0] if self.detector_shape == 'L' else np.sum(arms, axis=0)

    def WFOverlap(self, WF1, WF2, evParams1, evParams2, res=1000, return_separate=False, **kwargs):
        """Overlap of two waveforms on two parameter sets in this detector (gwfast/signal.py:1759-1921).
        return_separate: (4 trapz(Re(h1 conj h2)/S), SNR_1, SNR_2) instead of the overlap."""
        ov, n1, n2 = overlap_batch([self], WF1, WF2, evParams1, evParams2, res)
        if return_separate:
            return ov[0], np.sqrt(n1[0]), np.sqrt(n2[0])
        return ov[0] / np.sqrt(n1[0] * n2[0])

    # ---- strain, amplitudes and phase at caller frequencies (gwfast/signal.py:425-655)
    def _strain_parts(self, evParams, f, rot, strain=False, amp=False, phase=False):
        """One library call: the requested parts for the detector's arm at rotation rot (degrees; 0 for
        an L, 0/60/120 for the arms of a triangle), reshaped to the shape of f. f: a scalar or (R,)
        for every event, or (R, N), one column per event (as gwfast's grids)."""
        wf = self.wf_model
        p = _prep(dict(evParams), wf)
        N = p.shape[1]
        fa = np.asarray(f, dtype=np.float64)
        if fa.ndim > 2:
            raise ValueError('f must be a scalar, (R,) or (R, N)')
        if fa.ndim == 2:
            if fa.shape[1] != N:
                raise ValueError('f of shape (R, N) needs one column per event (N = %d)' % N)
            freqs = np.ascontiguousarray(fa.T)
        else:
            freqs = np.ascontiguousarray(np.atleast_1d(fa))
        if np.any(~(freqs > 0.)):
            raise ValueError('frequencies must be positive')
        rots = (0.,) if self.detector_shape == 'L' else (0., 60., 120.)
        arm = [i for i, r in enumerate(rots) if abs(float(rot) - r) < 1e-9]
        if not arm:
            raise NotImplementedError('rot must be one of %s for this detector' % (rots,))
        arms, R = len(rots), freqs.shape[-1]
        hs = np.empty((arms, N, R), dtype=np.complex128) if strain else None
        am = np.empty((arms, N, R), dtype=np.complex128) if amp else None
        ph = np.empty((2, N, R)) if phase else None
        _lib.context(self.device).strain(self.det_id, wf.gpu_desc(), p, freqs, out_strain=hs, out_amp=am, out_phase=ph)

        def shaped(x):   # (N, R) -> the shape of f
            if fa.ndim == 2:
                return np.ascontiguousarray(x.T)
            if fa.ndim == 0:
                return x[0, 0] if N == 1 else x[:, 0]
            return x[0] if N == 1 else np.ascontiguousarray(x.T)
        out = {}
        if strain:
            out['h'] = shaped(hs[arm[0]])
        if amp:
            out['Ap'], out['Ac'] = shaped(am[arm[0]].real), shaped(am[arm[0]].imag)
        if phase:
            out['GWPhase'], out['Psi'] = shaped(ph[0]), shaped(ph[1])
        return out

    def GWAmplitudes(self, evParams, f, rot=0.):
        """Plus and cross amplitudes at the detector (gwfast/signal.py:425-466): A F+ (1 + cos^2 i)/2 and
        A Fx cos i (IMRPhenomHM: |h+| F+, |hx| Fx), pattern functions at the Earth-rotation time of each
        frequency."""
        o = self._strain_parts(evParams, f, rot, amp=True)
        return o['Ap'], o['Ac']

    def GWPhase(self, evParams, f):
        """2 pi f tcoal - Phicoal - Phi(f) (gwfast/signal.py:468-483), tcoal in days; the 22-mode models
        (IMRPhenomHM has one phase per mode)."""
        if self.wf_model.is_HigherModes:
            raise NotImplementedError('GWPhase of a higher-mode model: its phase is one per mode')
        return self._strain_parts(evParams, f, 0., phase=True)['GWPhase']

    def GWstrain(self, f, Mc, eta, dL, theta, phi, iota, psi, tcoal, Phicoal, chiS, chiA, chi1x=0., chi2x=0., chi1y=0.,
                 chi2y=0., LambdaTilde=0., deltaLambda=0., ecc=0., rot=0., is_m1m2=False, is_chi1chi2=False,
                 is_prec_ang=False, is_Lam1Lam2=False, return_single_comp=None):
        """The complex strain at the detector, (A+ + i Ax) e^{i Psi} (gwfast/signal.py:485-655), or one
        component with return_single_comp ('Ap', 'Ac', 'Psip', 'Psic', 'At', 'Psit'). Aligned spins:
        chiS, chiA (or chi1z, chi2z with is_chi1chi2); the in-plane components must be zero."""
        if is_prec_ang or self.wf_model.is_Precessing:
            raise NotImplementedError('precessing waveforms are not implemented on the GPU path')
        if np.any(np.asarray(chi1x) != 0.) or np.any(np.asarray(chi2x) != 0.) or np.any(np.asarray(chi1y) != 0.) \
                or np.any(np.asarray(chi2y) != 0.):
            raise NotImplementedError('in-plane spins need a precessing waveform')
        if is_m1m2:
            Mc, eta = utils.Mceta_from_m1m2(Mc, eta)
        chi1z, chi2z = (chiS, chiA) if is_chi1chi2 else (chiS + chiA, chiS - chiA)
        ev = {'Mc': Mc, 'eta': eta, 'dL': dL, 'theta': theta, 'phi': phi, 'iota': iota, 'psi': psi, 'tcoal': tcoal,
              'Phicoal': Phicoal, 'chi1z': chi1z, 'chi2z': chi2z}
        if self.wf_model.is_tidal:
            if is_Lam1Lam2:
                ev['Lambda1'], ev['Lambda2'] = LambdaTilde, deltaLambda
            else:
                ev['LambdaTilde'], ev['deltaLambda'] = LambdaTilde, deltaLambda
        if self.wf_model.is_eccentric:
            ev['ecc'] = ecc
        hm = self.wf_model.is_HigherModes
        if return_single_comp is None:
            return self._strain_parts(ev, f, rot, strain=True)['h']
        if return_single_comp not in ('Ap', 'Ac', 'Psip', 'Psic', 'At', 'Psit'):
            raise ValueError('Single component to return has to be among Ap, Ac, Psip, Psic')
        if hm:
            if return_single_comp.startswith('Psi'):
                raise NotImplementedError('the phases of a higher-mode strain are not returned separately')
            if return_single_comp == 'At':
                return np.abs(self._strain_parts(ev, f, rot, strain=True)['h'])
            o = self._strain_parts(ev, f, rot, amp=True)
            return np.abs(o[return_single_comp])
        o = self._strain_parts(ev, f, rot, amp=True, phase=True)
        if return_single_comp in ('Ap', 'Ac'):
            return o[return_single_comp]
        if return_single_comp == 'Psip':
            return o['Psi']
        if return_single_comp == 'Psic':
            return o['Psi'] + np.pi * 0.5
        if return_single_comp == 'At':
            return np.abs(o['Ap'] + 1j * o['Ac'])
        return o['Psi'] + np.arctan2(o['Ac'], o['Ap'])

    def _resolve_res(self, evParams, res, df):
        if res is None and df is not None:
            utils.check_evparams(evParams)
            fcut = self.wf_model.fcut(**evParams)
            if self.fmax is not None:
                fcut = np.where(fcut > self.fmax, self.fmax, fcut)
            res = np.amax(np.floor(1 + (fcut - self.fmin) / df))
        elif res is None:
            raise ValueError('Provide either resolution in frequency or step size.')
        return int(res)
