"""Waveform model descriptors with gwfast's interface (gwfast/waveforms.py:49-199, :697, :959, :1838).

The waveforms themselves are evaluated inside the fused CUDA kernels; these
objects carry what gwfast's callers read from a model (``ParNums``, ``nParams``,
the ``is_*`` flags, ``objType``, ``fcut``) plus the descriptor the C ABI needs.
Supported: TaylorF2_RestrictedPN (optionally with the 3.5PN spin-spin terms and with the tidal
terms, 13 parameters), IMRPhenomD, IMRPhenomHM and IMRPhenomD_NRTidalv2 (13 parameters), aligned
spins, no eccentricity.
"""
import numpy as np

from . import _lib
from . import gwfastGlobals as glob

PARAMS = ('Mc', 'eta', 'dL', 'theta', 'phi', 'iota', 'psi', 'tcoal', 'Phicoal', 'chi1z', 'chi2z')
PARAMS_TIDAL = PARAMS + ('LambdaTilde', 'deltaLambda')   # gwfast/waveforms.py:106-109


class WaveFormModel:
    """Base class mirroring gwfast's WaveFormModel (gwfast/waveforms.py:49-147)."""

    def __init__(self, objType, fcutPar, is_newtonian=False, is_tidal=False, is_HigherModes=False, is_chi1chi2=True,
                 is_Precessing=False, is_LAL=False, is_prec_ang=False, is_eccentric=False, is_holomorphic=False,
                 apply_fcut=True):
        tidal_ok = type(self).__name__ in ('TaylorF2_RestrictedPN', 'IMRPhenomD_NRTidalv2')
        for flag, name in ((is_newtonian, 'is_newtonian'), (is_tidal and not tidal_ok, 'is_tidal'),
                           (is_Precessing, 'is_Precessing'), (is_LAL, 'is_LAL'), (is_eccentric, 'is_eccentric')):
            if flag:
                raise NotImplementedError('%s waveforms are not implemented on the GPU path' % name)
        if not apply_fcut:
            raise NotImplementedError('apply_fcut=False is not implemented on the GPU path')
        self.objType = objType
        self.fcutPar = fcutPar
        self.is_newtonian = is_newtonian
        self.is_tidal = is_tidal
        self.is_HigherModes = is_HigherModes
        self.is_chi1chi2 = is_chi1chi2
        self.is_Precessing = is_Precessing
        self.is_LAL = is_LAL
        self.is_prec_ang = is_prec_ang
        self.is_eccentric = is_eccentric
        self.is_holomorphic = is_holomorphic
        self.apply_fcut = apply_fcut
        self.nParams = 13 if is_tidal else 11
        if is_chi1chi2:
            self.ParNums = {'Mc': 0, 'eta': 1, 'dL': 2, 'theta': 3, 'phi': 4, 'iota': 5, 'psi': 6, 'tcoal': 7,
                            'Phicoal': 8, 'chi1z': 9, 'chi2z': 10}
        else:
            self.ParNums = {'Mc': 0, 'eta': 1, 'dL': 2, 'theta': 3, 'phi': 4, 'iota': 5, 'psi': 6, 'tcoal': 7,
                            'Phicoal': 8, 'chiS': 9, 'chiA': 10}
        if is_tidal:
            self.ParNums['LambdaTilde'] = 11
            self.ParNums['deltaLambda'] = 12

    @property
    def params(self):
        """Names of the Fisher parameters in order (the rows of the event array)."""
        return PARAMS_TIDAL if self.is_tidal else PARAMS

    def fcut(self, **kwargs):
        """Cut frequency in Hz (gwfast/waveforms.py:190-199)."""
        return self.fcutPar / (np.asarray(kwargs['Mc']) / (np.asarray(kwargs['eta']) ** (3. / 5.)))

    def gpu_desc(self):
        name = type(self).__name__
        model = _lib.MODEL_TF2_TIDAL if (self.is_tidal and name == 'TaylorF2_RestrictedPN') else _lib.MODEL_IDS[name]
        return _lib.WfDesc(model, int(getattr(self, 'use_3p5PN_SpinHO', False)), float(self.fcutPar))

    def _device_only(self, *a, **k):
        raise NotImplementedError('%s is evaluated inside the fused GPU kernels; use GWSignal / DetNet'
                                  % type(self).__name__)

    Phi = Ampl = hphc = _device_only


class TaylorF2_RestrictedPN(WaveFormModel):
    """gwfast/waveforms.py:697-953 (fcut: twice the Schwarzschild ISCO by default). is_tidal adds the
    5PN and 6PN tidal phase terms and the parameters LambdaTilde, deltaLambda (FP64 path only)."""

    def __init__(self, fHigh=None, is_tidal=False, use_3p5PN_SpinHO=False, phiref_vlso=False, is_eccentric=False,
                 fRef_ecc=None, which_ISCO='Schw', use_QuadMonTid=False, **kwargs):
        if fHigh is None:
            fHigh = 1. / (6. * np.pi * np.sqrt(6.) * glob.GMsun_over_c3)
        if phiref_vlso or which_ISCO != 'Schw' or use_QuadMonTid:
            raise NotImplementedError('phiref_vlso, Kerr ISCO and QuadMonTid are not implemented on the GPU path')
        self.use_3p5PN_SpinHO = use_3p5PN_SpinHO
        self.phiref_vlso = phiref_vlso
        self.fRef_ecc = fRef_ecc
        self.which_ISCO = which_ISCO
        self.use_QuadMonTid = use_QuadMonTid
        super().__init__('BNS' if is_tidal else 'BBH', fHigh, is_tidal=is_tidal, is_eccentric=is_eccentric,
                         is_holomorphic=True, **kwargs)


class IMRPhenomD(WaveFormModel):
    """gwfast/waveforms.py:959-1333 (fRef = lowest grid frequency)."""

    def __init__(self, fRef=None, **kwargs):
        if fRef is not None:
            raise NotImplementedError('a fixed fRef is not implemented on the GPU path')
        self.AMP_fJoin_INS = 0.014
        self.PHI_fJoin_INS = 0.018
        self.fRef = fRef
        super().__init__('BBH', 0.2, **kwargs)

    def fcut(self, **kwargs):
        """gwfast/waveforms.py:1324-1333."""
        return self.fcutPar / (np.asarray(kwargs['Mc']) * glob.GMsun_over_c3 / (np.asarray(kwargs['eta']) ** (3. / 5.)))


class IMRPhenomHM(IMRPhenomD):
    """gwfast/waveforms.py:1838-2750 (modes 21, 22, 32, 33, 43, 44)."""

    def __init__(self, fRef=None, **kwargs):
        kwargs['is_HigherModes'] = True
        super().__init__(fRef=fRef, **kwargs)
        self.complShiftm = np.array([0., np.pi * 0.5, 0., -np.pi * 0.5, np.pi, np.pi * 0.5, 0.])


class IMRPhenomD_NRTidalv2(WaveFormModel):
    """gwfast/waveforms.py:1339-1836: IMRPhenomD with the spin-induced quadrupole, the NRTidalv2 tidal
    phase and amplitude and a Planck taper (13 parameters, FP64 path only)."""

    def __init__(self, fRef=None, **kwargs):
        if fRef is not None:
            raise NotImplementedError('a fixed fRef is not implemented on the GPU path')
        self.AMP_fJoin_INS = 0.014
        self.PHI_fJoin_INS = 0.018
        self.fRef = fRef
        super().__init__('BNS', 0.2, is_tidal=True, **kwargs)

    def fcut(self, **kwargs):
        """1.2 times the merger frequency of the Planck taper, in Hz (gwfast/waveforms.py:1798-1832)."""
        from . import gwfastUtils as utils
        Mc, eta = np.asarray(kwargs['Mc']), np.asarray(kwargs['eta'])
        M = Mc / eta ** (3. / 5.)
        if 'Lambda1' in kwargs:
            l1, l2 = np.asarray(kwargs['Lambda1']), np.asarray(kwargs['Lambda2'])
        elif 'LambdaTilde' in kwargs:
            l1, l2 = utils.Lam12_from_Lamt_delLam(np.asarray(kwargs['LambdaTilde']), np.asarray(kwargs['deltaLambda']), eta)
        else:
            l1, l2 = np.zeros(M.shape), np.zeros(M.shape)
        seta = np.sqrt(np.where(eta < 0.25, 1.0 - 4.0 * eta, 0.))
        q = 0.5 * (1.0 + seta - 2.0 * eta) / eta
        xa, xb = 0.5 * (1.0 + seta), 0.5 * (1.0 - seta)
        kap = (3.0 / 13.0) * ((1.0 + 12.0 * xb / xa) * xa ** 5 * l1 + (1.0 + 12.0 * xa / xb) * xb ** 5 * l2)
        num = 1.0 + 3.35411203e-2 * kap + 4.31460284e-5 * kap * kap
        den = 1.0 + 7.54224145e-2 * kap + 2.23626859e-4 * kap * kap
        f_merger = 0.3586 / np.sqrt(q) * (num / den) / (2. * np.pi)
        return 1.2 * f_merger / (M * glob.GMsun_over_c3)

