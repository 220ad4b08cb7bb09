"""Waveform model descriptors with gwfast's interface (gwfast/waveforms.py:49-199, :697, :959, :1838).

The waveforms themselves are evaluated inside the fused CUDA kernels; these
objects carry what gwfast's callers read from a model (``ParNums``, ``nParams``,
the ``is_*`` flags, ``objType``, ``fcut``) plus the descriptor the C ABI needs.
Supported: TaylorF2_RestrictedPN (with its options: the 3.5PN spin-spin terms, the tidal terms (13
parameters), orbital eccentricity (+ ecc: 12 or 14 parameters), the phase referenced at the last
stable orbit, the Kerr-ISCO cut, the spin-induced quadrupole of tidal bodies), IMRPhenomD,
IMRPhenomHM, IMRPhenomD_NRTidalv2 and IMRPhenomNSBH (13 parameters), aligned spins.
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
        tidal_ok = type(self).__name__ in ('TaylorF2_RestrictedPN', 'IMRPhenomD_NRTidalv2', 'IMRPhenomNSBH')
        ecc_ok = type(self).__name__ == 'TaylorF2_RestrictedPN'
        for flag, name in ((is_newtonian, 'is_newtonian'), (is_tidal and not tidal_ok, 'is_tidal'),
                           (is_Precessing, 'is_Precessing'), (is_LAL, 'is_LAL'),
                           (is_eccentric and not ecc_ok, 'is_eccentric')):
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
        self.nParams = 11 + (2 if is_tidal else 0) + (1 if is_eccentric else 0)
        if is_chi1chi2:
            self.ParNums = {'Mc': 0, 'eta': 1, 'dL': 2, 'theta': 3, 'phi': 4, 'iota': 5, 'psi': 6, 'tcoal': 7,
                            'Phicoal': 8, 'chi1z': 9, 'chi2z': 10}
        else:
            self.ParNums = {'Mc': 0, 'eta': 1, 'dL': 2, 'theta': 3, 'phi': 4, 'iota': 5, 'psi': 6, 'tcoal': 7,
                            'Phicoal': 8, 'chiS': 9, 'chiA': 10}
        if is_tidal:
            self.ParNums['LambdaTilde'] = 11
            self.ParNums['deltaLambda'] = 12
        if is_eccentric:   # gwfast/waveforms.py:110-123
            self.ParNums['ecc'] = 13 if is_tidal else 11

    @property
    def params(self):
        """Names of the Fisher parameters in order (the rows of the event array)."""
        return (PARAMS_TIDAL if self.is_tidal else PARAMS) + (('ecc',) if self.is_eccentric else ())

    def fcut(self, **kwargs):
        """Cut frequency in Hz (gwfast/waveforms.py:190-199)."""
        return self.fcutPar / (np.asarray(kwargs['Mc']) / (np.asarray(kwargs['eta']) ** (3. / 5.)))

    def gpu_desc(self):
        return _lib.WfDesc(_lib.MODEL_IDS[type(self).__name__], 0, float(self.fcutPar))

    def _device_only(self, *a, **k):
        raise NotImplementedError('%s is evaluated inside the fused GPU kernels; use GWSignal / DetNet'
                                  % type(self).__name__)

    Phi = Ampl = hphc = _device_only


class TaylorF2_RestrictedPN(WaveFormModel):
    """gwfast/waveforms.py:697-953 (fcut: twice the Schwarzschild ISCO by default, or of the Kerr
    remnant with which_ISCO='Kerr'). is_tidal adds the 5PN and 6PN tidal phase terms and the parameters
    LambdaTilde, deltaLambda (with use_QuadMonTid also the spin-induced quadrupole moments);
    is_eccentric adds the low-eccentricity phase to 3PN and the parameter ecc, referenced at fRef_ecc
    (None: the lowest grid frequency). The tidal and eccentric forms run on the FP64 path only."""

    def __init__(self, fHigh=None, is_tidal=False, use_3p5PN_SpinHO=False, phiref_vlso=False, is_eccentric=False,
                 fRef_ecc=None, which_ISCO='Schw', use_QuadMonTid=False, **kwargs):
        if fHigh is None:
            fHigh = 1. / (6. * np.pi * np.sqrt(6.) * glob.GMsun_over_c3)
        if which_ISCO not in ('Schw', 'Kerr'):
            raise ValueError("which_ISCO must be 'Schw' or 'Kerr'")
        self.use_3p5PN_SpinHO = use_3p5PN_SpinHO
        self.phiref_vlso = phiref_vlso
        self.fRef_ecc = fRef_ecc
        self.which_ISCO = which_ISCO
        self.use_QuadMonTid = use_QuadMonTid
        super().__init__('BNS' if is_tidal else 'BBH', fHigh, is_tidal=is_tidal, is_eccentric=is_eccentric,
                         is_holomorphic=True, **kwargs)

    def fcut(self, **kwargs):
        """Cut frequency in Hz (gwfast/waveforms.py:903-951)."""
        Mc, eta = np.asarray(kwargs['Mc'], dtype=np.float64), np.asarray(kwargs['eta'], dtype=np.float64)
        if self.which_ISCO == 'Schw':
            return self.fcutPar / (Mc / (eta ** (3. / 5.)))
        chi1, chi2 = np.asarray(kwargs['chi1z'], dtype=np.float64), np.asarray(kwargs['chi2z'], dtype=np.float64)
        eta2 = eta * eta
        Mtot = Mc / eta ** (3. / 5.)
        seta = np.sqrt(np.where(eta < 0.25, 1.0 - 4.0 * eta, 0.))
        m1, m2 = 0.5 * (1.0 + seta), 0.5 * (1.0 - seta)
        s = (m1 * m1 * chi1 + m2 * m2 * chi2) / (m1 * m1 + m2 * m2)
        atot = (chi1 + chi2 * (m2 / m1) ** 2) / (1. + m2 / m1) ** 2
        aeff = atot + 0.41616 * eta * (chi1 + chi2)

        def r_isco(chi):
            z1 = 1.0 + np.cbrt(1.0 - chi * chi) * (np.cbrt(1.0 + chi) + np.cbrt(1.0 - chi))
            z2 = np.sqrt(3.0 * chi * chi + z1 * z1)
            r = np.sqrt((3.0 - z1) * (3.0 + z1 + 2.0 * z2))
            return np.where(chi > 0., 3.0 + z2 - r, 3.0 + z2 + r)

        r0 = r_isco(aeff)
        ens = eta * (0.055974469826360077 + 0.5809510763115132 * eta - 0.9606726679372312 * eta2
                     + 3.352411249771192 * eta2 * eta)
        erad = (ens * (1. + (-0.0030302335878845507 - 2.0066110851351073 * eta + 7.7050567802399215 * eta2) * s)
                / (1. + (-0.6714403054720589 - 1.4756929437702908 * eta + 7.304676214885011 * eta2) * s))
        L = 2. / (3. * np.sqrt(3.)) * (1. + 2. * np.sqrt(3. * r0 - 2.))
        E = np.sqrt(1. - 2. / (3. * r0))
        chif = (atot + eta * (L - 2. * atot * (E - 1.)) + (-3.821158961 - 1.2019 * aeff - 1.20764 * aeff ** 2) * eta2
                + (3.79245 + 1.18385 * aeff + 4.90494 * aeff ** 2) * eta2 * eta)
        rf = r_isco(chif)
        return 1. / (rf ** 1.5 + chif) / (np.pi * Mtot * (1. - erad) * glob.GMsun_over_c3)

    def gpu_desc(self):
        if self.is_eccentric:
            model = _lib.MODEL_TF2_TIDAL_ECC if self.is_tidal else _lib.MODEL_TF2_ECC
        else:
            model = _lib.MODEL_TF2_TIDAL if self.is_tidal else _lib.MODEL_IDS['TaylorF2_RestrictedPN']
        flags = ((_lib.TF2_PHIREF_VLSO if self.phiref_vlso else 0) | (_lib.TF2_KERR_ISCO if self.which_ISCO == 'Kerr' else 0)
                 | (_lib.TF2_QUADMON_TIDAL if (self.use_QuadMonTid and self.is_tidal) else 0))
        fre = float(self.fRef_ecc) if (self.is_eccentric and self.fRef_ecc is not None) else 0.
        return _lib.WfDesc(model, int(self.use_3p5PN_SpinHO), float(self.fcutPar), flags, 0, fre)


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


class IMRPhenomNSBH(WaveFormModel):
    """gwfast/waveforms.py:2752-3374: object 1 is the black hole, object 2 the neutron star (only Lambda2
    enters); IMRPhenomD phase with the NSBH remnant and the NRTidalv2 tidal phase, IMRPhenomC-based
    amplitude with the merger-type windows of arXiv:1509.00512 (13 parameters, FP64 path only). Its
    xi_tide table is built on the GPU, as gwfast tabulates it when the h5 file is absent."""

    def __init__(self, fRef=None, verbose=True, **kwargs):
        if fRef is not None:
            raise NotImplementedError('a fixed fRef is not implemented on the GPU path')
        self.PHI_fJoin_INS = 0.018
        self.verbose = verbose
        self.fRef = fRef
        super().__init__('NSBH', 0.2, is_tidal=True, **kwargs)

    def fcut(self, **kwargs):
        """gwfast/waveforms.py:3274-3284."""
        return self.fcutPar / (np.asarray(kwargs['Mc']) * glob.GMsun_over_c3 / (np.asarray(kwargs['eta']) ** (3. / 5.)))
