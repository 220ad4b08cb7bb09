"""float64 CPU restatement of the gwfast Fisher-forecast hot path (test infrastructure).

This module is the oracle: ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` use it as the checker.  Nothing in the
``gwfast_gb300`` package imports it.

Layout: every per-event parameter is a torch float64 tensor of shape (N, 1);
frequency grids have shape (N, R).  Jacobians are taken with forward-mode AD
(``torch.func.jvp``), one tangent direction per parameter, over all events at
once (events are independent).  gwfast itself uses reverse mode
(``gwfast/signal.py:1178-1189``) plus closed-form extrinsic derivatives
(``gwfast/signal.py:1303-1584``); both are exact derivatives of the same strain,
so they agree to rounding.  The golden fixtures under ``tests/golden`` hold
gwfast's own closed-form derivatives and pin that claim.

Parameter order of the Fisher matrix (``gwfast/waveforms.py:78``, ``:125-129``):
Mc, eta, dL, theta, phi, iota, psi, tcoal, Phicoal, chi1z, chi2z.
"""
import math
import os

import numpy as np
import torch

DT = torch.float64
PI = math.pi

# ---------------------------------------------------------------- constants
# gwfast/gwfastGlobals.py:38-124
GMSUN_OVER_C3 = 4.925491025543575903411922162094833998e-6   # s
GMSUN_OVER_C2 = 1.476625061404649406193430731479084713e3    # m
U_GPC = 3.085677581491367278913937957796471611e25           # m
GMSUN_OVER_C2_GPC = GMSUN_OVER_C2 / U_GPC
R_EARTH_KM = 6371.00
C_KMS = 2.99792458e5
C_GPC = C_KMS / 3.0856778570831e+22
EULER_GAMMA = 0.5772156649015329
DAY_S = 3600. * 24.

PARAMS = ('Mc', 'eta', 'dL', 'theta', 'phi', 'iota', 'psi', 'tcoal', 'Phicoal', 'chi1z', 'chi2z')
PARAMS_TIDAL = PARAMS + ('LambdaTilde', 'deltaLambda')   # gwfast/waveforms.py:106-109
NPAR = 11
TC_INDEX = 7

# gwfast/gwfastGlobals.py:143-214 (lat, long, xax in degrees; shape)
DETECTORS = {
    'L1': (30.563, -90.774, 242.71636956358617, 'L'),
    'H1': (46.455, -119.408, 170.99924234706103, 'L'),
    'Virgo': (43.631, 10.504, 115.56756342034298, 'L'),
    'KAGRA': (36.412, 137.306, 15.396, 'L'),
    'LIGOI': (19.613, 77.031, 287.384, 'L'),
    'ETS': (40. + 31. / 60., 9. + 25. / 60., 0., 'T'),
    'ETMR': (50. + 43. / 60. + 23. / 3600., 5. + 55. / 60. + 14. / 3600., 0., 'T'),
    'CE1Id': (43.827, -112.825, -45., 'L'),
    'CE2NM': (33.160, -106.480, -105., 'L'),
    'CE2NSW': (-34., 145., 0., 'L'),
}


def _T(x):
    return torch.as_tensor(x, dtype=DT)


def _seta(eta):
    # sqrt(1-4 eta) guarded at equal mass: gwfast/waveforms.py:759
    return torch.sqrt(torch.where(eta < 0.25, 1.0 - 4.0 * eta, torch.zeros_like(eta)))


# ---------------------------------------------------------------- PN phase coefficients
def pn_coeffs(eta, chi1, chi2, spin_ho=False, drop_3pn_ss=False, dq1=0., dq2=0.):
    """TaylorF2 phase coefficients (gwfast/waveforms.py:784-812).

    ``drop_3pn_ss`` removes the 3PN spin-spin terms, as IMRPhenomD does
    (gwfast/waveforms.py:1077). ``dq1``, ``dq2``: spin-induced quadrupole moments minus one, which
    IMRPhenomD_NRTidalv2 keeps in its 2PN and 3PN spin-spin terms (gwfast/waveforms.py:1461-1467).
    """
    seta = _seta(eta)
    m1 = 0.5 * (1.0 + seta)
    m2 = 0.5 * (1.0 - seta)
    chis = 0.5 * (chi1 + chi2)
    chia = 0.5 * (chi1 - chi2)
    eta2 = eta * eta
    c = {}
    c['two'] = 3715. / 756. + 55. * eta / 9.
    c['three'] = -16. * PI + 113. * seta * chia / 3. + (113. / 3. - 76. * eta / 3.) * chis
    m1s, m2s = m1 * m1 * chi1 * chi1, m2 * m2 * chi2 * chi2
    q1, q2 = 1. + dq1, 1. + dq2
    c['four'] = (5. * (3058.673 / 7.056 + 5429. / 7. * eta + 617. * eta2) / 72.
                 + (247. / 4.8 - 721. / 4.8) * eta * chi1 * chi2
                 + (-720. / 9.6 * q1 + 1. / 9.6) * m1s + (-720. / 9.6 * q2 + 1. / 9.6) * m2s
                 + (240. / 9.6 * q1 - 7. / 9.6) * m1s + (240. / 9.6 * q2 - 7. / 9.6) * m2s)
    t5 = ((732985. / 2268. - 24260. * eta / 81. - 340. * eta2 / 9.) * chis
          + (732985. / 2268. + 140. * eta / 9.) * seta * chia)
    c['five'] = 38645. * PI / 756. - 65. * PI * eta / 9. - t5
    c['five_log'] = 3. * c['five']
    six = (11583.231236531 / 4.694215680 - 640. / 3. * PI * PI - 684.8 / 2.1 * EULER_GAMMA
           + eta * (-15737.765635 / 3.048192 + 225.5 / 1.2 * PI * PI)
           + eta2 * 76.055 / 1.728 - eta2 * eta * 127.825 / 1.296 - math.log(4.) * 684.8 / 2.1
           + PI * chi1 * m1 * (1490. / 3. + 260. * m1) + PI * chi2 * m2 * (1490. / 3. + 260. * m2))
    # the quadrupole excess of the 3PN spin-spin terms (:806, :1464-1467; zero for black holes)
    six = six + ((4703.5 / 8.4 + 2935. / 6. * m1 - 120. * m1 * m1) * m1s * dq1
                 + (4703.5 / 8.4 + 2935. / 6. * m2 - 120. * m2 * m2) * m2s * dq2)
    if not drop_3pn_ss:
        def ss(m):
            return (4703.5 / 8.4 + 2935. / 6. * m - 120. * m * m) + (-4108.25 / 6.72 - 108.5 / 1.2 * m + 125.5 / 3.6 * m * m)
        six = six + (326.75 / 1.12 + 557.5 / 1.8 * eta) * eta * chi1 * chi2 + ss(m1) * m1s + ss(m2) * m2s
    c['six'] = six
    c['six_log'] = -6848. / 21.
    sev = (77096675. * PI / 254016. + 378515. * PI * eta / 1512. - 74045. * PI * eta2 / 756.)
    if spin_ho:
        sev = sev + ((-25150083775. / 3048192. + 10566655595. * eta / 762048. - 1042165. * eta2 / 3024.
                      + 5345. * eta2 * eta / 36. + (14585. / 8. - 7270. * eta + 80. * eta2) * chia * chia) * chis
                     + (14585. / 24. - 475. * eta / 6. + 100. * eta2 / 3.) * chis ** 3
                     + seta * ((-25150083775. / 3048192. + 26804935. * eta / 6048. - 1985. * eta2 / 48.) * chia
                               + (14585. / 24. - 2380. * eta) * chia ** 3 + (14585. / 8. - 215. * eta / 2.) * chia * chis * chis))
    else:
        sev = sev + ((-25150083775. / 3048192. + 10566655595. * eta / 762048. - 1042165. * eta2 / 3024.
                      + 5345. * eta2 * eta / 36.) * chis
                     + seta * (-25150083775. / 3048192. + 26804935. * eta / 6048. - 1985. * eta2 / 48.) * chia)
    c['seven'] = sev
    return c


# ---------------------------------------------------------------- TaylorF2
def tf2_fcut(Mc, eta):
    """Twice the Schwarzschild ISCO frequency: gwfast/waveforms.py:730-731, :918-920."""
    fhigh = 1. / (6. * PI * math.sqrt(6.) * GMSUN_OVER_C3)
    return fhigh / (Mc / eta ** (3. / 5.))


def _r_isco(chi):
    z1 = 1.0 + (1.0 - chi * chi) ** (1. / 3.) * ((1.0 + chi) ** (1. / 3.) + (1.0 - chi) ** (1. / 3.))
    z2 = torch.sqrt(3.0 * chi * chi + z1 * z1)
    r = torch.sqrt((3.0 - z1) * (3.0 + z1 + 2.0 * z2))
    return torch.where(chi > 0., 3.0 + z2 - r, 3.0 + z2 + r)


def tf2_fcut_kerr(Mc, eta, chi1, chi2):
    """Twice the ISCO frequency of the Kerr remnant (which_ISCO='Kerr'): gwfast/waveforms.py:921-951."""
    eta2 = eta * eta
    Mtot = Mc / eta ** (3. / 5.)
    seta = _seta(eta)
    m1, m2 = 0.5 * (1. + seta), 0.5 * (1. - seta)
    s = (m1 * m1 * chi1 + m2 * m2 * chi2) / (m1 * m1 + m2 * m2)
    atot = (chi1 + chi2 * (m2 / m1) ** 2) / (1. + m2 / m1) ** 2
    aeff = atot + 0.41616 * eta * (chi1 + chi2)
    r0 = _r_isco(aeff)
    ens = eta * (0.055974469826360077 + 0.5809510763115132 * eta - 0.9606726679372312 * eta2 + 3.352411249771192 * eta2 * eta)
    erad = (ens * (1. + (-0.0030302335878845507 - 2.0066110851351073 * eta + 7.7050567802399215 * eta2) * s)
            / (1. + (-0.6714403054720589 - 1.4756929437702908 * eta + 7.304676214885011 * eta2) * s))
    L = 2. / (3. * math.sqrt(3.)) * (1. + 2. * torch.sqrt(3. * r0 - 2.))
    E = torch.sqrt(1. - 2. / (3. * r0))
    chif = (atot + eta * (L - 2. * atot * (E - 1.)) + (-3.821158961 - 1.2019 * aeff - 1.20764 * aeff ** 2) * eta2
            + (3.79245 + 1.18385 * aeff + 4.90494 * aeff ** 2) * eta2 * eta)
    rf = _r_isco(chif)
    return 1. / (rf ** 1.5 + chif) / (PI * Mtot * (1. - erad) * GMSUN_OVER_C3)


# eccentric TaylorF2 coefficients (arXiv:1605.00304, as gwfast/waveforms.py:826-843 writes them):
# name -> function of eta
def _ecc_coeffs(eta):
    e2, e3 = eta * eta, eta * eta * eta
    pi2, l2, l3, g = PI * PI, math.log(2.), math.log(3.), EULER_GAMMA
    return {
        'twoV': 29.9076223 / 8.1976608 + 18.766963 / 2.927736 * eta,
        'twoV0': 2.833 / 1.008 - 19.7 / 3.6 * eta,
        'threeV': -28.19123 / 2.82600 * PI,
        'threeV0': 37.7 / 7.2 * PI,
        'fourV4': 16.237683263 / 3.330429696 + 241.33060753 / 9.71375328 * eta + 156.2608261 / 6.9383952 * e2,
        'fourV2V02': 84.7282939759 / 8.2632420864 - 7.18901219 / 3.68894736 * eta - 36.97091711 / 1.05398496 * e2,
        'fourV04': -1.193251 / 3.048192 - 66.317 / 9.072 * eta + 18.155 / 1.296 * e2,
        'fiveV5': -28.31492681 / 1.18395270 * PI - 115.52066831 / 2.70617760 * PI * eta,
        'fiveV3V02': -79.86575459 / 2.84860800 * PI + 55.5367231 / 1.0173600 * PI * eta,
        'fiveV2V03': 112.751736071 / 5.902315776 * PI + 70.75145051 / 2.10796992 * PI * eta,
        'fiveV05': 76.4881 / 9.0720 * PI - 94.9457 / 2.2680 * PI * eta,
        'sixV6': (-436.03153867072577087 / 1.32658535116800000 + 53.6803271 / 1.9782000 * g + 157.22503703 / 3.25555200 * pi2
                  + (2991.72861614477 / 6.89135247360 - 15.075413 / 1.446912 * pi2) * eta + 345.5209264991 / 4.1019955200 * e2
                  + 506.12671711 / 8.78999040 * e3 + 384.3505163 / 5.9346000 * l2 - 112.1397129 / 1.7584000 * l3),
        'sixV4V02': (46.001356684079 / 3.357073133568 + 253.471410141755 / 5.874877983744 * eta
                     - 169.3852244423 / 2.3313007872 * e2 - 307.833827417 / 2.497822272 * e3),
        'sixV3V03': -106.2809371 / 2.0347200 * pi2,
        'sixV2V04': (-3.56873002170973 / 2.49880440692736 - 260.399751935005 / 8.924301453312 * eta
                     + 15.0484695827 / 3.5413894656 * e2 + 340.714213265 / 3.794345856 * e3),
        'sixV06': (265.31900578691 / 1.68991764480 - 33.17 / 1.26 * g + 12.2833 / 1.0368 * pi2
                   + (91.55185261 / 5.48674560 - 3.977 / 1.152 * pi2) * eta - 5.732473 / 1.306368 * e2
                   - 30.90307 / 1.39968 * e3 + 87.419 / 1.890 * l2 - 260.01 / 5.60 * l3),
    }


def tf2_ecc_series(v, v0, eta, ecc):
    """phi_Ecc of gwfast/waveforms.py:824-845: -2355/1462 e0^2 (v0/v)^(19/3) times the 3PN series in v, v0."""
    k = _ecc_coeffs(eta)
    pre = -2.355 / 1.462 * ecc * ecc * (v0 / v) ** (19. / 3.)
    ser = (1. + (k['twoV'] * v * v + k['twoV0'] * v0 * v0) + (k['threeV'] * v ** 3 + k['threeV0'] * v0 ** 3)
           + (k['fourV4'] * v ** 4 + k['fourV2V02'] * v * v * v0 * v0 + k['fourV04'] * v0 ** 4)
           + (k['fiveV5'] * v ** 5 + k['fiveV3V02'] * v ** 3 * v0 ** 2 + k['fiveV2V03'] * v ** 2 * v0 ** 3
              + k['fiveV05'] * v0 ** 5)
           + ((k['sixV6'] + 53.6803271 / 3.9564000 * torch.log(16. * v * v)) * v ** 6 + k['sixV4V02'] * v ** 4 * v0 ** 2
              + k['sixV3V03'] * v ** 3 * v0 ** 3 + k['sixV2V04'] * v ** 2 * v0 ** 4
              + (k['sixV06'] - 33.17 / 2.52 * torch.log(16. * v0 * v0)) * v0 ** 6))
    return pre * ser


def tf2_phase(f, Mc, eta, chi1, chi2, spin_ho=False, lam_t=None, del_lam=None, ecc=None, fref_ecc=None, vlso=False,
              quadmon=False):
    """gwfast/waveforms.py:743-862 (fRef at v = 0); with lam_t/del_lam the tidal terms
    (-39/2 LambdaTilde) v^10 + (-3115/64 LambdaTilde + 6595/364 sqrt(1-4 eta) deltaLambda) v^12 of
    :849-855 join the series (``quadmon``: with the spin-induced quadrupole moments of :780-788); with
    ``ecc`` the eccentric terms of :814-845, referenced at fref_ecc or the lowest frequency of each
    row of f; ``vlso``: phiref_vlso (:796-798)."""
    Mtot_s = Mc * GMSUN_OVER_C3 / eta ** (3. / 5.)
    v = (PI * Mtot_s * f) ** (1. / 3.)
    dq1 = dq2 = 0.
    if quadmon and lam_t is not None:
        l1, l2 = lam12_from_lamt_dellam(lam_t, del_lam, eta)
        dq1, dq2 = quad_mon(l1) - 1., quad_mon(l2) - 1.
    c = pn_coeffs(eta, chi1, chi2, spin_ho=spin_ho, dq1=dq1, dq2=dq2)
    five = c['five'] * (1. - 3. * math.log(1. / math.sqrt(6.))) if vlso else c['five']
    lv = torch.log(v)
    ser = (1. + c['two'] * v * v + c['three'] * v ** 3 + c['four'] * v ** 4
           + (five + c['five_log'] * lv) * v ** 5 + (c['six'] + c['six_log'] * lv) * v ** 6 + c['seven'] * v ** 7)
    if lam_t is not None:
        seta = torch.sqrt(torch.where(eta < 0.25, 1.0 - 4.0 * eta, torch.zeros_like(eta)))
        ser = ser + (-0.5 * 39. * lam_t) * v ** 10 + (-3115. / 64. * lam_t + 6595. / 364. * seta * del_lam) * v ** 12
    if ecc is not None:
        v0 = torch.amin(v, dim=-1, keepdim=True) if fref_ecc is None else (PI * Mtot_s * fref_ecc) ** (1. / 3.)
        ser = ser + tf2_ecc_series(v, v0, eta, ecc)
    return 3. / (128. * eta) * ser / v ** 5 + (0. if vlso else PI) - PI * 0.25


def tf2_ampl(f, Mc, dL):
    """gwfast/waveforms.py:864-876."""
    return (math.sqrt(5. / 24.) * PI ** (-2. / 3.) * C_GPC / dL
            * (GMSUN_OVER_C3 * Mc) ** (5. / 6.) * f ** (-7. / 6.))


def tau_star(f, Mc, eta):
    """3.5PN time to coalescence, shared by the three models: gwfast/waveforms.py:878-901."""
    Mtot_s = Mc * GMSUN_OVER_C3 / eta ** (3. / 5.)
    v = (PI * Mtot_s * f) ** (1. / 3.)
    eta2 = eta * eta
    pre = 5. / 256 * Mtot_s / (eta * v ** 8)
    t05 = (1. + (743. / 252. + 11. / 3. * eta) * v * v - 32. / 5. * PI * v ** 3
           + (3058673. / 508032. + 5429. / 504. * eta + 617. / 72. * eta2) * v ** 4
           - (7729. / 252. - 13. / 3. * eta) * PI * v ** 5)
    t6 = (-10052469856691. / 23471078400. + 128. / 3. * PI * PI + 6848. / 105. * EULER_GAMMA
          + (3147553127. / 3048192. - 451. / 12. * PI * PI) * eta - 15211. / 1728. * eta2
          + 25565. / 1296. * eta2 * eta + 3424. / 105. * torch.log(16. * v * v)) * v ** 6
    t7 = (-15419335. / 127008. - 75703. / 756. * eta + 14809. / 378. * eta2) * PI * v ** 7
    return pre * (t05 + t6 + t7)


# ---------------------------------------------------------------- IMRPhenomD fits
# 11-coefficient fits in (eta, xi): gwfast/waveforms.py:1039-1056, :1132-1133, :1189-1197, :1223
def _fit(c, eta, xi):
    e2 = eta * eta
    return c[0] + c[1] * eta + (c[2] + c[3] * eta + c[4] * e2 + (c[5] + c[6] * eta + c[7] * e2) * xi
                                + (c[8] + c[9] * eta + c[10] * e2) * xi * xi) * xi


FITS = {
    'sigma1': (2096.551999295543, 1463.7493168261553, 1312.5493286098522, 18307.330017082117, -43534.1440746107, -833.2889543511114, 32047.31997183187, -108609.45037520859, 452.25136398112204, 8353.439546391714, -44531.3250037322),
    'sigma2': (-10114.056472621156, -44631.01109458185, -6541.308761668722, -266959.23419307504, 686328.3229317984, 3405.6372187679685, -437507.7208209015, 1.6318171307344697e6, -7462.648563007646, -114585.25177153319, 674402.4689098676),
    'sigma3': (22933.658273436497, 230960.00814979506, 14961.083974183695, 1.1940181342318142e6, -3.1042239693052764e6, -3038.166617199259, 1.8720322849093592e6, -7.309145012085539e6, 42738.22871475411, 467502.018616601, -3.064853498512499e6),
    'sigma4': (-14621.71522218357, -377812.8579387104, -9608.682631509726, -1.7108925257214056e6, 4.332924601416521e6, -22366.683262266528, -2.5019716386377467e6, 1.0274495902259542e7, -85360.30079034246, -570025.3441737515, 4.396844346849777e6),
    'beta1': (97.89747327985583, -42.659730877489224, 153.48421037904913, -1417.0620760768954, 2752.8614143665027, 138.7406469558649, -1433.6585075135881, 2857.7418952430758, 41.025109467376126, -423.680737974639, 850.3594335657173),
    'beta2': (-3.282701958759534, -9.051384468245866, -12.415449742258042, 55.4716447709787, -106.05109938966335, -11.953044553690658, 76.80704618365418, -155.33172948098394, -3.4129261592393263, 25.572377569952536, -54.408036707740465),
    'beta3': (-0.000025156429818799565, 0.000019750256942201327, -0.000018370671469295915, 0.000021886317041311973, 0.00008250240316860033, 7.157371250566708e-6, -0.000055780000112270685, 0.00019142082884072178, 5.447166261464217e-6, -0.00003220610095021982, 0.00007974016714984341),
    'alpha1': (43.31514709695348, 638.6332679188081, -32.85768747216059, 2415.8938269370315, -5766.875169379177, -61.85459307173841, 2953.967762459948, -8986.29057591497, -21.571435779762044, 981.2158224673428, -3239.5664895930286),
    'alpha2': (-0.07020209449091723, -0.16269798450687084, -0.1872514685185499, 1.138313650449945, -2.8334196304430046, -0.17137955686840617, 1.7197549338119527, -4.539717148261272, -0.049983437357548705, 0.6062072055948309, -1.682769616644546),
    'alpha3': (9.5988072383479, -397.05438595557433, 16.202126189517813, -1574.8286986717037, 3600.3410843831093, 27.092429659075467, -1786.482357315139, 5152.919378666511, 11.175710130033895, -577.7999423177481, 1808.730762932043),
    'alpha4': (-0.02989487384493607, 1.4022106448583738, -0.07356049468633846, 0.8337006542278661, 0.2240008282397391, -0.055202870001177226, 0.5667186343606578, 0.7186931973380503, -0.015507437354325743, 0.15750322779277187, 0.21076815715176228),
    'alpha5': (0.9974408278363099, -0.007884449714907203, -0.059046901195591035, 1.3958712396764088, -4.516631601676276, -0.05585343136869692, 1.7516580039343603, -5.990208965347804, -0.017945336522161195, 0.5965097794825992, -2.0608879367971804),
    'gamma1': (0.006927402739328343, 0.03020474290328911, 0.006308024337706171, -0.12074130661131138, 0.26271598905781324, 0.0034151773647198794, -0.10779338611188374, 0.27098966966891747, 0.0007374185938559283, -0.02749621038376281, 0.0733150789135702),
    'gamma2': (1.010344404799477, 0.0008993122007234548, 0.283949116804459, -4.049752962958005, 13.207828172665366, 0.10396278486805426, -7.025059158961947, 24.784892370130475, 0.03093202475605892, -2.6924023896851663, 9.609374464684983),
    'gamma3': (1.3081615607036106, -0.005537729694807678, -0.06782917938621007, -0.6689834970767117, 3.403147966134083, -0.05296577374411866, -0.9923793203111362, 4.820681208409587, -0.006134139870393713, -0.38429253308696365, 1.7561754421985984),
    'rho1': (3931.8979897196696, -17395.758706812805, 3132.375545898835, 343965.86092361377, -1.2162565819981997e6, -70698.00600428853, 1.383907177859705e6, -3.9662761890979446e6, -60017.52423652596, 803515.1181825735, -2.091710365941658e6),
    'rho2': (-40105.47653771657, 112253.0169706701, 23561.696065836168, -3.476180699403351e6, 1.137593670849482e7, 754313.1127166454, -1.308476044625268e7, 3.6444584853928134e7, 596226.612472288, -7.4277901143564405e6, 1.8928977514040343e7),
    'rho3': (83208.35471266537, -191237.7264145924, -210916.2454782992, 8.71797508352568e6, -2.6914942420669552e7, -1.9889806527362722e6, 3.0888029960154563e7, -8.390870279256162e7, -1.4535031953446497e6, 1.7063528990822166e7, -4.2748659731120914e7),
    'v2': (0.8149838730507785, 2.5747553517454658, 1.1610198035496786, -2.3627771785551537, 6.771038707057573, 0.7570782938606834, -2.7256896890432474, 7.1140380397149965, 0.1766934149293479, -0.7978690983168183, 2.1162391502005153),
}

PHI_FJOIN_INS = 0.018   # gwfast/waveforms.py:980
AMP_FJOIN_INS = 0.014   # gwfast/waveforms.py:978
MF_CUT = 0.2            # gwfast/waveforms.py:982


def phd_fcut(Mc, eta):
    """gwfast/waveforms.py:1324-1333."""
    return MF_CUT / (Mc * GMSUN_OVER_C3 / eta ** (3. / 5.))


def final_spin(eta, chi1, chi2):
    """gwfast/waveforms.py:1256-1276."""
    seta = _seta(eta)
    m1, m2 = 0.5 * (1. + seta), 0.5 * (1. - seta)
    s = m1 * m1 * chi1 + m2 * m2 * chi2
    af1 = eta * (3.4641016151377544 - 4.399247300629289 * eta + 9.397292189321194 * eta * eta - 13.180949901606242 * eta ** 3)
    af2 = eta * (s * ((1.0 / eta - 0.0850917821418767 - 5.837029316602263 * eta) + (0.1014665242971878 - 2.0967746996832157 * eta) * s))
    af3 = eta * (s * ((-1.3546806617824356 + 4.108962025369336 * eta) * s * s + (-0.8676969352555539 + 2.064046835273906 * eta) * s ** 3))
    return af1 + af2 + af3


def radiated_energy(eta, chi1, chi2):
    """gwfast/waveforms.py:1278-1297."""
    seta = _seta(eta)
    m1, m2 = 0.5 * (1. + seta), 0.5 * (1. - seta)
    s = (m1 * m1 * chi1 + m2 * m2 * chi2) / (m1 * m1 + m2 * m2)
    ens = eta * (0.055974469826360077 + 0.5809510763115132 * eta - 0.9606726679372312 * eta * eta + 3.352411249771192 * eta ** 3)
    return (ens * (1. + (-0.0030302335878845507 - 2.0066110851351073 * eta + 7.7050567802399215 * eta * eta) * s)
            / (1. + (-0.6714403054720589 - 1.4756929437702908 * eta + 7.304676214885011 * eta * eta) * s))


_QNM = None


def qnm_table():
    global _QNM
    if _QNM is None:
        here = os.path.dirname(os.path.abspath(__file__))
        tab = np.loadtxt(os.path.join(here, '..', 'gwfast_gb300', 'data', 'qnm_220.txt'))
        _QNM = torch.as_tensor(tab, dtype=DT)
    return _QNM


def interp(x, xp, fp):
    """Piecewise-linear interpolation whose derivative in x is the segment slope (jnp.interp semantics)."""
    idx = torch.searchsorted(xp, x.detach().contiguous(), right=True).clamp(1, xp.numel() - 1)
    x0, x1 = xp[idx - 1], xp[idx]
    y0, y1 = fp[idx - 1], fp[idx]
    return y0 + (x - x0) * ((y1 - y0) / (x1 - x0))


def _ins_phase(Mf, c, A, sig, eta):
    """Inspiral phase of IMRPhenomD: TF2 series in (pi Mf) plus the sigma terms (gwfast/waveforms.py:1079-1094, :1145)."""
    x = PI * Mf
    lx = torch.log(x) / 3.
    x13 = x ** (1. / 3.)
    tf2 = (x ** (-5. / 3.) + c['two'] / x + c['three'] * x ** (-2. / 3.) + c['four'] * x ** (-1. / 3.)
           + c['five'] + c['five_log'] * lx + (c['six'] + c['six_log'] * lx) * x13 + c['seven'] * x13 * x13)
    return A * tf2 + (sig[0] * Mf + 0.75 * sig[1] * Mf ** (4. / 3.) + 0.6 * sig[2] * Mf ** (5. / 3.) + 0.5 * sig[3] * Mf * Mf) / eta


def _ins_phase_deriv(Mf, c, A, sig, eta):
    """d/dMf of _ins_phase (the reference writes this out as DPhiIns, gwfast/waveforms.py:1108-1109)."""
    x = PI * Mf
    lx = torch.log(x) / 3.
    x13 = x ** (1. / 3.)
    d = (-5. / 3. * x ** (-8. / 3.) - c['two'] / (x * x) - 2. / 3. * c['three'] * x ** (-5. / 3.)
         - 1. / 3. * c['four'] * x ** (-4. / 3.) + c['five_log'] / (3. * x)
         + c['six_log'] / (3. * x) * x13 + (c['six'] + c['six_log'] * lx) / 3. * x13 / x
         + 2. / 3. * c['seven'] * x13 * x13 / x) * PI
    return A * d + (sig[0] + sig[1] * Mf ** (1. / 3.) + sig[2] * Mf ** (2. / 3.) + sig[3] * Mf) / eta


def _int_phase_raw(Mf, b, eta):
    return (b[0] * Mf - b[2] / (3. * Mf ** 3) + b[1] * torch.log(Mf)) / eta


def _int_phase_raw_d(Mf, b, eta):
    return (b[0] + b[2] / Mf ** 4 + b[1] / Mf) / eta


def _mrd_phase_raw(Mf, a, fring, fdamp, eta, rho=1., tau=1.):
    return (-a[1] / Mf + 4. / 3. * a[2] * Mf ** 0.75 + a[0] * Mf
            + a[3] * rho * torch.atan((Mf - a[4] * fring) / (fdamp * rho * tau))) / eta


def _mrd_phase_raw_d(Mf, a, fring, fdamp, eta, rho=1., tau=1.):
    u = (Mf - a[4] * fring) / (fdamp * rho * tau)
    return (a[0] + a[1] / (Mf * Mf) + a[2] / Mf ** 0.25 + a[3] / (fdamp * tau * (1. + u * u))) / eta


def _phenom_core(Mc, eta, chi1, chi2, fring, fdamp, dq1=0., dq2=0.):
    """Per-event IMRPhenomD phase/amplitude coefficients common to PhenomD, PhenomHM and
    PhenomD_NRTidalv2 (whose spin-induced quadrupole moments enter through ``dq1``, ``dq2``)."""
    seta = _seta(eta)
    chis, chia = 0.5 * (chi1 + chi2), 0.5 * (chi1 - chi2)
    chiPN = chis * (1.0 - eta * 76.0 / 113.0) + seta * chia
    xi = -1.0 + chiPN
    k = {nm: _fit(FITS[nm], eta, xi) for nm in FITS}
    k['M'] = Mc / eta ** (3. / 5.)
    k['eta'] = eta
    k['seta'] = seta
    k['fring'], k['fdamp'] = fring, fdamp
    c = pn_coeffs(eta, chi1, chi2, drop_3pn_ss=True, dq1=dq1, dq2=dq2)
    k['c'] = c
    k['A'] = 3. / (128. * eta) * PI ** (-5. / 3.)
    # normalise the TF2 series so that x**(-5/3) carries coefficient 1 (A absorbs it)
    k['c'] = {kk: c[kk] for kk in c}
    sig = (k['sigma1'], k['sigma2'], k['sigma3'], k['sigma4'])
    bet = (k['beta1'], k['beta2'], k['beta3'])
    alp = (k['alpha1'], k['alpha2'], k['alpha3'], k['alpha4'], k['alpha5'])
    k['sig'], k['bet'], k['alp'] = sig, bet, alp
    fj = _T(PHI_FJOIN_INS)
    A = 3. / (128. * eta)
    k['A'] = A
    # C1 join inspiral -> intermediate at Mf = 0.018 (gwfast/waveforms.py:1098-1120)
    k['C2Int'] = _ins_phase_deriv(fj, c, A, sig, eta) - _int_phase_raw_d(fj, bet, eta)
    k['C1Int'] = _ins_phase(fj, c, A, sig, eta) - _int_phase_raw(fj, bet, eta) - k['C2Int'] * fj
    # C1 join intermediate -> merger-ringdown at 0.5 fring (gwfast/waveforms.py:1122-1129)
    fm = 0.5 * fring
    k['fMRDJoin'] = fm
    k['PhiIntTempVal'] = _int_phase_raw(fm, bet, eta) + k['C1Int'] + k['C2Int'] * fm
    k['DPhiIntTempVal'] = k['C2Int'] + _int_phase_raw_d(fm, bet, eta)
    k['C2MRD'] = k['DPhiIntTempVal'] - _mrd_phase_raw_d(fm, alp, fring, fdamp, eta)
    k['C1MRD'] = k['PhiIntTempVal'] - _mrd_phase_raw(fm, alp, fring, fdamp, eta) - k['C2MRD'] * fm
    return k


def _phase_pieces(Mf, k, C1MRD, C2MRD, rho=1., tau=1.):
    """Piecewise IMRPhenomD phase with the Mf < 0.2 cut (gwfast/waveforms.py:1145, :2497-2499)."""
    eta = k['eta']
    ins = _ins_phase(Mf, k['c'], k['A'], k['sig'], eta)
    itm = _int_phase_raw(Mf, k['bet'], eta) + k['C1Int'] + k['C2Int'] * Mf
    mrd = _mrd_phase_raw(Mf, k['alp'], k['fring'], k['fdamp'], eta, rho, tau) + C1MRD + C2MRD * Mf
    zero = torch.zeros_like(Mf + C1MRD)
    return torch.where(Mf < PHI_FJOIN_INS, ins, torch.where(Mf < k['fMRDJoin'], itm, torch.where(Mf < MF_CUT, mrd, zero)))


def _amp_coeffs(k, chi1, chi2):
    """Inspiral amplitude coefficients and the intermediate polynomial (gwfast/waveforms.py:1198-1245)."""
    eta, seta = k['eta'], k['seta']
    sp1 = 1. + seta
    eta2 = eta * eta
    a = {}
    a['23'] = (-969. + 1804. * eta) * PI ** (2. / 3.) / 672.
    a['1'] = (chi1 * (81. * sp1 - 44. * eta) + chi2 * (81. - 81. * seta - 44. * eta)) * PI / 48.
    a['43'] = ((-27312085.0 - 10287648. * chi2 ** 2 - 10287648. * chi1 ** 2 * sp1 + 10287648. * chi2 ** 2 * seta
                + 24. * (-1975055. + 857304. * chi1 ** 2 - 994896. * chi1 * chi2 + 857304. * chi2 ** 2) * eta
                + 35371056 * eta2) * PI ** (4. / 3.)) / 8.128512e6
    a['53'] = (PI ** (5. / 3.) * (chi2 * (-285197. * (-1. + seta) + 4. * (-91902. + 1579. * seta) * eta - 35632. * eta2)
                                   + chi1 * (285197. * sp1 - 4. * (91902. + 1579. * seta) * eta - 35632. * eta2)
                                   + 42840. * (-1.0 + 4. * eta) * PI)) / 32256.
    a['2'] = -(PI ** 2 * (-336. * (-3248849057.0 + 2943675504. * chi1 ** 2 - 3339284256. * chi1 * chi2 + 2943675504. * chi2 ** 2) * eta2
                          - 324322727232. * eta2 * eta
                          - 7. * (-177520268561. + 107414046432. * chi2 ** 2 + 107414046432. * chi1 ** 2 * sp1
                                  - 107414046432. * chi2 ** 2 * seta + 11087290368. * (chi1 + chi2 + chi1 * seta - chi2 * seta) * PI)
                          + 12. * eta * (-545384828789. - 176491177632. * chi1 * chi2 + 202603761360. * chi2 ** 2
                                         + 77616. * chi1 ** 2 * (2610335. + 995766. * seta) - 77287373856. * chi2 ** 2 * seta
                                         + 5841690624. * (chi1 + chi2) * PI + 21384760320. * PI * PI))) / 6.0085960704e10
    a['73'], a['83'], a['3'] = k['rho1'], k['rho2'], k['rho3']
    return a


def _ins_amp(Mf, a):
    return (1. + Mf ** (2. / 3.) * a['23'] + Mf ** (4. / 3.) * a['43'] + Mf ** (5. / 3.) * a['53']
            + Mf ** (7. / 3.) * a['73'] + Mf ** (8. / 3.) * a['83'] + Mf * (a['1'] + Mf * a['2'] + Mf * Mf * a['3']))


def _ins_amp_d(Mf, a):
    return (2. / 3. * a['23'] * Mf ** (-1. / 3.) + a['1'] + 4. / 3. * a['43'] * Mf ** (1. / 3.) + 5. / 3. * a['53'] * Mf ** (2. / 3.)
            + 2. * a['2'] * Mf + 7. / 3. * a['73'] * Mf ** (4. / 3.) + 8. / 3. * a['83'] * Mf ** (5. / 3.) + 3. * a['3'] * Mf * Mf)


def _mrd_amp(Mf, k):
    fr, fd, g1, g2, g3 = k['fring'], k['fdamp'], k['gamma1'], k['gamma2'], k['gamma3']
    return torch.exp(-(Mf - fr) * g2 / (fd * g3)) * (fd * g3 * g1) / ((Mf - fr) ** 2 + (fd * g3) ** 2)


def _mrd_amp_d(Mf, k):
    fr, fd, g1, g2, g3 = k['fring'], k['fdamp'], k['gamma1'], k['gamma2'], k['gamma3']
    D = (Mf - fr) ** 2 + (fd * g3) ** 2
    return (-2. * fd * (Mf - fr) * g3 * g1 / D - g2 * g1) / (torch.exp((Mf - fr) * g2 / (fd * g3)) * D)


def _int_amp_coeffs(k, a, fpeak):
    """delta_0..delta_4: the quartic through (f1, v1, d1), (f2, v2), (f3, v3, d2) (gwfast/waveforms.py:1199-1245).

    Solved as the 5x5 linear system those conditions define.
    """
    f1 = _T(AMP_FJOIN_INS) * torch.ones_like(fpeak)
    f3 = fpeak
    f2 = f1 + 0.5 * (f3 - f1)
    v1, d1 = _ins_amp(f1, a), _ins_amp_d(f1, a)
    v3, d2 = _mrd_amp(f3, k), _mrd_amp_d(f3, k)
    v2 = k['v2']
    one, zero = torch.ones_like(f1), torch.zeros_like(f1)

    def row_v(x):
        return torch.stack([one, x, x * x, x ** 3, x ** 4], dim=-1)

    def row_d(x):
        return torch.stack([zero, one, 2. * x, 3. * x * x, 4. * x ** 3], dim=-1)

    Mat = torch.stack([row_v(f1), row_d(f1), row_v(f2), row_v(f3), row_d(f3)], dim=-2)   # (N,1,5,5)
    rhs = torch.stack([v1, d1, v2 * one, v3, d2], dim=-1).unsqueeze(-1)                   # (N,1,5,1)
    sol = torch.linalg.solve(Mat, rhs).squeeze(-1)
    return [sol[..., i] for i in range(5)]


def _amp_pieces(Mf, k, a, delta, fpeak):
    ins = _ins_amp(Mf, a)
    itm = delta[0] + Mf * delta[1] + Mf * Mf * (delta[2] + Mf * delta[3] + Mf * Mf * delta[4])
    mrd = _mrd_amp(Mf, k)
    zero = torch.zeros_like(Mf + fpeak)
    return torch.where(Mf < AMP_FJOIN_INS, ins, torch.where(Mf < fpeak, itm, torch.where(Mf < MF_CUT, mrd, zero)))


def _phd_event(Mc, eta, chi1, chi2, dq1=0., dq2=0.):
    aeff = final_spin(eta, chi1, chi2)
    Erad = radiated_energy(eta, chi1, chi2)
    q = qnm_table()
    fring = interp(aeff, q[:, 0].contiguous(), q[:, 1].contiguous()) / (1.0 - Erad)
    fdamp = interp(aeff, q[:, 0].contiguous(), q[:, 2].contiguous()) / (1.0 - Erad)
    return _phenom_core(Mc, eta, chi1, chi2, fring, fdamp, dq1, dq2)


def phd_phase(f, Mc, eta, chi1, chi2, dq1=0., dq2=0.):
    """IMRPhenomD.Phi with fRef = min of the grid (gwfast/waveforms.py:992-1147)."""
    k = _phd_event(Mc, eta, chi1, chi2, dq1, dq2)
    M = k['M']
    Mf = M * GMSUN_OVER_C3 * f
    fr, fd, g2, g3 = k['fring'], k['fdamp'], k['gamma2'], k['gamma3']
    fpeak = torch.where(g2 >= 1.0, torch.abs(fr - fd * g3 / g2),
                        torch.abs(fr + fd * (-1.0 + torch.sqrt(torch.clamp(1.0 - g2 * g2, min=0.))) * g3 / g2))
    t0 = _mrd_phase_raw_d(fpeak, k['alp'], fr, fd, eta)
    fRef = torch.amin(Mf, dim=-1, keepdim=True)
    phis = _phase_pieces(Mf, k, k['C1MRD'], k['C2MRD'])
    phiRef = _phase_pieces(fRef, k, k['C1MRD'], k['C2MRD'])
    return phis + torch.where(Mf < MF_CUT, -t0 * (Mf - fRef) - phiRef, torch.zeros_like(Mf))


def _amp_fpeak(k):
    fr, fd, g2, g3 = k['fring'], k['fdamp'], k['gamma2'], k['gamma3']
    return torch.where(g2 >= 1.0, torch.abs(fr - fd * g3 / g2),
                       fr + fd * (-1.0 + torch.sqrt(torch.clamp(1.0 - g2 * g2, min=0.))) * g3 / g2)


def phd_ampl(f, Mc, eta, chi1, chi2, dL):
    """IMRPhenomD.Ampl (gwfast/waveforms.py:1155-1254)."""
    k = _phd_event(Mc, eta, chi1, chi2)
    M = k['M']
    Mf = M * GMSUN_OVER_C3 * f
    fpeak = _amp_fpeak(k)
    a = _amp_coeffs(k, chi1, chi2)
    delta = _int_amp_coeffs(k, a, fpeak)
    amp0 = torch.sqrt(2.0 * eta / 3.0) * PI ** (-1. / 6.)
    over = 2. * math.sqrt(5. / (64. * PI)) * M * GMSUN_OVER_C2_GPC * M * GMSUN_OVER_C3 / dL
    return over * amp0 * Mf ** (-7. / 6.) * _amp_pieces(Mf, k, a, delta, fpeak)


# ---------------------------------------------------------------- IMRPhenomD_NRTidalv2
def lam12_from_lamt_dellam(lt, dlt, eta):
    """Lambda1, Lambda2 from (LambdaTilde, deltaLambda), gwfast/gwfastUtils.py:419-446."""
    e2 = eta * eta
    seta = _seta(eta)
    lp_ = (8. / 13.) * (1. + 7. * eta - 31. * e2)
    lm_ = (8. / 13.) * seta * (1. + 9. * eta - 11. * e2)
    dp_ = 0.5 * seta * (1. - 13272. / 1319. * eta + 8944. / 1319. * e2)
    dm_ = 0.5 * (1. - 15910. / 1319. * eta + 32850. / 1319. * e2 + 3380. / 1319. * e2 * eta)
    det = (306656. / 1319.) * eta ** 5 - (5936. / 1319.) * eta ** 4
    return ((dp_ - dm_) * lt + (lm_ - lp_) * dlt) / det, ((-dm_ - dp_) * lt + (lm_ + lp_) * dlt) / det


def quad_mon(lam):
    """Spin-induced quadrupole moment from Lambda (arXiv:1608.02582 eq. 15; gwfast/waveforms.py:1402-1403)."""
    ll = torch.log(torch.clamp(lam, min=1.))
    big = torch.exp(0.1940 + 0.09163 * ll + 0.04812 * ll ** 2 - 4.283e-3 * ll ** 3 + 1.245e-4 * ll ** 4)
    small = 1. + lam * (0.427688866723244 + lam * (-0.324336526985068 + lam * 0.1107439432180572))
    return torch.where(lam < 1., small, big)


def oct_mon_m1(qm):
    """Octupole moment minus one from the quadrupole moment (gwfast/waveforms.py:1564-1565)."""
    lq = torch.log(qm)
    return torch.exp(0.003131 + 2.071 * lq - 0.7152 * lq ** 2 + 0.2458 * lq ** 3 - 0.03309 * lq ** 4) - 1.


def nrt_kappa2t(eta, l1, l2):
    """Tidal coupling constant kappa_2^T (arXiv:1905.06011 eq. 8; gwfast/waveforms.py:1546)."""
    seta = _seta(eta)
    xa, xb = 0.5 * (1. + seta), 0.5 * (1. - seta)
    return (3. / 13.) * ((1. + 12. * xb / xa) * xa ** 5 * l1 + (1. + 12. * xa / xb) * xb ** 5 * l2)


def nrt_fmerger(eta, kap):
    """Merger frequency in M f of the Planck taper (gwfast/waveforms.py:1688-1700)."""
    seta = _seta(eta)
    q = 0.5 * (1. + seta - 2. * eta) / eta
    num = 1. + 3.35411203e-2 * kap + 4.31460284e-5 * kap * kap
    den = 1. + 7.54224145e-2 * kap + 2.23626859e-4 * kap * kap
    return 0.3586 / torch.sqrt(q) * (num / den) / (2. * PI)


def nrt_fcut(Mc, eta, lt, dlt):
    """1.2 times the merger frequency, in Hz (gwfast/waveforms.py:1798-1832)."""
    l1, l2 = lam12_from_lamt_dellam(lt, dlt, eta)
    return 1.2 * nrt_fmerger(eta, nrt_kappa2t(eta, l1, l2)) / (Mc * GMSUN_OVER_C3 / eta ** (3. / 5.))


def planck_taper(x, y):
    """Planck taper between y and 1.2 y (gwfast/waveforms.py:1702-1723). As gwfast's custom derivative,
    the tangent flows through the merger frequency y only; NaN values and tangents become zero."""
    a = 1.2
    xv, yv = x.detach(), y.detach()
    yp = a * yv
    z = (yp - yv) / (xv - yv) + (yp - yv) / (xv - yp)
    E = torch.exp(z)
    mid = 1. - 1. / (E + 1.)
    dmid = E * ((a - 1.) / (xv - yv) + (a - 1.) / (xv - yp) + (yp - yv) / (xv - yv) ** 2
                + a * (yp - yv) / (xv - yp) ** 2) / (E + 1.) ** 2
    inside = (xv >= yv) & (xv <= yp)
    t = torch.where(xv < yv, torch.ones_like(xv), torch.where(xv > yp, torch.zeros_like(xv), mid))
    dt = torch.where(inside, dmid, torch.zeros_like(xv))
    t = torch.nan_to_num(t, nan=0.)
    dt = torch.where(torch.isfinite(dt), dt, torch.zeros_like(dt))
    return t + dt * (y - yv)


def _nrt_event(Mc, eta, chi1, chi2, lt, dlt):
    l1, l2 = lam12_from_lamt_dellam(lt, dlt, eta)
    q1, q2 = quad_mon(l1), quad_mon(l2)
    return l1, l2, q1, q2


def nrt_phase(f, Mc, eta, chi1, chi2, lt, dlt):
    """IMRPhenomD_NRTidalv2.Phi (gwfast/waveforms.py:1375-1582): IMRPhenomD with the quadrupole moments
    in the 2PN and 3PN spin-spin terms, plus the NRTidalv2 Pade tidal phase and the 3.5PN spin-squared
    and spin-cubed terms, all under the Mf < 0.2 cut."""
    l1, l2, q1, q2 = _nrt_event(Mc, eta, chi1, chi2, lt, dlt)
    ph = phd_phase(f, Mc, eta, chi1, chi2, q1 - 1., q2 - 1.)
    M = Mc / eta ** (3. / 5.)
    Mf = M * GMSUN_OVER_C3 * f
    px = PI * Mf
    seta = _seta(eta)
    m1, m2 = 0.5 * (1. + seta), 0.5 * (1. - seta)
    kap = nrt_kappa2t(eta, l1, l2)
    num = (1. - 12.615214237993088 * px ** (2. / 3.) + 19.0537346970349 * px - 21.166863146081035 * px ** (4. / 3.)
           + 90.55082156324926 * px ** (5. / 3.) - 60.25357801943598 * px * px)
    den = 1. - 15.11120782773667 * px ** (2. / 3.) + 22.195327350624694 * px + 8.064109635305156 * px ** (4. / 3.)
    tidal = -kap * 2.4375 / (m1 * m2) * px ** (5. / 3.) * num / den
    c12, c22 = chi1 * chi1, chi2 * chi2
    ss = -400. * PI * (q1 - 1.) * c12 * m1 * m1 - 400. * PI * (q2 - 1.) * c22 * m2 * m2
    sss = (10. * ((m1 * m1 + 308. / 3. * m1) * chi1 + (m2 * m2 - 89. / 3. * m2) * chi2) * (q1 - 1.) * m1 * m1 * c12
           + 10. * ((m2 * m2 + 308. / 3. * m2) * chi2 + (m1 * m1 - 89. / 3. * m1) * chi1) * (q2 - 1.) * m2 * m2 * c22
           - 440. * oct_mon_m1(q1) * m1 ** 3 * c12 * chi1 - 440. * oct_mon_m1(q2) * m2 ** 3 * c22 * chi2)
    extra = tidal + (ss + sss) * 3. / (128. * eta) * px ** (2. / 3.)
    return ph + torch.where(Mf < MF_CUT, extra, torch.zeros_like(extra))


def nrt_ampl(f, Mc, eta, chi1, chi2, dL, lt, dlt, taper_last=None):
    """IMRPhenomD_NRTidalv2.Ampl (gwfast/waveforms.py:1584-1723): the IMRPhenomD amplitude plus the
    NRTidalv2 tidal amplitude, times the Planck taper.

    The grid ends at fcut = 1.2 f_merger, so its last point sits on the end of the taper, x = 1.2 y,
    up to rounding; there the formula gives 1 when x equals 1.2 y exactly (the exponent is +inf) and 0
    on either side. ``taper_last`` (bool per event, shape (N, 1)) fixes that point's taper to 1 or 0,
    with no tangent, to reproduce either outcome.
    """
    l1, l2, _, _ = _nrt_event(Mc, eta, chi1, chi2, lt, dlt)
    M = Mc / eta ** (3. / 5.)
    Mf = M * GMSUN_OVER_C3 * f
    kap = nrt_kappa2t(eta, l1, l2)
    xt = (PI * Mf) ** (2. / 3.)
    poly = (1. + 4.157407407407407 * xt + 2519.111111111111 * xt ** 2.89) / (1. + 13477.8073677 * xt ** 4)
    amp_t = -9. * kap * xt ** 3.25 * poly
    over = 2. * math.sqrt(5. / (64. * PI)) * M * GMSUN_OVER_C2_GPC * M * GMSUN_OVER_C3 / dL
    base = phd_ampl(f, Mc, eta, chi1, chi2, dL)
    taper = planck_taper(Mf, nrt_fmerger(eta, kap))
    if taper_last is not None:
        last = torch.zeros(taper.shape, dtype=torch.bool)
        last[..., -1] = True
        forced = torch.as_tensor(taper_last, dtype=DT).reshape(-1, 1).expand(taper.shape)
        taper = torch.where(last, forced, taper)
    return (base + over * 2. * math.sqrt(PI / 5.) * amp_t) * taper


# ---------------------------------------------------------------- IMRPhenomNSBH
# xi_tide of arXiv:1509.00512 eq. 8 on gwfast's regular grid (gwfast/waveforms.py:3286-3343): compactness
# in [0.1, 0.5], mass ratio in [1, 100], BH spin in [-1, 1], 200 points each (numpy linspace)
XI_GRID = (np.linspace(0.1, 0.5, 200), np.linspace(1., 100., 200), np.linspace(-1., 1., 200))
_XI_CACHE = {}


def xitide_node(i, j, k):
    """The table value at grid node (i, j, k): the largest square of the real positive roots of the
    degree-10 polynomial in sqrt(xi) (:3310-3330), found by numpy's companion-matrix roots as gwfast does."""
    key = (i, j, k)
    if key not in _XI_CACHE:
        C, q, chi = XI_GRID[0][i], XI_GRID[1][j], XI_GRID[2][k]
        mu = q * C
        coeffs = np.array([1., 0., -3. * mu, 2. * chi * (mu ** (3. / 2.)), 0., 0., -3. * q, 0., 6. * q * mu, 0.,
                           -3. * q * mu * chi * mu * chi])
        r = np.roots(coeffs)
        rp = np.real(r[(abs(np.imag(r)) < 1e-5) & (np.real(r) > 0.)])
        _XI_CACHE[key] = max(rp * rp)
    return _XI_CACHE[key]


_XI_DENSE = None
_XI_GRID_T = tuple(torch.as_tensor(g, dtype=DT) for g in XI_GRID)


def _xi_dense():
    """The table as a dense tensor, filled node by node as events need them (NaN elsewhere)."""
    global _XI_DENSE
    if _XI_DENSE is None:
        _XI_DENSE = torch.full((200, 200, 200), float('nan'), dtype=DT)
    return _XI_DENSE


def _xi_cells(xs):
    """Cell indices and the out-of-bounds flag of gwfast's RegularGridInterpolator_JAX
    (gwfast/gwfastUtils.py:1182-1200), from plain (detached) coordinates."""
    idx = []
    oob = torch.zeros(xs[0].shape[0], dtype=DT)
    for x, g in zip(xs, _XI_GRID_T):
        i = torch.searchsorted(g, x.contiguous()) - 1
        idx.append(torch.clamp(i, 0, g.numel() - 2))
        oob = ((oob + x) < g[0]).to(DT)
        oob = ((oob + x) > g[-1]).to(DT)
    return idx, oob > 0


def xitide_prepare(C, q, chi):
    """Fill the table nodes around the given points (numpy roots, as gwfast tabulates them)."""
    xs = tuple(torch.as_tensor(np.asarray(a, dtype=np.float64).reshape(-1)) for a in (C, q, chi))
    idx, _ = _xi_cells(xs)
    T = _xi_dense()
    for a, b, c in zip(*(i.numpy() for i in idx)):
        for e0 in (0, 1):
            for e1 in (0, 1):
                for e2 in (0, 1):
                    if torch.isnan(T[a + e0, b + e1, c + e2]):
                        T[a + e0, b + e1, c + e2] = xitide_node(a + e0, b + e1, c + e2)


def xitide_interp(C, q, chi):
    """Trilinear interpolation on the xi_tide grid as gwfast's RegularGridInterpolator_JAX
    (gwfast/gwfastUtils.py:1024-1200): the cell from searchsorted (clamped to the grid), linear
    extrapolation outside it, the edge sum in itertools.product order, and the out-of-bounds test as
    that code writes it (which in effect only flags BH spins above 1). Written in torch operations so
    that it runs inside torch.func.jvp; the nodes are filled beforehand (xitide_prepare, which runs
    here directly when the inputs are plain tensors)."""
    xs = (C.reshape(-1), q.reshape(-1), chi.reshape(-1))
    try:
        xitide_prepare(*(x.detach().numpy() for x in xs))
    except RuntimeError:   # inside a functorch transform: Model.prepare filled the nodes
        pass
    idx, oob = _xi_cells(tuple(x.detach() for x in xs))
    nd = [(x - g[i]) / (g[i + 1] - g[i]) for x, g, i in zip(xs, _XI_GRID_T, idx)]
    T = _xi_dense()
    out = torch.zeros_like(xs[0])
    for e0 in (0, 1):
        for e1 in (0, 1):
            for e2 in (0, 1):
                vals = T[idx[0] + e0, idx[1] + e1, idx[2] + e2]
                w = ((1. - nd[0]) if e0 == 0 else nd[0]) * ((1. - nd[1]) if e1 == 0 else nd[1]) \
                    * ((1. - nd[2]) if e2 == 0 else nd[2])
                out = out + vals * w
    out = torch.where(oob, torch.full_like(out, float('nan')), out)
    return out.reshape(C.shape)


def nsbh_xi_inputs(eta, chi1, lt, dlt):
    """(compactness, m1/m2, BH spin) at which IMRPhenomNSBH reads xi_tide."""
    lam = _nsbh_lambda(eta, lt, dlt)
    seta = _seta(eta)
    q = 0.5 * (1.0 + seta - 2.0 * eta) / eta
    ll = torch.log(torch.clamp(lam, min=1e-300))
    Comp = torch.where(lam > 1., 0.360 - 0.0355 * ll + 0.000705 * ll * ll,
                       0.5 + (3. * 0.360 + 0.0355 - 1.5) * lam * lam + (-2. * 0.360 - 0.0355 + 1.) * lam ** 3)
    return Comp, q, chi1


def _nsbh_common(eta, chi1, lam):
    """Remnant fits shared by the phase and the amplitude (gwfast/waveforms.py:2854-2874, :3124-3151):
    remnant spin chif (arXiv:1903.11622, arXiv:1611.00332 eq. 16) and the spin-weighted BH spin."""
    seta = _seta(eta)
    m1, m2 = 0.5 * (1. + seta), 0.5 * (1. - seta)
    eta2 = eta * eta
    chi12 = chi1 * chi1

    def rem_model(c):
        p1 = ((c[0] * chi1 + c[1]) + (c[2] * chi1 + c[3]) * eta) * eta
        p2 = ((c[4] * chi1 + c[5]) + (c[6] * chi1 + c[7]) * eta) * eta
        p3 = ((c[8] * chi1 + c[9]) + (c[10] * chi1 + c[11]) * eta) * eta
        m = (1. + lam * p1 + lam * lam * p2) / ((1. + lam * p3 * p3) * (1. + lam * p3 * p3))
        one = torch.ones_like(m)
        m = torch.where((chi1 < 0.) & (eta < 0.188), one, m)
        m = torch.where(chi1 < -0.5, one, m)
        return torch.where(m > 1., one, m)

    rem_sp = rem_model((-5.44187381e-03, 7.91165608e-03, 2.33362046e-02, 2.47764497e-02, -8.56844797e-07,
                        -2.81727682e-06, 6.61290966e-06, 4.28979016e-05, -3.04174272e-02, 2.54889050e-01,
                        1.47549350e-01, -4.27905832e-01))
    rem_m = rem_model((-1.83417425e-03, 2.39226041e-03, 4.29407902e-03, 9.79775571e-03, 2.33868869e-07,
                       -8.28090025e-07, -1.64315549e-06, 8.08340931e-06, -2.00726981e-02, 1.31986011e-01,
                       6.50754064e-02, -1.42749961e-01))
    S1 = chi1 * m1 * m1
    Sh = S1 / (m1 * m1 + m2 * m2)
    lorb = ((2. * math.sqrt(3.) * eta + 5.24 * 3.8326341618708577 * eta2 + 1.3 * (-9.487364155598392) * eta * eta2)
            / (1. + 2.88 * 2.5134875145648374 * eta)
            + ((-0.194) * 1.0009563702914628 * Sh * (4.409160174224525 * eta + 0.5118334706832706 * eta2
                                                    + (64. - 16. * 4.409160174224525 - 4. * 0.5118334706832706) * eta2 * eta)
               + 0.0851 * 0.7877509372255369 * Sh * Sh * (8.77367320110712 * eta + (-32.060648277652994) * eta2
                                                          + (64. - 16. * 8.77367320110712 - 4. * (-32.060648277652994)) * eta2 * eta)
               + 0.00954 * 0.6540138407185817 * Sh * Sh * Sh * (22.830033250479833 * eta + (-153.83722669033995) * eta2
                                                                + (64. - 16. * 22.830033250479833 - 4. * (-153.83722669033995)) * eta2 * eta))
            / (1. + (-0.579) * 0.8396665722805308 * Sh * (1.8804718791591157 + (-4.770246856212403) * eta + 0. * eta2
                                                        + (64. - 64. * 1.8804718791591157 - 16. * (-4.770246856212403) - 4. * 0.) * eta2 * eta))
            + 0.3223660562764661 * seta * eta2 * (1. + 9.332575956437443 * eta) * chi1
            + 2.3170397514509933 * Sh * seta * eta2 * eta * (1. + (-3.2624649875884852) * eta) * chi1
            + (-0.059808322561702126) * eta2 * eta * chi12)
    chif = (lorb + S1) * rem_sp
    erad = ((((1. - 2.0 / 3.0 * math.sqrt(2.)) * eta + 0.5609904135313374 * eta2 + (-0.84667563764404) * eta2 * eta
              + 3.145145224278187 * eta2 * eta2)
             * (1. + 0.346 * (-0.2091189048177395) * Sh * (1.8083565298668276 + 15.738082204419655 * eta
                                                          + (16. - 16. * 1.8083565298668276 - 4. * 15.738082204419655) * eta2)
                + 0.211 * (-0.19709136361080587) * Sh * Sh * (4.271313308472851 + 0. * eta + (16. - 16. * 4.271313308472851 - 4. * 0.) * eta2)
                + 0.128 * (-0.1588185739358418) * Sh * Sh * Sh * (31.08987570280556 + (-243.6299258830685) * eta
                                                                  + (16. - 16. * 31.08987570280556 - 4. * (-243.6299258830685)) * eta2)))
            / (1. + (-0.212) * 2.9852925538232014 * Sh * (1.5673498395263061 + (-0.5808669012986468) * eta
                                                        + (16. - 16. * 1.5673498395263061 - 4. * (-0.5808669012986468)) * eta2))
            + (-0.09803730445895877) * seta * eta2 * (1. + (-3.2283713377939134) * eta) * chi1
            + (-0.01978238971523653) * Sh * seta * eta * (1. + (-4.91667749015812) * eta) * chi1
            + 0.01118530335431078 * eta2 * eta * chi12)
    final_mass = (1. - erad) * rem_m
    return m1, m2, chif, final_mass


def nsbh_quad_mon(lam):
    """NS spin-induced quadrupole moment of IMRPhenomNSBH (arXiv:1303.1528 eq. 54; gwfast/waveforms.py:2832)."""
    ll = torch.log(torch.clamp(lam, min=1e-5))
    return torch.where(lam < 1e-5, torch.ones_like(lam),
                       torch.exp(0.194 + 0.0936 * ll + 0.0474 * ll ** 2 - 0.00421 * ll ** 3 + 0.000123 * ll ** 4))


def _nsbh_lambda(eta, lt, dlt):
    # the BH deformability recovered from (LambdaTilde, deltaLambda) is discarded (:2825-2828)
    _, l2 = lam12_from_lamt_dellam(lt, dlt, eta)
    return l2


def _mf_last(Mf, cut_last):
    """M f with its last column moved to just below (cut_last False) or to (True) the M f = 0.2 cut,
    keeping its tangent: the grid ends at M f = 0.2 up to rounding, which decides the side."""
    if cut_last is None:
        return Mf
    c = torch.as_tensor(cut_last).reshape(-1, 1).expand(Mf.shape[0], 1)
    last = Mf[..., -1:]
    tgt = torch.where(c, torch.full_like(last, MF_CUT), torch.full_like(last, np.nextafter(MF_CUT, 0.)))
    return torch.cat([Mf[..., :-1], last + (tgt - last.detach())], dim=-1)


def nsbh_phase(f, Mc, eta, chi1, chi2, lt, dlt, cut_last=None):
    """IMRPhenomNSBH.Phi (gwfast/waveforms.py:2802-3015): IMRPhenomD with the NS quadrupole moment, the
    ringdown from the NSBH remnant spin, t0 taken at the highest grid frequency, + pi, and the NRTidalv2
    tidal phase of the NS."""
    lam = _nsbh_lambda(eta, lt, dlt)
    _, m2, chif, _ = _nsbh_common(eta, chi1, lam)
    seta = _seta(eta)
    m1 = 0.5 * (1. + seta)
    Erad = radiated_energy(eta, chi1, chi2)
    qt = qnm_table()
    fring = interp(chif, qt[:, 0].contiguous(), qt[:, 1].contiguous()) / (1.0 - Erad)
    fdamp = interp(chif, qt[:, 0].contiguous(), qt[:, 2].contiguous()) / (1.0 - Erad)
    k = _phenom_core(Mc, eta, chi1, chi2, fring, fdamp, 0., nsbh_quad_mon(lam) - 1.)
    M = k['M']
    Mf0 = M * GMSUN_OVER_C3 * f
    fpeak = torch.amax(Mf0, dim=-1, keepdim=True)
    Mf = _mf_last(Mf0, cut_last)
    t0 = _mrd_phase_raw_d(fpeak, k['alp'], fring, fdamp, eta)
    fRef = torch.amin(Mf, dim=-1, keepdim=True)
    phis = _phase_pieces(Mf, k, k['C1MRD'], k['C2MRD'])
    phiRef = _phase_pieces(fRef, k, k['C1MRD'], k['C2MRD'])
    kap = (3. / 13.) * ((1. + 12. * m1 / m2) * m2 ** 5 * lam)
    px = PI * Mf
    num = (1. - 12.615214237993088 * px ** (2. / 3.) + 19.0537346970349 * px - 21.166863146081035 * px ** (4. / 3.)
           + 90.55082156324926 * px ** (5. / 3.) - 60.25357801943598 * px * px)
    den = 1. - 15.11120782773667 * px ** (2. / 3.) + 22.195327350624694 * px + 8.064109635305156 * px ** (4. / 3.)
    tidal = -kap * 2.4375 / (m1 * m2) * px ** (5. / 3.) * num / den
    extra = -t0 * (Mf - fRef) - phiRef + PI + tidal
    return phis + torch.where(Mf < MF_CUT, extra, torch.zeros_like(extra))


def nsbh_ampl(f, Mc, eta, chi1, chi2, dL, lt, dlt, cut_last=None):
    """IMRPhenomNSBH.Ampl (gwfast/waveforms.py:3017-3226): the IMRPhenomC-based amplitude with the
    NSBH merger-type windows (arXiv:1509.00512). ``cut_last`` (bool per event) puts the last grid
    point on either side of the M f = 0.2 cut (see _mf_last)."""
    lam = _nsbh_lambda(eta, lt, dlt)
    m1, m2, chif, final_mass = _nsbh_common(eta, chi1, lam)
    seta = _seta(eta)
    q = 0.5 * (1.0 + seta - 2.0 * eta) / eta
    eta2 = eta * eta
    M = Mc / eta ** (3. / 5.)
    MG = M * GMSUN_OVER_C3
    Mf = _mf_last(MG * f, cut_last)
    chieff = m1 * chi1 + m2 * chi2
    chisum = 2. * chieff
    chiprod = chieff * chieff
    eg = EULER_GAMMA
    xdotaN = 64. * eta / 5.
    xdota2 = -7.43 / 3.36 - 11. * eta / 4.
    xdota3 = 4. * PI - 11.3 * chieff / 1.2 + 19. * eta * chisum / 6.
    xdota4 = 3.4103 / 1.8144 + 5 * chiprod + eta * (13.661 / 2.016 - chiprod / 8.) + 5.9 * eta2 / 1.8
    xdota5 = (-PI * (41.59 / 6.72 + 189. * eta / 8.) - chieff * (31.571 / 1.008 - 116.5 * eta / 2.4)
              + chisum * (21.863 * eta / 1.008 - 79. * eta2 / 6.) - 3 * chieff * chiprod / 4. + 9. * eta * chieff * chiprod / 4.)
    xdota6 = (164.47322263 / 1.39708800 - 17.12 * eg / 1.05 + 16. * PI * PI / 3 - 8.56 * math.log(16.) / 1.05
              + eta * (45.1 * PI * PI / 4.8 - 561.98689 / 2.17728) + 5.41 * eta2 / 8.96 - 5.605 * eta * eta2 / 2.592
              - 80. * PI * chieff / 3. + eta * chisum * (20. * PI / 3. - 113.5 * chieff / 3.6)
              + chiprod * (64.153 / 1.008 - 45.7 * eta / 3.6) - chiprod * (7.87 * eta / 1.44 - 30.37 * eta2 / 1.44))
    xdota6log = -856. / 105.
    xdota7 = (-PI * (4.415 / 4.032 - 358.675 * eta / 6.048 - 91.495 * eta2 / 1.512)
              - chieff * (252.9407 / 2.7216 - 845.827 * eta / 6.048 + 415.51 * eta2 / 8.64)
              + chisum * (158.0239 * eta / 5.4432 - 451.597 * eta2 / 6.048 + 20.45 * eta2 * eta / 4.32
                          + 107. * eta * chiprod / 6. - 5. * eta2 * chiprod / 24.)
              + 12. * PI * chiprod - chiprod * chieff * (150.5 / 2.4 + eta / 8.) + chieff * chiprod * (10.1 * eta / 2.4 + 3. * eta2 / 8.))
    AN = 8. * eta * math.sqrt(PI / 5.)
    A2 = (-107. + 55. * eta) / 42.
    A3 = 2. * PI - 4. * chieff / 3. + 2. * eta * chisum / 3.
    A4 = -2.173 / 1.512 - eta * (10.69 / 2.16 - 2. * chiprod) + 2.047 * eta2 / 1.512
    A5 = -10.7 * PI / 2.1 + eta * (3.4 * PI / 2.1)
    A5imag = -24. * eta
    A6 = (270.27409 / 6.46800 - 8.56 * eg / 1.05 + 2. * PI * PI / 3. + eta * (4.1 * PI * PI / 9.6 - 27.8185 / 3.3264)
          - 20.261 * eta2 / 2.772 + 11.4635 * eta * eta2 / 9.9792 - 4.28 * math.log(16.) / 1.05)
    A6log = -428. / 105.
    A6imag = 4.28 * PI / 1.05
    g1 = 4.149e+00 * chieff - 4.070e+00 * chiprod - 8.752e+01 * eta * chieff - 4.897e+01 * eta + 6.665e+02 * eta2
    g1 = torch.where(g1 < 0., torch.zeros_like(g1), g1)
    del1 = -5.472e-02 * chieff + 2.094e-02 * chiprod + 3.554e-01 * eta * chieff + 1.151e-01 * eta + 9.640e-01 * eta2
    del2 = -1.235e+00 * chieff + 3.423e-01 * chiprod + 6.062e+00 * eta * chieff + 5.949e+00 * eta - 1.069e+01 * eta2
    del1 = torch.where(del1 < 0., torch.zeros_like(del1), del1)
    del2 = torch.where(del2 < 1.0e-4, torch.full_like(del2, 1.0e-4), del2)
    d0 = 0.015
    Comp, _, _ = nsbh_xi_inputs(eta, chi1, lt, dlt)
    xi = xitide_interp(Comp, q, chi1)
    r_isco = _r_isco(chi1)
    mt = 0.296 * xi * (1.0 - 2.0 * Comp) - 0.171 * q * Comp * r_isco
    Mtorus = torch.where(mt > 0., mt, torch.zeros_like(mt))
    kap = torch.sqrt(torch.log(2. - chif) / math.log(3.))
    cw = [(1.5578, 2.9031), (1.9510, 5.9210), (2.0997, 2.7606), (1.4109, 5.9143), (0.4106, 2.7952)]
    om_re = 1.0 + kap * sum(a * math.cos(b) * kap ** n for n, (a, b) in enumerate(cw))
    om_im = kap * sum(a * math.sin(b) * kap ** n for n, (a, b) in enumerate(cw))
    fring = 0.5 * om_re / PI / final_mass
    rtide = xi * (1.0 - 2.0 * Comp) / (q * Comp)
    qfac = 0.5 * om_re / om_im
    ftide = torch.abs(1.0 / (PI * (chi1 + torch.sqrt(rtide * rtide * rtide))) * (1.0 + 1.0 / q))
    frt = 0.99 * 0.98 * fring
    gcorr = torch.where(lam > 1.0, torch.full_like(lam, 1.25), 1.0 + 0.5 * lam - 0.25 * lam * lam)
    d2p = torch.where(lam > 1.0, 1.62496 * 0.25 * (1. + torch.tanh(4.0 * ((ftide / frt - 1.) - 0.0188092) / 0.338737)),
                      del2 - 2. * (del2 - 0.81248) * lam + (del2 - 0.81248) * lam * lam)
    sigma = d2p * fring / qfac
    low = ftide < fring
    eps_tide = torch.where(low, torch.zeros_like(ftide),
                           2. * 0.25 * (1 + torch.tanh(4.0 * (((ftide / frt - 1.) * (ftide / frt - 1.) - 0.571505 * Comp
                                                                - 0.00508451 * chi1) + 0.0796251) / 0.0801192)))
    X = 1.29971 - 1.61724 * (Mtorus + 0.424912 * Comp + 0.363604 * torch.sqrt(eta) - 0.0605591 * chi1)
    eps_ins = torch.where(low, torch.where(X > 1., torch.ones_like(X), X), torch.where(Mtorus > 0., X, torch.ones_like(X)))
    Y = 0.137722 - 0.293237 * (Mtorus - 0.132754 * Comp + 0.576669 * torch.sqrt(eta) - 0.0603749 * chi1
                               - 0.0601185 * chi1 * chi1 - 0.0729134 * chi1 * chi1 * chi1)
    W = 0.5 * (1. - torch.tanh(4.0 * (((ftide / frt - 1.) * (ftide / frt - 1.) - 0.657424 * Comp - 0.0259977 * chi1)
                                      + 0.206465) / 0.226844))
    sig_tide = torch.where(low, torch.where(Mtorus > 0., Y, 0.5 * Y + W), W)
    ring_end = torch.where(lam > 1., frt, (1.0 - 0.02 * lam + 0.01 * lam * lam) * 0.98 * fring) / MG
    f0_pn = torch.where(low, torch.where(Mtorus > 0., ftide / MG, ((1.0 - 1.0 / q) * frt + eps_ins * ftide / q) / MG), ring_end)
    f0_pm = torch.where(low, torch.where(Mtorus > 0., ftide / MG, ((1.0 - 1.0 / q) * frt + ftide / q) / MG), ring_end)
    f0_rd = torch.where(low, torch.zeros_like(ring_end), ring_end)
    v = (Mf * PI) ** (1. / 3.)
    px = Mf * PI
    xdot = xdotaN * v ** 10 * (1. + xdota2 * v * v + xdota3 * px + xdota4 * px * v + xdota5 * v * v * px
                               + (xdota6 + xdota6log * 2. * torch.log(v)) * px * px + xdota7 * v * px * px)
    amp_t = torch.sqrt(torch.abs(PI / (1.5 * v * xdot)))
    re = amp_t * AN * v * v * (1. + A2 * v * v + A3 * px + A4 * v * px + A5 * v * v * px + (A6 + A6log * 2. * torch.log(v)) * px * px)
    im = amp_t * AN * v * v * (A5imag * v * v * px + A6imag * px * px)
    aPN = torch.sqrt(re * re + im * im)
    aPM = gcorr * g1 * Mf ** (5. / 6.)
    LRD = sigma * sigma / ((Mf - fring) * (Mf - fring) + sigma * sigma * 0.25)
    aRD = eps_tide * del1 * LRD * Mf ** (-7. / 6.)
    w_pn = 0.5 * (1. - torch.tanh(4. * (Mf - (eps_ins * f0_pn) * MG) / (d0 + sig_tide)))
    w_pm = 0.5 * (1. - torch.tanh(4. * (Mf - f0_pm * MG) / (d0 + sig_tide)))
    w_rd = 0.5 * (1. + torch.tanh(4. * (Mf - f0_rd * MG) / (d0 + sig_tide)))
    imr = aPN * w_pn + aPM * w_pm + aRD * w_rd
    over = 2. * math.sqrt(5. / (64. * PI)) * M * GMSUN_OVER_C2_GPC * M * GMSUN_OVER_C3 / dL
    return over * torch.where(Mf < MF_CUT, imr, torch.zeros_like(imr))


# ---------------------------------------------------------------- IMRPhenomHM
HM_MODES = ((2, 1), (2, 2), (3, 2), (3, 3), (4, 3), (4, 4))
# complex ringdown-frequency fits in kappa (gwfast/waveforms.py:2661-2710): list of (modulus, phase)
RD_FITS = {
    (2, 2): ((1.0, 0.), (1.557847, 2.903124), (1.95097051, 5.920970), (2.09971716, 2.760585), (1.41094660, 5.914340), (0.41063923, 2.795235)),
    (3, 2): ((1.022464, 0.004870), (0.24731213, 0.665292), (1.70468239, 3.138283), (0.94604882, 0.163247), (1.53189884, 5.703573), (2.28052668, 2.685231), (0.92150314, 5.841704)),
    (4, 4): ((2.0, 0.), (2.658908, 3.002787), (2.97825567, 6.050955), (3.21842350, 2.877514), (2.12764967, 5.989669), (0.60338186, 2.830031)),
    (2, 1): ((0.589113, 0.043525), (0.18896353, 2.289868), (1.15012965, 5.810057), (6.04585476, 2.741967), (11.12627777, 5.844130), (9.34711461, 2.669372), (3.03838318, 5.791518)),
    (3, 3): ((1.5, 0.), (2.095657, 2.964973), (2.46964352, 5.996734), (2.66552551, 2.817591), (1.75836443, 5.932693), (0.49905688, 2.781658)),
    (4, 3): ((1.5, 0.), (0.205046, 0.595328), (3.10333396, 3.016200), (4.23612166, 6.038842), (3.02890198, 2.826239), (0.90843949, 5.915164)),
}
COMPL_SHIFT_M = (0., PI * 0.5, 0., -PI * 0.5, PI, PI * 0.5, 0.)   # gwfast/waveforms.py:1872


def rd_freq(finmass, finspin, l, m):
    """Ringdown and damping frequency of mode (l, m) from the fits (gwfast/waveforms.py:2661-2710)."""
    alpha = torch.log(2. - finspin) / math.log(3.)
    beta = 1. / (2. + l - abs(m))
    kappa = alpha ** beta
    re = torch.zeros_like(kappa)
    im = torch.zeros_like(kappa)
    for j, (mod, ph) in enumerate(RD_FITS[(l, m)]):
        kj = kappa ** j if j else torch.ones_like(kappa)
        re = re + mod * math.cos(ph) * kj
        im = im + mod * math.sin(ph) * kj
    return re / (2. * PI * finmass), im / (2. * PI * finmass)


def _hm_pn(x, l, m, eta, seta, chis, chia):
    """Leading-order PN amplitude of mode (l, m) (gwfast/waveforms.py:2503-2515); returns real |H| scaled."""
    v = (2. * PI * x / m) ** (1. / 3.)
    v2 = v * v
    v3 = v2 * v
    if (l, m) == (2, 1):
        re = (math.sqrt(2.0) / 3.0) * (v * seta - v2 * 1.5 * (chia + seta * chis) + v3 * seta * (335.0 / 672.0 + eta * 117.0 / 56.0)
                                        + v3 * v * (chia * (3427.0 / 1344. - eta * 2101.0 / 336.) + seta * chis * (3427.0 / 1344 - eta * 965 / 336) - seta * PI))
        im = (math.sqrt(2.0) / 3.0) * v3 * v * seta * (-0.5 - 2. * 0.69314718056)
        H = torch.sqrt(re * re + im * im)
    elif (l, m) == (2, 2):
        H = torch.ones_like(v)
    elif (l, m) == (3, 2):
        H = torch.abs((1.0 / 3.0) * math.sqrt(5.0 / 7.0) * v2 * (1.0 - 3.0 * eta))
    elif (l, m) == (3, 3):
        H = torch.abs(0.75 * math.sqrt(5.0 / 7.0) * v * seta)
    elif (l, m) == (4, 3):
        H = torch.abs(0.75 * math.sqrt(3.0 / 35.0) * v3 * seta * (1.0 - 2.0 * eta))
    else:
        H = torch.abs((4.0 / 9.0) * math.sqrt(10.0 / 7.0) * v2 * (1.0 - 3.0 * eta))
    return PI * torch.sqrt(eta * 2. / 3.) * v ** (-3.5) * H


def sw_harmonics(iota, l, m):
    """s=-2 spin-weighted spherical harmonics Y_lm and Y_l-m at phi=0 (gwfast/waveforms.py:2517-2524)."""
    c, s = torch.cos(iota), torch.sin(iota)
    ch, sh = torch.cos(iota * 0.5), torch.sin(iota * 0.5)
    if (l, m) == (2, 1):
        return math.sqrt(5.0 / (16.0 * PI)) * s * (1.0 + c), math.sqrt(5.0 / (16.0 * PI)) * s * (1.0 - c)
    if (l, m) == (2, 2):
        return math.sqrt(5.0 / (64.0 * PI)) * (1.0 + c) ** 2, math.sqrt(5.0 / (64.0 * PI)) * (1.0 - c) ** 2
    if (l, m) == (3, 2):
        return math.sqrt(7.0 / PI) * ch ** 4 * (-2.0 + 3.0 * c) * 0.5, math.sqrt(7.0 / (4.0 * PI)) * (2.0 + 3.0 * c) * sh ** 4
    if (l, m) == (3, 3):
        return -math.sqrt(21.0 / (2.0 * PI)) * ch ** 5 * sh, math.sqrt(21.0 / (2.0 * PI)) * ch * sh ** 5
    if (l, m) == (4, 3):
        return (-3.0 * math.sqrt(7.0 / (2.0 * PI)) * ch ** 5 * (-1.0 + 2.0 * c) * sh,
                3.0 * math.sqrt(7.0 / (2.0 * PI)) * ch * (1.0 + 2.0 * c) * sh ** 5)
    return 3.0 * math.sqrt(7.0 / PI) * ch ** 6 * sh * sh, 3.0 * math.sqrt(7.0 / PI) * ch * ch * sh ** 6


def phm_hphc(f, Mc, eta, chi1, chi2, iota, dL):
    """IMRPhenomHM.hphc: plus and cross polarisations summed over modes 21,22,32,33,43,44
    (gwfast/waveforms.py:2256-2616).  Returns (hp, hc) as complex tensors."""
    aeff = final_spin(eta, chi1, chi2)
    finmass = 1. - radiated_energy(eta, chi1, chi2)
    fring, fdamp = rd_freq(finmass, aeff, 2, 2)
    k = _phenom_core(Mc, eta, chi1, chi2, fring, fdamp)
    M = k['M']
    Mf = M * GMSUN_OVER_C3 * f
    fRef = torch.amin(Mf, dim=-1, keepdim=True)
    fpeak = _amp_fpeak(k)
    t0 = _mrd_phase_raw_d(fpeak, k['alp'], fring, fdamp, eta)
    phiRef = _phase_pieces(fRef, k, k['C1MRD'], k['C2MRD'])
    phi0 = 0.5 * phiRef
    a = _amp_coeffs(k, chi1, chi2)
    delta = _int_amp_coeffs(k, a, fpeak)
    amp0 = torch.sqrt(2.0 * eta / 3.0) * PI ** (-1. / 6.)
    over = M * GMSUN_OVER_C2_GPC * M * GMSUN_OVER_C3 / dL
    seta = k['seta']
    chis, chia = 0.5 * (chi1 + chi2), 0.5 * (chi1 - chi2)
    fm = k['fMRDJoin']

    def complete_amp(x):
        return over * amp0 * x ** (-7. / 6.) * _amp_pieces(x, k, a, delta, fpeak)

    hp = torch.zeros_like(Mf, dtype=torch.complex128)
    hc = torch.zeros_like(Mf, dtype=torch.complex128)
    for (l, m) in HM_MODES:
        fr_lm, fd_lm = rd_freq(finmass, aeff, l, m)
        rho, tau = fring / fr_lm, fd_lm / fdamp
        # per-mode merger-ringdown C1 join (gwfast/waveforms.py:2534-2540)
        C2 = k['DPhiIntTempVal'] - _mrd_phase_raw_d(fm, k['alp'], fring, fdamp, eta, rho, tau)
        C1 = k['PhiIntTempVal'] - _mrd_phase_raw(fm, k['alp'], fring, fdamp, eta, rho, tau) - C2 * fm

        def cphase(x):
            return _phase_pieces(x, k, C1, C2, rho, tau)
        # phase frequency map (gwfast/waveforms.py:2544-2563)
        fi_p = PHI_FJOIN_INS / rho
        ai = 2. / m
        Ti = 2. * fi_p / m
        am = (fr_lm * rho - Ti) / (fr_lm - fi_p)
        bm = Ti - fi_p * am
        PhDB = cphase(am * fi_p + bm) / am
        PhDC = cphase(rho * fr_lm) / rho
        PhDBA = cphase(ai * fi_p) / ai
        phC = -PhDB + PhDBA + cphase(am * fr_lm + bm) / am
        ph = torch.where(Mf < fi_p, cphase(Mf * ai) / ai,
                         torch.where(Mf < fr_lm, -PhDB + PhDBA + cphase(Mf * am + bm) / am,
                                     -PhDC + phC + cphase(Mf * rho) / rho))
        ph = ph - t0 * (Mf - fRef) - m * phi0 + COMPL_SHIFT_M[m]
        # amplitude frequency map (gwfast/waveforms.py:2546-2568)
        fi_a = AMP_FJOIN_INS / rho
        Ti_a = 2. * fi_a / m
        am_a = (fring - Ti_a) / (fr_lm - fi_a)
        bm_a = Ti_a - fi_a * am_a
        fs = torch.where(Mf < fi_a, Mf * ai, torch.where(Mf < fr_lm, Mf * am_a + bm_a, Mf - fr_lm + fring))
        bt1 = _hm_pn(Mf, l, m, eta, seta, chis, chia)
        bt2 = _hm_pn(2. * Mf / m, l, m, eta, seta, chis, chia)
        hm1 = _hm_pn(fs, l, m, eta, seta, chis, chia)
        hm2 = PI * torch.sqrt(eta * 2. / 3.) * (PI * fs) ** (-7. / 6.)
        amp = torch.nan_to_num(complete_amp(fs) * (bt1 / bt2) * hm1 / hm2)
        Y, Ym = sw_harmonics(iota, l, m)
        sgn = (-1.) ** l
        e = amp * torch.exp(-1j * ph)
        hp = hp + e * (0.5 * (Y + sgn * Ym))
        hc = hc - e * (-1j * 0.5 * (Y - sgn * Ym))
    return hp, hc


# ---------------------------------------------------------------- detector projection
class Detector:
    """Geometry of one interferometer (gwfast/signal.py:68-160); angles in degrees as in the reference."""

    def __init__(self, lat, lon, xax, shape='L', fmin=2., fmax=None, psd_f=None, psd_S=None, earth=False):
        self.lat = lat * PI / 180.
        self.lon = lon * PI / 180.
        self.xax = xax * PI / 180.
        self.shape = shape
        self.zeta = 0.5 * PI if shape == 'L' else PI / 3.
        self.fmin, self.fmax = fmin, fmax
        self.psd_f = None if psd_f is None else torch.as_tensor(np.asarray(psd_f), dtype=DT)
        self.psd_S = None if psd_S is None else torch.as_tensor(np.asarray(psd_S), dtype=DT)
        self.earth = earth

    @property
    def rots(self):
        return (0.,) if self.shape == 'L' else (0., 60.)


def pattern(det, theta, phi, t, psi, rot=0.):
    """Pattern functions F+, Fx (gwfast/signal.py:342-387)."""
    ra, dec = phi, 0.5 * PI - theta
    x = ra - det.lon - 2. * PI * t
    g = det.xax + rot * PI / 180.
    s2g, c2g = math.sin(2 * g), math.cos(2 * g)
    la = det.lat
    a = (0.0625 * s2g * (3. - math.cos(2. * la)) * (3. - torch.cos(2. * dec)) * torch.cos(2. * x)
         - 0.25 * c2g * math.sin(la) * (3. - torch.cos(2. * dec)) * torch.sin(2. * x)
         + 0.25 * s2g * math.sin(2. * la) * torch.sin(2. * dec) * torch.cos(x)
         - 0.5 * c2g * math.cos(la) * torch.sin(2. * dec) * torch.sin(x)
         + 0.75 * s2g * (math.cos(la) * torch.cos(dec)) ** 2)
    b = (c2g * math.sin(la) * torch.sin(dec) * torch.cos(2. * x)
         + 0.25 * s2g * (3. - math.cos(2. * la)) * torch.sin(dec) * torch.sin(2. * x)
         + c2g * math.cos(la) * torch.cos(dec) * torch.cos(x)
         + 0.5 * s2g * math.sin(2. * la) * torch.cos(dec) * torch.sin(x))
    sz = math.sin(det.zeta)
    return sz * (a * torch.cos(2. * psi) + b * torch.sin(2 * psi)), sz * (b * torch.cos(2. * psi) - a * torch.sin(2 * psi))


def delt_loc(det, theta, phi, t):
    """Earth-centre to detector delay in seconds (gwfast/signal.py:401-423)."""
    ra, dec = phi, 0.5 * PI - theta
    w = det.lon + 2. * PI * t
    comp = (torch.cos(dec) * torch.cos(ra) * math.cos(det.lat) * torch.cos(w)
            + torch.cos(dec) * torch.sin(ra) * math.cos(det.lat) * torch.sin(w)
            + torch.sin(dec) * math.sin(det.lat))
    return -R_EARTH_KM * comp / C_KMS


# ---------------------------------------------------------------- model descriptor
class Model:
    """Which waveform to evaluate: 'TF2' (``tidal``: with the tidal terms), 'PhenomD', 'PhenomHM' or
    'PhenomD_NRTidalv2'."""

    def __init__(self, name, spin_ho=False, tidal=False, taper_last=None, ecc=False, fref_ecc=None, vlso=False,
                 kerr=False, quadmon=False, cut_last=None):
        assert name in ('TF2', 'PhenomD', 'PhenomHM', 'PhenomD_NRTidalv2', 'PhenomNSBH')
        assert not (tidal or ecc or vlso or kerr or quadmon) or name == 'TF2'
        self.name = name
        self.spin_ho = spin_ho
        self.tidal = tidal or name in ('PhenomD_NRTidalv2', 'PhenomNSBH')
        self.taper_last = taper_last   # PhenomD_NRTidalv2: see nrt_ampl
        self.cut_last = cut_last       # PhenomNSBH: see _mf_last
        # TaylorF2 options: is_eccentric (fRef_ecc), phiref_vlso, which_ISCO='Kerr', use_QuadMonTid
        self.ecc, self.fref_ecc, self.vlso, self.kerr, self.quadmon = ecc, fref_ecc, vlso, kerr, quadmon


    @property
    def params(self):
        return (PARAMS_TIDAL if self.tidal else PARAMS) + (('ecc',) if self.ecc else ())

    def prepare(self, p):
        """Work done outside torch.func transforms: IMRPhenomNSBH's xi_tide nodes around the events."""
        if self.name == 'PhenomNSBH':
            C, q, chi = nsbh_xi_inputs(p['eta'], p['chi1z'], p['LambdaTilde'], p['deltaLambda'])
            xitide_prepare(C.detach().numpy(), q.detach().numpy(), chi.detach().numpy())

    @property
    def is_hm(self):
        return self.name == 'PhenomHM'

    def fcut(self, Mc, eta):
        return tf2_fcut(Mc, eta) if self.name == 'TF2' else phd_fcut(Mc, eta)

    def fcut_of(self, p):
        """Upper grid frequency of each event, in Hz."""
        if self.name == 'PhenomD_NRTidalv2':
            return nrt_fcut(p['Mc'], p['eta'], p['LambdaTilde'], p['deltaLambda'])
        if self.kerr:
            return tf2_fcut_kerr(p['Mc'], p['eta'], p['chi1z'], p['chi2z'])
        return self.fcut(p['Mc'], p['eta'])

    def ampl(self, f, p):
        if self.name == 'TF2':
            return tf2_ampl(f, p['Mc'], p['dL'])
        if self.name == 'PhenomD_NRTidalv2':
            return nrt_ampl(f, p['Mc'], p['eta'], p['chi1z'], p['chi2z'], p['dL'], p['LambdaTilde'], p['deltaLambda'],
                            self.taper_last)
        if self.name == 'PhenomNSBH':
            return nsbh_ampl(f, p['Mc'], p['eta'], p['chi1z'], p['chi2z'], p['dL'], p['LambdaTilde'], p['deltaLambda'],
                             self.cut_last)
        return phd_ampl(f, p['Mc'], p['eta'], p['chi1z'], p['chi2z'], p['dL'])

    def phase(self, f, p):
        if self.name == 'TF2':
            lt, dl = (p['LambdaTilde'], p['deltaLambda']) if self.tidal else (None, None)
            return tf2_phase(f, p['Mc'], p['eta'], p['chi1z'], p['chi2z'], self.spin_ho, lt, dl,
                             p['ecc'] if self.ecc else None, self.fref_ecc, self.vlso, self.quadmon)
        if self.name == 'PhenomD_NRTidalv2':
            return nrt_phase(f, p['Mc'], p['eta'], p['chi1z'], p['chi2z'], p['LambdaTilde'], p['deltaLambda'])
        if self.name == 'PhenomNSBH':
            return nsbh_phase(f, p['Mc'], p['eta'], p['chi1z'], p['chi2z'], p['LambdaTilde'], p['deltaLambda'],
                              self.cut_last)
        return phd_phase(f, p['Mc'], p['eta'], p['chi1z'], p['chi2z'])

    def hphc(self, f, p):
        return phm_hphc(f, p['Mc'], p['eta'], p['chi1z'], p['chi2z'], p['iota'], p['dL'])


# ---------------------------------------------------------------- grids and PSD
def freq_grid(fmin, fcut, res, spacing='geom'):
    """Per-event grid (gwfast/signal.py:715-721, :889-898); numpy float64, shape (N, res)."""
    fcut = np.asarray(fcut, dtype=np.float64).reshape(-1)
    fm = np.full(fcut.shape, float(fmin))
    if spacing == 'geom':
        g = np.geomspace(fm, fcut, num=int(res))
    else:
        g = np.linspace(fm, fcut, num=int(res))
    return g.T.copy()


def psd_on_grid(det, f):
    """np.interp with left=right=1 (gwfast/signal.py:723, :901)."""
    return torch.as_tensor(np.interp(f, det.psd_f.numpy(), det.psd_S.numpy(), left=1., right=1.), dtype=DT)


def event_grid(det, model, p, res, spacing='geom'):
    fc = model.fcut_of(p).reshape(-1).detach().numpy()
    if det.fmax is not None:
        fc = np.where(fc > det.fmax, det.fmax, fc)
    f = freq_grid(det.fmin, fc, res, spacing)
    return torch.as_tensor(f, dtype=DT), psd_on_grid(det, f)


def to_params(events, params=PARAMS):
    """dict of 1-D arrays -> dict of (N,1) float64 tensors in the Fisher order."""
    return {k: torch.as_tensor(np.asarray(events[k], dtype=np.float64), dtype=DT).reshape(-1, 1) for k in params}


# ---------------------------------------------------------------- strain
def _time_and_delay(det, model, f, p):
    if det.earth:
        tnoloc = p['tcoal'] - tau_star(f, p['Mc'], p['eta']) / DAY_S
    else:
        tnoloc = p['tcoal']
    dl = delt_loc(det, p['theta'], p['phi'], tnoloc)
    return tnoloc + dl / DAY_S, dl


def amplitudes(det, model, f, p, rot=0.):
    """GWAmplitudes (gwfast/signal.py:425-466): (Ap, Ac) as used by SNRInteg."""
    t, _ = _time_and_delay(det, model, f, p)
    Fp, Fc = pattern(det, p['theta'], p['phi'], t, p['psi'], rot)
    if model.is_hm:
        hp, hc = model.hphc(f, p)
        return torch.abs(hp) * Fp, torch.abs(hc) * Fc
    A = model.ampl(f, p)
    ci = torch.cos(p['iota'])
    return A * Fp * 0.5 * (1. + ci * ci), A * Fc * ci


def strain_parts(det, model, f, p, rot=0.):
    """GWstrain (gwfast/signal.py:485-655) as (Re h, Im h)."""
    t, dl = _time_and_delay(det, model, f, p)
    Fp, Fc = pattern(det, p['theta'], p['phi'], t, p['psi'], rot)
    phiL = 2. * PI * f * dl
    base = 2. * PI * f * (p['tcoal'] * DAY_S) - p['Phicoal']
    if model.is_hm:
        hp, hc = model.hphc(f, p)
        h = (hp * Fp + hc * Fc) * torch.exp(1j * (phiL + base))
        return h.real, h.imag
    A = model.ampl(f, p)
    ci = torch.cos(p['iota'])
    Ap, Ac = A * Fp * 0.5 * (1. + ci * ci), A * Fc * ci
    psi_tot = base - model.phase(f, p) + phiL
    return Ap * torch.cos(psi_tot) - Ac * torch.sin(psi_tot), Ap * torch.sin(psi_tot) + Ac * torch.cos(psi_tot)


def strain(det, model, f, p, rot=0.):
    re, im = strain_parts(det, model, f, p, rot)
    return torch.complex(re, im)


def strain_jacobian(det, model, f, p, rot=0.):
    """d h / d theta_i for the 11 parameters, (11, N, R) complex, tcoal in days (as gwfast/signal.py:1301)."""
    model.prepare(p)
    out = []
    for name in model.params:
        def fn(x, name=name):
            q = dict(p)
            q[name] = x
            return strain_parts(det, model, f, q, rot)
        _, (dre, dim) = torch.func.jvp(fn, (p[name],), (torch.ones_like(p[name]),))
        out.append(torch.complex(dre, dim))
    return torch.stack(out, 0)


def _trapz(y, f):
    return torch.trapezoid(y, f, dim=-1)


# ---------------------------------------------------------------- SNR and Fisher
def snr_arms(det, model, p, res=1000, spacing='geom'):
    """Per-arm SNR^2 integrals (gwfast/signal.py:658-777).  Returns list of (N,) tensors of SNR (not squared)."""
    f, S = event_grid(det, model, p, res, spacing)
    if det.shape == 'L':
        Ap, Ac = amplitudes(det, model, f, p, 0.)
        return [2. * torch.sqrt(_trapz((Ap * Ap + Ac * Ac) / S, f))]
    Ap1, Ac1 = amplitudes(det, model, f, p, 0.)
    Ap2, Ac2 = amplitudes(det, model, f, p, 60.)
    Ap3, Ac3 = -(Ap1 + Ap2), -(Ac1 + Ac2)
    return [2. * torch.sqrt(_trapz((a * a + c * c) / S, f)) for a, c in ((Ap1, Ac1), (Ap2, Ac2), (Ap3, Ac3))]


def snr(det, model, p, res=1000):
    arms = snr_arms(det, model, p, res)
    return torch.sqrt(sum(a * a for a in arms))


def _gram(D, S, f):
    """4 trapz(Re(conj(D_a) D_b)/S, f): (11, N, R) -> (N, 11, 11) (gwfast/signal.py:922-931)."""
    G = torch.einsum('anr,bnr->nabr', D.conj(), D).real / S[:, None, None, :]
    return 4. * _trapz(G, f[:, None, None, :])


def fisher_arms(det, model, p, res=1000, spacing='geom'):
    """Per-arm Fisher matrices, (N, 11, 11) each, tcoal in seconds (gwfast/signal.py:782-1098)."""
    f, S = event_grid(det, model, p, res, spacing)
    Ds = []
    for rot in det.rots:
        D = strain_jacobian(det, model, f, p, rot)
        D[TC_INDEX] = D[TC_INDEX] / DAY_S
        Ds.append(D)
    if det.shape == 'T':
        Ds.append(-(Ds[0] + Ds[1]))
    return [_gram(D, S, f) for D in Ds]


def fisher(det, model, p, res=1000):
    return sum(fisher_arms(det, model, p, res))


def network_snr(dets, model, p, res=1000):
    """DetNet.SNR (gwfast/network.py:53-82)."""
    return torch.sqrt(sum(snr(d, model, p, res) ** 2 for d in dets))


def network_fisher(dets, model, p, res=1000):
    """DetNet.FisherMatr (gwfast/network.py:84-153): (N, 11, 11)."""
    return sum(fisher(d, model, p, res) for d in dets)


# ---------------------------------------------------------------- inversion (fisherTools)
def cov_matr(F, dps=None):
    """Equilibrated Cholesky inverse, per event (gwfast/fisherTools.py:32-196, 'cho' path).

    F: (N, P, P) float64 numpy.  Returns (Cov (N,P,P), eps (N,), cond (N,)) with eps the
    inversion error max|Cov F - 1| (gwfast/fisherTools.py:199-212) and cond the
    condition number of the equilibrated matrix from mpmath.eigh.
    """
    import mpmath
    F = np.asarray(F, dtype=np.float64)
    N, P, _ = F.shape
    cov = np.full_like(F, np.nan)
    cond = np.full(N, np.nan)
    for k in range(N):
        if np.all(np.isnan(F[k])):
            continue
        ctx = mpmath.mp if dps is None else mpmath.mp.clone()
        if dps is not None:
            ctx.dps = dps
        ff = ctx.matrix(F[k].tolist())
        ws = ctx.diag([1 / ctx.sqrt(ff[i, i]) for i in range(P)])
        Fn = ws * ff * ws
        E, _ = ctx.eigh(Fn)
        E = np.array([float(e) for e in E])
        cond[k] = np.max(np.abs(E)) / np.min(np.abs(E))
        try:
            c = ctx.cholesky(Fn) ** -1
            cc = c.T * c
        except Exception:
            U, Sm, V = ctx.svd_r(Fn)
            cc = V.T * ctx.diag([1 / s for s in Sm]) * U.T
        cc = (cc + cc.T) / 2
        C = ws * cc * ws
        cov[k] = np.array(C.tolist(), dtype=np.float64)
    eps = np.array([np.max(np.abs(cov[k] @ F[k] - np.eye(P))) for k in range(N)])
    return cov, eps, cond


def cov_matr_fast(F):
    """float64 numpy version of the same equilibrated Cholesky inverse (for large batches)."""
    F = np.asarray(F, dtype=np.float64)
    d = 1. / np.sqrt(np.einsum('nii->ni', F))
    Fn = F * d[:, :, None] * d[:, None, :]
    L = np.linalg.cholesky(Fn)
    Li = np.linalg.inv(L)
    cc = np.einsum('nki,nkj->nij', Li, Li)
    cc = 0.5 * (cc + np.swapaxes(cc, 1, 2))
    cov = cc * d[:, :, None] * d[:, None, :]
    eps = np.abs(cov @ F - np.eye(F.shape[-1])).max(axis=(1, 2))
    return cov, eps


# ---------------------------------------------------------------- analytic aLIGO PSD
def aligo_psd(f):
    """S(f) = 1e-49 [x^-4.14 - 5 x^-2 + 111 (1 - x^2 + x^4/2)/(1 + x^2/2)], x = f/215 Hz."""
    x = np.asarray(f, dtype=np.float64) / 215.
    return 1e-49 * (x ** -4.14 - 5. * x ** -2 + 111. * (1. - x * x + 0.5 * x ** 4) / (1. + 0.5 * x * x))


def snr_derivs_arms(det, model, p, res=1000):
    """Per-arm 4 trapz(Re(h conj(dh/dtheta)) / S, f), (11, N) each, tcoal in seconds
    (gwfast/signal.py:938-945, :1016-1022, :1090-1094)."""
    f, S = event_grid(det, model, p, res)
    hs, Ds = [], []
    for rot in det.rots:
        D = strain_jacobian(det, model, f, p, rot)
        D[TC_INDEX] = D[TC_INDEX] / DAY_S
        Ds.append(D)
        hs.append(strain(det, model, f, p, rot))
    if det.shape == 'T':
        Ds.append(-(Ds[0] + Ds[1]))
        hs.append(-(hs[0] + hs[1]))
    return [4. * _trapz((h[None] * D.conj()).real / S[None], f[None]) for h, D in zip(hs, Ds)]


def strain_derivs_arms(det, model, p, res=1000, spacing='geom'):
    """Per-arm d h / d theta on the event grids, (11, N, R) complex each, tcoal row in 1/s
    (gwfast/signal.py:913-916, :938-939; triangle arms: 0, 60 degrees and minus their sum, :1057)."""
    f, _ = event_grid(det, model, p, res, spacing)
    Ds = []
    for rot in det.rots:
        D = strain_jacobian(det, model, f, p, rot)
        D[TC_INDEX] = D[TC_INDEX] / DAY_S
        Ds.append(D)
    if det.shape == 'T':
        Ds.append(-(Ds[0] + Ds[1]))
    return Ds


def overlap_parts(det, model1, p1, model2, p2, res=1000):
    """One detector of WFOverlap (gwfast/signal.py:1759-1921): (h1|h2), SNR_1^2, SNR_2^2 summed over
    the arms, on the geometric grid from fmin to max(fcut_1, fcut_2) (with fmax: fmax where that
    maximum exceeds it, else fcut_1, as :1865-1866 reads)."""
    fc1 = model1.fcut_of(p1).reshape(-1).detach().numpy()
    fc2 = model2.fcut_of(p2).reshape(-1).detach().numpy()
    fu = np.where(fc1 > fc2, fc1, fc2)
    if det.fmax is not None:
        fu = np.where(fu > det.fmax, det.fmax, fc1)
    fn = freq_grid(det.fmin, fu, res)
    S = psd_on_grid(det, fn)
    f = torch.as_tensor(fn, dtype=DT)
    h1 = [strain(det, model1, f, p1, rot) for rot in det.rots]
    h2 = [strain(det, model2, f, p2, rot) for rot in det.rots]
    if det.shape == 'T':
        h1.append(-(h1[0] + h1[1]))
        h2.append(-(h2[0] + h2[1]))
    ov = sum(4. * _trapz((a * b.conj()).real / S, f) for a, b in zip(h1, h2))
    n1 = sum(4. * _trapz((a * a.conj()).real / S, f) for a in h1)
    n2 = sum(4. * _trapz((b * b.conj()).real / S, f) for b in h2)
    return ov, n1, n2

