"""Host-side helpers used on the hot path (gwfast/gwfastUtils.py:151-164, :450-482, :965-1020)."""
import numpy as np


def ra_dec_from_th_phi_rad(theta, phi):
    """(theta, phi) -> (ra, dec) in radians (gwfast/gwfastUtils.py:151-164)."""
    return phi, 0.5 * np.pi - theta


def th_phi_from_ra_dec_rad(ra, dec):
    return 0.5 * np.pi - dec, ra


def m1m2_from_Mceta(Mc, eta):
    """gwfast/gwfastUtils.py:450-465."""
    seta = np.sqrt(np.where(eta < 0.25, 1.0 - 4.0 * eta, 0.))
    M = Mc / eta ** (3. / 5.)
    return 0.5 * M * (1. + seta), 0.5 * M * (1. - seta)


def Mceta_from_m1m2(m1, m2):
    """gwfast/gwfastUtils.py:467-482."""
    Mc = (m1 * m2) ** (3. / 5.) / (m1 + m2) ** (1. / 5.)
    eta = (m1 * m2) / ((m1 + m2) * (m1 + m2))
    return Mc, eta


def check_evparams(evParams):
    """Fill the derived parameters in place, as gwfast/gwfastUtils.py:965-1020 does.

    tcoal from tGPS needs a GMST conversion (astropy in gwfast); it is not provided
    here, so a dict without tcoal raises the same ValueError as a dict without tGPS.
    """
    if 'tcoal' not in evParams:
        if 'tGPS' in evParams:
            raise ValueError('tcoal must be given as GMST (days); the tGPS conversion needs astropy, which this '
                             'package does not use.')
        raise ValueError('One among tGPS and tcoal has to be provided.')
    if 'iota' not in evParams:
        if 'thetaJN' in evParams:
            evParams['iota'] = evParams['thetaJN']
        else:
            raise ValueError('One among iota and thetaJN has to be provided.')
    if 'Mc' not in evParams:
        if 'm1' in evParams and 'm2' in evParams:
            evParams['Mc'], evParams['eta'] = Mceta_from_m1m2(evParams['m1'], evParams['m2'])
        else:
            raise ValueError('Two among (Mc, eta) and (m1, m2) have to be provided.')
    if 'theta' not in evParams:
        if 'dec' in evParams and 'ra' in evParams:
            evParams['theta'] = np.pi / 2 - evParams['dec']
            evParams['phi'] = evParams['ra']
        else:
            raise ValueError('Two among (theta, phi) and (ra, dec) have to be provided.')
    return evParams


def fill_spins(evParams):
    """chi1z/chi2z from chiS/chiA when missing (gwfast/signal.py:694-704)."""
    if 'chi1z' not in evParams:
        try:
            evParams['chi1z'] = evParams['chiS'] + evParams['chiA']
            evParams['chi2z'] = evParams['chiS'] - evParams['chiA']
        except KeyError:
            raise ValueError('Two among chi1z, chi2z and chiS, chiA have to be provided.')
    return evParams


def Lamt_delLam_from_Lam12(Lambda1, Lambda2, eta):
    """(LambdaTilde, deltaLambda) from the component tidal deformabilities (gwfast/gwfastUtils.py:398-417;
    arXiv:1402.5156 eqs. 5-6)."""
    eta = np.asarray(eta)
    eta2 = eta * eta
    seta = np.sqrt(np.where(eta < 0.25, 1.0 - 4.0 * eta, 0.))
    lp, lm = Lambda1 + Lambda2, Lambda1 - Lambda2
    lamt = (8. / 13.) * ((1. + 7. * eta - 31. * eta2) * lp + seta * (1. + 9. * eta - 11. * eta2) * lm)
    dlam = 0.5 * (seta * (1. - 13272. / 1319. * eta + 8944. / 1319. * eta2) * lp
                  + (1. - 15910. / 1319. * eta + 32850. / 1319. * eta2 + 3380. / 1319. * eta2 * eta) * lm)
    return lamt, dlam


def Lam12_from_Lamt_delLam(Lamt, delLam, eta):
    """The inverse map (gwfast/gwfastUtils.py:419-446): solve the 2 x 2 linear system of the forward map."""
    eta = np.asarray(eta)
    eta2 = eta * eta
    seta = np.sqrt(np.where(eta < 0.25, 1.0 - 4.0 * eta, 0.))
    a_p = (8. / 13.) * (1. + 7. * eta - 31. * eta2)            # LambdaTilde = a_p L+ + a_m L-
    a_m = (8. / 13.) * seta * (1. + 9. * eta - 11. * eta2)
    b_p = 0.5 * seta * (1. - 13272. / 1319. * eta + 8944. / 1319. * eta2)   # deltaLambda = b_p L+ + b_m L-
    b_m = 0.5 * (1. - 15910. / 1319. * eta + 32850. / 1319. * eta2 + 3380. / 1319. * eta2 * eta)
    det = a_p * b_m - a_m * b_p
    lp = (b_m * Lamt - a_m * delLam) / det
    lm = (a_p * delLam - b_p * Lamt) / det
    return 0.5 * (lp + lm), 0.5 * (lp - lm)


def fill_tidal(evParams):
    """LambdaTilde/deltaLambda from Lambda1/Lambda2 (or the reverse) as gwfast/signal.py:706-713, :863-871 do;
    the dict gains both pairs."""
    if 'Lambda1' in evParams and 'Lambda2' in evParams:
        evParams['LambdaTilde'], evParams['deltaLambda'] = Lamt_delLam_from_Lam12(
            np.asarray(evParams['Lambda1']), np.asarray(evParams['Lambda2']), evParams['eta'])
    elif 'LambdaTilde' in evParams and 'deltaLambda' in evParams:
        evParams['Lambda1'], evParams['Lambda2'] = Lam12_from_Lamt_delLam(
            np.asarray(evParams['LambdaTilde']), np.asarray(evParams['deltaLambda']), evParams['eta'])
    else:
        raise ValueError('Two among Lambda1, Lambda2 and LambdaTilde and deltaLambda have to be provided.')
    return evParams

