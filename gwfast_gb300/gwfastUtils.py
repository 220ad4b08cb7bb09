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
