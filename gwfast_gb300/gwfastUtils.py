"""Host-side helpers used on the hot path (gwfast/gwfastUtils.py:151-164, :450-482, :731-769, :965-1020)."""
import datetime as _dt

import numpy as np

from . import gwfastGlobals as _glob


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


# UTC dates at which a leap second took effect (published by the IERS); GPS - UTC is the number of
# these at or before an instant (GPS time started at 1980-01-06 00:00:00 UTC, GPS - UTC = 0)
_LEAP_DATES = ((1981, 7, 1), (1982, 7, 1), (1983, 7, 1), (1985, 7, 1), (1988, 1, 1), (1990, 1, 1), (1991, 1, 1),
               (1992, 7, 1), (1993, 7, 1), (1994, 7, 1), (1996, 1, 1), (1997, 7, 1), (1999, 1, 1), (2006, 1, 1),
               (2009, 1, 1), (2012, 7, 1), (2015, 7, 1), (2017, 1, 1))
_GPS_EPOCH = _dt.date(1980, 1, 6)
# GPS second of the leap second inserted before each date (the i leaps before it already counted)
_LEAP_GPS = np.array([(_dt.date(*d) - _GPS_EPOCH).days * 86400 + i for i, d in enumerate(_LEAP_DATES)],
                     dtype=np.float64)
# 2000-01-01 12:00:00 on the GPS calendar, in GPS seconds (7300 days and 12 h after the GPS epoch)
_GPS_NOON_J2000 = float((_dt.date(2000, 1, 1) - _GPS_EPOCH).days * 86400 + 43200)
_TT_MINUS_GPS = 19.0 + 32.184   # TAI - GPS = 19 s, TT - TAI = 32.184 s


def GPSt_to_J200t(t_GPS):
    """Seconds since J2000 (gwfast/gwfastUtils.py:731-733, the same constant)."""
    return t_GPS - 630763148.0


def leap_seconds(t_GPS):
    """GPS - UTC in seconds at GPS time(s) t_GPS (from the published leap-second dates)."""
    return np.searchsorted(_LEAP_GPS, np.asarray(t_GPS, dtype=np.float64), side='right').astype(np.float64)


def GPSt_to_GMST(t_GPS):
    """Greenwich mean sidereal time as a fraction of a day, from GPS time (s).

    gwfast calls astropy (``Time(t, format='gps').sidereal_time('mean')``, gwfast/gwfastUtils.py:735-755),
    which evaluates the IAU 2006 GMST: the Earth rotation angle of UT1,
    ERA = 2 pi (0.7790572732640 + 1.00273781191135448 Du), Du = JD(UT1) - 2451545.0, plus the precession
    polynomial 0.014506" + 4612.156534" t + 1.3915817" t^2 - 0.00000044" t^3 - 0.000029956" t^4
    - 0.0000000368" t^5 in TT Julian centuries t (Capitaine et al. 2003, A&A 412, 567; IERS Conventions
    2010 eq. 5.32). This evaluates the same formula with UTC (GPS minus the leap seconds) standing in
    for UT1: |UT1 - UTC| <= 0.9 s by the definition of UTC, so the result is within 1.05e-5 of a day of
    astropy's value (0.34 s for GW170817, when UT1 - UTC was +0.34 s). Du is split into whole days and
    the fraction so that the fraction keeps full precision.
    """
    t = np.asarray(t_GPS, dtype=np.float64)
    du = (t - leap_seconds(t) - _GPS_NOON_J2000) / 86400.
    era = np.mod(np.mod(du, 1.0) + 0.7790572732640 + 0.00273781191135448 * du, 1.0)
    T = (t + _TT_MINUS_GPS - _GPS_NOON_J2000) / 86400. / 36525.
    arcsec = 0.014506 + T * (4612.156534 + T * (1.3915817 + T * (-0.00000044 + T * (-0.000029956 + T * (-0.0000000368)))))
    return np.mod(era + arcsec / (3600. * 360.), 1.0)


def GPSt_to_LMST(t_GPS, lat, long):
    """Local mean sidereal time as a fraction of a day (gwfast/gwfastUtils.py:735-755): GMST plus the
    longitude (deg). The latitude does not enter the mean sidereal time."""
    del lat
    return np.mod(GPSt_to_GMST(t_GPS) + np.asarray(long, dtype=np.float64) / 360., 1.0)


def GPSt_to_GMST_alt(t_GPS):
    """gwfast's approximate GMST (fraction of a day), linear in GPS time with no leap seconds
    (gwfast/gwfastUtils.py:757-769)."""
    return np.mod(9.533088395981618 + (np.asarray(t_GPS, dtype=np.float64) - 1126260000.) / 3600. * 24.
                  / _glob.siderealDay, 24.) / 24.


def check_evparams(evParams):
    """Fill the derived parameters in place, as gwfast/gwfastUtils.py:965-1020 does: tcoal (GMST,
    fraction of a day) from tGPS, iota from thetaJN, (Mc, eta) from (m1, m2), (theta, phi) from (ra, dec)."""
    if 'tcoal' not in evParams:
        if 'tGPS' in evParams:
            print('Adding tcoal from tGPS')
            # gwfast's convention: GMST, i.e. the local mean sidereal time at longitude 0
            evParams['tcoal'] = GPSt_to_LMST(evParams['tGPS'], lat=0., long=0.)
        else:
            raise ValueError('One among tGPS and tcoal has to be provided.')
    if 'iota' not in evParams:
        if 'thetaJN' in evParams:
            evParams['iota'] = evParams['thetaJN']
        else:
            raise ValueError('One among iota and thetaJN has to be provided.')
    if 'Mc' not in evParams:
        if 'm1' in evParams and 'm2' in evParams:
            print('Adding Mc and eta from the individual detector-frame masses')
            evParams['Mc'], evParams['eta'] = Mceta_from_m1m2(evParams['m1'], evParams['m2'])
        else:
            raise ValueError('Two among (Mc, eta) and (m1, m2) have to be provided.')
    if 'theta' not in evParams:
        if 'dec' in evParams and 'ra' in evParams:
            print('Adding (theta, phi) from (ra, dec)')
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

