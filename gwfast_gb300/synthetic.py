"""Seeded synthetic event catalogues and detector networks for the benchmark workloads.

No public catalogue is used; each workload draws its events from the stated
distributions with numpy's default_rng(seed), in the fixed order
m1, m2 (or q), chi1z, chi2z, dL, theta, phi, iota, psi, tcoal, Phicoal.
"""
import numpy as np

from . import gwfastGlobals as glob
from .gwfastUtils import Mceta_from_m1m2
from .psd import aligo_table


def _angles(rng, n, ev):
    ev['theta'] = np.arccos(rng.uniform(-1., 1., n))
    ev['phi'] = rng.uniform(0., 2. * np.pi, n)
    ev['iota'] = np.arccos(rng.uniform(-1., 1., n))
    ev['psi'] = rng.uniform(0., np.pi, n)
    ev['tcoal'] = rng.uniform(0., 1., n)
    ev['Phicoal'] = rng.uniform(0., 2. * np.pi, n)
    return ev


def bns_events(n, seed=1000, chimax=0.05, dl=(0.05, 0.5)):
    """BNS: m1, m2 ~ U[1.1, 2.0] Msun (m1 >= m2), chi ~ U[-chimax, chimax], dL ~ U[dl] Gpc."""
    rng = np.random.default_rng(seed)
    m = np.sort(rng.uniform(1.1, 2.0, (n, 2)), axis=1)[:, ::-1]
    Mc, eta = Mceta_from_m1m2(m[:, 0], m[:, 1])
    ev = {'Mc': Mc, 'eta': eta, 'chi1z': rng.uniform(-chimax, chimax, n), 'chi2z': rng.uniform(-chimax, chimax, n),
          'dL': rng.uniform(dl[0], dl[1], n)}
    return _angles(rng, n, ev)


def bbh_events(n, seed=1001, mmin=5., mmax=80., alpha=-2.3, qmin=0.2, chimax=0.8, dl=(0.5, 10.)):
    """BBH: m1 ~ power law alpha on [mmin, mmax] (inverse CDF), q ~ U[qmin, 1], chi ~ U[-chimax, chimax]."""
    rng = np.random.default_rng(seed)
    a1 = alpha + 1.
    u = rng.uniform(0., 1., n)
    m1 = (mmin ** a1 + u * (mmax ** a1 - mmin ** a1)) ** (1. / a1)
    q = rng.uniform(qmin, 1., n)
    Mc, eta = Mceta_from_m1m2(m1, q * m1)
    ev = {'Mc': Mc, 'eta': eta, 'chi1z': rng.uniform(-chimax, chimax, n), 'chi2z': rng.uniform(-chimax, chimax, n),
          'dL': rng.uniform(dl[0], dl[1], n)}
    return _angles(rng, n, ev)


def mixed_events(n, seed=1002, bns_fraction=0.5):
    """Mixed catalogue: the first round(n * bns_fraction) events BNS (bns_events distributions), the
    rest BBH (bbh_events distributions), each part from its own stream of the seed."""
    nb = int(round(n * bns_fraction))
    a, b = bns_events(nb, seed=seed), bbh_events(n - nb, seed=seed + 1)
    return {k: np.concatenate([np.asarray(a[k]), np.asarray(b[k])]) for k in a}


def screen_population(n, seed=1004, dl_max=30.):
    """Learned-screen population: the mixed catalogue's distributions with dL ~ U[dL_min, dl_max] Gpc."""
    ev = mixed_events(n, seed=seed)
    rng = np.random.default_rng(seed + 10)
    nb = int(round(n * 0.5))
    ev['dL'] = np.concatenate([rng.uniform(0.05, dl_max, nb), rng.uniform(0.5, dl_max, n - nb)])
    return ev


def chirp_time(Mc, f):
    """Leading-order time to coalescence from frequency f [Hz] for chirp mass Mc [Msun], seconds."""
    tM = np.asarray(Mc) * glob.GMsun_over_c3
    return 5. / 256. * (np.pi * f) ** (-8. / 3.) * tM ** (-5. / 3.)


def res_from_chirp_time(Mc, fmin, lo=200, hi=40000, mc_ref=None):
    """Per-event grid length R = clip(round(k sqrt(tau)), lo, hi) with tau the Newtonian chirp time
    from fmin; k puts the lightest BNS of the bns_events distribution (m1 = m2 = 1.1 Msun) at hi."""
    if mc_ref is None:
        mc_ref = Mceta_from_m1m2(np.array([1.1]), np.array([1.1]))[0][0]
    k = hi / np.sqrt(chirp_time(mc_ref, fmin))
    r = k * np.sqrt(chirp_time(Mc, fmin))
    return np.clip(np.rint(r), lo, hi).astype(np.int32)


# detector networks: name -> (low-frequency wall / fmin in Hz)
NETWORK_LHET = (('L1', 10.), ('H1', 10.), ('ETS', 5.))
NETWORK_ET_CE = (('ETS', 5.), ('CE1Id', 5.), ('CE2NM', 5.))
NETWORK_LHET2 = (('L1', 10.), ('H1', 10.), ('ETS', 2.))   # mixed catalogue: ET wall at 2 Hz


def detector_spec(name, fmin):
    d = glob.detectors[name]
    f, S = aligo_table(fmin)
    return dict(det_lat=d['lat'], det_long=d['long'], det_xax=d['xax'], detector_shape=d['shape'], fmin=fmin,
                psd_path=(f, S), is_ASD=False)


def make_network(wf_model, dets=NETWORK_LHET, earth=True, device=0):
    """DetNet of GWSignal objects with the analytic aLIGO PSD tabulated from each detector's wall."""
    from .network import DetNet
    from .signal import GWSignal
    sigs = {}
    for name, fmin in dets:
        sigs[name] = GWSignal(wf_model, useEarthMotion=earth, verbose=False, device=device, **detector_spec(name, fmin))
    return DetNet(sigs, verbose=False)
