"""Generate golden vectors by running gwfast's own sources (v1.1.2) in this container.

gwfast imports jax, h5py and numdifftools, none of which are installed here.  The
hot-path code it runs is plain array arithmetic, so this script installs small
stand-in modules before importing it:

* ``jax.numpy`` is numpy itself (float64, same function names);
* ``jax.jacrev`` is a 5-point central finite difference (only used for the Fisher
  golden; its rounding through the ~1e5-rad phase limits that golden, see the tests); where the
  unperturbed strain is exactly zero (the frequency cut of the IMR models, ``np.where(Mf < 0.2, ..., 0)``)
  the derivative is zero, as JAX's derivative of that branch is, instead of the jump a finite
  difference across the cut would see at the last grid point;
* ``jax.vmap`` loops over the leading (event) axis;
* ``jax.custom_jvp`` calls the function; for a function whose tangents gwfast gives with
  ``defjvps`` (the Planck taper of IMRPhenomD_NRTidalv2, with no tangent in its first argument),
  the perturbed evaluations of the finite differences return the unperturbed value plus those
  registered tangents times the argument changes, so the differences follow the same rule;
* ``h5py`` / ``numdifftools`` are empty modules (only touched off the hot path).

numpy 2 removed ``trapz`` and ``NaN`` and scipy removed ``cumtrapz``; aliases to
``trapezoid``/``nan``/``cumulative_trapezoid`` are installed for the reference's calls.

The outputs are written to ``tests/golden/*.npz`` and committed; the GPU machine
never needs the reference.  Run:  python tests/golden/make_golden.py <gwfast checkout> [part ...]
(with parts, e.g. ``overlap``, only those ``make_<part>()`` run).
"""
import os
import sys
import types

import numpy as np

if __name__ == '__main__' and len(sys.argv) < 2:
    sys.exit('usage: python make_golden.py <gwfast checkout> [part ...]')
REF = sys.argv[1] if len(sys.argv) > 1 else None
OUT = os.path.dirname(os.path.abspath(__file__))


# ------------------------------------------------------------------ stand-in modules
# finite-difference state shared by the jacrev and custom_jvp stand-ins: 'record' stores the
# arguments and value of every defjvps custom_jvp call of the unperturbed evaluation, 'replay'
# linearises the perturbed calls, in call order, about them
_FD = {'mode': None, 'store': [], 'i': 0, 'lam_h': None}


def _install_shims():
    jax = types.ModuleType('jax')
    jax.numpy = np
    cfg = types.SimpleNamespace(update=lambda *a, **k: None)
    jax.config = cfg
    jax.devices = lambda *a, **k: ['cpu']
    jax.local_device_count = lambda: 1
    jax.device_count = lambda: 1

    def vmap(fn):
        def run(*args):
            n = len(args[1])
            outs = [fn(*[a[i] for a in args]) for i in range(n)]
            if isinstance(outs[0], tuple):
                return tuple(np.stack([o[j] for o in outs]) for j in range(len(outs[0])))
            return np.stack(outs)
        return run

    def jacrev(fn, argnums=0, holomorphic=False):
        nums = argnums if isinstance(argnums, tuple) else (argnums,)

        def run(*args):
            res = []
            for j in nums:
                x = args[j]
                xr = np.real(x)
                # Mc, eta: relative steps. LambdaTilde, deltaLambda (arguments 16, 17): the phase is
                # linear in them and their tangents are tiny at low frequency, so the steps must be
                # large enough to keep the rounding of the ~1e5-rad phase out of the difference and
                # small enough that the phase change stays << 1 rad at the top of the band
                # (d Phi / d deltaLambda ~ sqrt(1 - 4 eta) v^7 is far smaller than d Phi / d LambdaTilde).
                # IMRPhenomD_NRTidalv2 is not linear in them (the spin-induced moments depend on
                # Lambda1, Lambda2 through exp(poly(log Lambda))) and its events include stars with
                # Lambda < 1: there a fixed small step (_FD['lam_h']) keeps both Lambdas positive.
                # The rest: 1e-6.
                if j in (1, 2):
                    h = 1e-7 * max(abs(float(xr)), 1e-1)
                elif j in (16, 17) and _FD['lam_h'] is not None:
                    h = _FD['lam_h']
                elif j == 16:
                    h = 1e-3 * max(abs(float(xr)), 1.)
                elif j == 17:
                    h = 10.
                else:
                    h = 1e-6
                def at(d):
                    a = list(args)
                    a[j] = x + d
                    _FD['i'] = 0
                    return np.asarray(fn(*a))
                _FD['mode'], _FD['store'] = 'record', []
                base = at(0.)
                _FD['mode'] = 'replay'
                d1 = (-at(2 * h) + 8 * at(h) - 8 * at(-h) + at(-2 * h)) / (12 * h)
                _FD['mode'] = None
                d1 = np.where(base == 0, 0., d1)
                res.append(d1)
            return tuple(res) if isinstance(argnums, tuple) else res[0]
        return run

    jax.vmap = vmap
    jax.jacrev = jacrev
    jax.jit = lambda f, **k: f
    jax.pmap = lambda f, **k: f

    class custom_jvp:
        def __init__(self, fun, nondiff_argnums=()):
            self.fun = fun
            self.jvps = None

        def defjvp(self, jvp):
            return jvp

        def defjvps(self, *jvps):
            self.jvps = jvps

        def __call__(self, *a, **k):
            if self.jvps is None or _FD['mode'] is None:
                return self.fun(*a, **k)
            if _FD['mode'] == 'record':
                out = self.fun(*a, **k)
                _FD['store'].append((a, out))
                return out
            a0, out0 = _FD['store'][_FD['i']]
            _FD['i'] += 1
            out = out0
            for q, jv in enumerate(self.jvps):
                if jv is not None:
                    out = out + jv(a[q] - a0[q], out0, *a0)
            return out
    jax.custom_jvp = custom_jvp
    interp = types.ModuleType('jax.interpreters')
    interp.xla = types.ModuleType('jax.interpreters.xla')
    jax.interpreters = interp
    sys.modules['jax'] = jax
    sys.modules['jax.numpy'] = np
    sys.modules['jax.interpreters'] = interp
    sys.modules['jax.interpreters.xla'] = interp.xla
    h5 = types.ModuleType('h5py')

    class _NoFile:   # IMRPhenomNSBH stores its xi_tide table with h5py: written nowhere here
        def __init__(self, *a, **k):
            self.attrs = {}

        def __enter__(self):
            return self

        def __exit__(self, *a):
            return False

        def create_dataset(self, *a, **k):
            return None
    h5.File = _NoFile
    sys.modules['h5py'] = h5
    ndt = types.ModuleType('numdifftools')
    sg = types.ModuleType('numdifftools.step_generators')
    sg.MaxStepGenerator = lambda **k: None
    ndt.step_generators = sg
    sys.modules['numdifftools'] = ndt
    sys.modules['numdifftools.step_generators'] = sg
    np.trapz = np.trapezoid
    np.NaN = np.nan
    import scipy.integrate as igt
    igt.cumtrapz = igt.cumulative_trapezoid


_install_shims()
sys.path.insert(0, REF)
import gwfast.gwfastGlobals as glob          # noqa: E402
import gwfast.waveforms as WF                 # noqa: E402
import gwfast.signal as SIG                   # noqa: E402
import gwfast.network as NET                  # noqa: E402
import time                                   # noqa: E402

WF.time = time   # gwfast/waveforms.py:3316 times the xi_tide tabulation without importing time

# IMRPhenomNSBH tabulates xi_tide on its 200^3 grid with gwfast's own routine (8 million np.roots
# calls, minutes) when xiTide_Table_200.h5 is absent, as here; the result is kept in /tmp between runs
_XI_CACHE = '/tmp/gwf_xitide_200.npz'
_tabulate = WF.IMRPhenomNSBH._tabulate_xiTide


def _tabulate_cached(self, res=200, store=True, Compmin=.1, qmax=100.):
    if res == 200 and Compmin == .1 and qmax == 100. and os.path.exists(_XI_CACHE):
        z = np.load(_XI_CACHE)
        return z['xi'], z['C'], z['q'], z['chi']
    out = _tabulate(self, res=res, store=False, Compmin=Compmin, qmax=qmax)
    if res == 200:
        np.savez(_XI_CACHE, xi=out[0], C=out[1], q=out[2], chi=out[3])
    return out


WF.IMRPhenomNSBH._tabulate_xiTide = _tabulate_cached


def _init_no_jit(self):
    self._SignalDerivatives_use = self._SignalDerivatives


SIG.GWSignal._init_jax = _init_no_jit


def aligo_psd(f):
    x = f / 215.
    return 1e-49 * (x ** -4.14 - 5. * x ** -2 + 111. * (1. - x * x + 0.5 * x ** 4) / (1. + 0.5 * x * x))


def psd_file(fwall, n=2000):
    f = np.geomspace(fwall, 1e4, n)
    path = os.path.join('/tmp', 'gwf_psd_%g.txt' % fwall)
    np.savetxt(path, np.stack([f, aligo_psd(f)], 1))
    return path


def events_bns(rng, n):
    m = np.sort(rng.uniform(1.1, 2.0, (n, 2)), axis=1)[:, ::-1]
    m1, m2 = m[:, 0], m[:, 1]
    Mc = (m1 * m2) ** 0.6 / (m1 + m2) ** 0.2
    eta = m1 * m2 / (m1 + m2) ** 2
    return _angles(rng, n, dict(Mc=Mc, eta=eta, chi1z=rng.uniform(-.05, .05, n), chi2z=rng.uniform(-.05, .05, n),
                                dL=rng.uniform(0.05, 0.5, n)))


def events_bbh(rng, n, mmax=80., qmin=0.2, chimax=0.8):
    u = rng.uniform(0, 1, n)
    a = -2.3 + 1.
    m1 = (5. ** a + u * (mmax ** a - 5. ** a)) ** (1. / a)
    q = rng.uniform(qmin, 1., n)
    m2 = q * m1
    Mc = (m1 * m2) ** 0.6 / (m1 + m2) ** 0.2
    eta = m1 * m2 / (m1 + m2) ** 2
    return _angles(rng, n, dict(Mc=Mc, eta=eta, chi1z=rng.uniform(-chimax, chimax, n),
                                chi2z=rng.uniform(-chimax, chimax, n), dL=rng.uniform(0.5, 10., n)))


def _angles(rng, n, ev):
    ev.update(theta=np.arccos(rng.uniform(-1, 1, n)), phi=rng.uniform(0, 2 * np.pi, n),
              iota=np.arccos(rng.uniform(-1, 1, n)), psi=rng.uniform(0, np.pi, n),
              tcoal=rng.uniform(0, 1, n), Phicoal=rng.uniform(0, 2 * np.pi, n))
    return ev


KEYS = ('Mc', 'eta', 'dL', 'theta', 'phi', 'iota', 'psi', 'tcoal', 'Phicoal', 'chi1z', 'chi2z')


def make_case(name, wf, dets, events, res, fisher=True):
    out = {'res': np.array(res)}
    for k in (KEYS + (('Lambda1', 'Lambda2', 'LambdaTilde', 'deltaLambda') if wf.is_tidal else ())
              + (('ecc',) if wf.is_eccentric else ())):
        out['ev_' + k] = np.asarray(events[k], dtype=np.float64)
    sigs = {}
    for dname, (fwall, earth) in dets.items():
        d = glob.detectors[dname]
        sigs[dname] = SIG.GWSignal(wf, psd_path=psd_file(fwall), detector_shape=d['shape'], det_lat=d['lat'],
                                   det_long=d['long'], det_xax=d['xax'], verbose=False, is_ASD=False,
                                   useEarthMotion=earth, fmin=fwall)
    net = NET.DetNet(sigs, verbose=False)
    ev = {k: np.array(v) for k, v in events.items()}
    snrs = net.SNR(dict(ev), res=res, return_all=True)
    for k, v in snrs.items():
        out['snr_' + k] = np.asarray(v)
    # waveform pieces on the first detector's grid
    d0 = list(sigs.values())[0]
    fc = wf.fcut(**ev)
    fg = np.geomspace(np.full(fc.shape, d0.fmin), fc, num=res)
    out['fgrid'] = fg
    out['tau_star'] = wf.tau_star(fg, **ev)
    out['fcut'] = fc
    if wf.is_HigherModes:
        hp, hc = wf.hphc(fg, **ev)
        out['hp'], out['hc'] = hp, hc
    else:
        out['Phi'] = wf.Phi(fg, **ev)
        out['Ampl'] = wf.Ampl(fg, **ev)
    for dname, s in sigs.items():
        rots = (0.,) if s.detector_shape == 'L' else (0., 60.)
        fc_d = fc if s.fmax is None else np.minimum(fc, s.fmax)
        fgd = np.geomspace(np.full(fc_d.shape, s.fmin), fc_d, num=res)
        for r in rots:
            tag = '%s_r%d' % (dname, int(r))
            args = [fgd] + [ev[k] for k in ('Mc', 'eta', 'dL', 'theta', 'phi', 'iota', 'psi', 'tcoal', 'Phicoal',
                                             'chi1z', 'chi2z')]
            z = np.zeros_like(ev['Mc'])
            lt = ev['LambdaTilde'] if wf.is_tidal else z
            dl = ev['deltaLambda'] if wf.is_tidal else z
            ec = ev['ecc'] if wf.is_eccentric else z
            h = s.GWstrain(*args, z, z, z, z, lt, dl, ec, rot=r, is_chi1chi2=True)
            out['strain_' + tag] = h
            der = s._AnalyticalDerivatives(*args, z, z, z, z, lt, dl, ec, rot=r, use_chi1chi2=True)
            for nm, dv in zip(('dL', 'theta', 'phi', 'iota', 'psi', 'tcoal', 'Phicoal'), der):
                if dv is not None:
                    out['dana_%s_%s' % (nm, tag)] = np.asarray(dv)
    if fisher:
        Fs = net.FisherMatr(dict(ev), res=res, return_all=True)
        for k, v in Fs.items():
            out['fisher_' + k] = np.asarray(v)
    np.savez_compressed(os.path.join(OUT, name + '.npz'), **out)
    print('wrote', name, sorted(out.keys())[:6], '...')


def make_gw170817():
    """Known answer of gwfast's tutorial (notebooks/gwfast_tutorial.ipynb, 'COMPLETE EXAMPLE: GW170817'):
    IMRPhenomD_NRTidalv2, L1 + H1 + Virgo with the O2 ASDs shipped in psds/LVC_O1O2O3, fmin 10 Hz,
    no Earth rotation, default resolution; published network SNR 33.16 and, after fixing
    deltaLambda, a 90 % sky area of 19.9 deg^2. The event is the tutorial's as it prints it (dL from
    Planck18 and tcoal from the GPS time need astropy, which is not installed). Stores the ASD
    tables, gwfast's own SNRs, Fisher matrix (finite-difference stand-in for jacrev) and sky area."""
    import gwfast.fisherTools as FT
    import gwfast.gwfastUtils as UT
    base = os.path.join(REF, 'psds', 'LVC_O1O2O3')
    files = {'L1': '2017-08-06_DCH_C02_L1_O2_Sensitivity_strain_asd.txt',
             'H1': '2017-06-10_DCH_C02_H1_O2_Sensitivity_strain_asd.txt',
             'Virgo': 'Hrec_hoft_V1O2Repro2A_16384Hz.txt'}
    ev = {'Mc': np.array([1.1859 * (1. + 0.00980)]), 'dL': np.array([0.04374755]),
          'theta': np.array([np.pi / 2. + 0.4080839999999999]), 'phi': np.array([3.4461599999999994]),
          'iota': np.array([2.545065595974997]), 'psi': np.array([0.]), 'tcoal': np.array([0.43432288]),
          'eta': np.array([0.24786618323504223]), 'Phicoal': np.array([0.]),
          'chi1z': np.array([0.005136138323169717]), 'chi2z': np.array([0.003235146993487445]),
          'Lambda1': np.array([368.17802383555687]), 'Lambda2': np.array([586.5487031450857])}
    out = {'ev_' + k: v for k, v in ev.items()}
    sigs = {}
    for d, fn in files.items():
        path = os.path.join(base, fn)
        tab = np.loadtxt(path, usecols=(0, 1))
        # the frequency columns are uniform grids of binary fractions: stored as (f0, df, n), exactly
        f0, df, n = tab[0, 0], tab[1, 0] - tab[0, 0], tab.shape[0]
        assert np.array_equal(tab[:, 0], f0 + df * np.arange(n))
        out['asd_grid_' + d], out['asd_' + d] = np.array([f0, df, n]), tab[:, 1].copy()
        g = glob.detectors[d]
        sigs[d] = SIG.GWSignal(WF.IMRPhenomD_NRTidalv2(), psd_path=path, detector_shape=g['shape'], det_lat=g['lat'],
                               det_long=g['long'], det_xax=g['xax'], verbose=False, is_ASD=True,
                               useEarthMotion=False, fmin=10.)
    net = NET.DetNet(sigs, verbose=False)
    for k, v in net.SNR(dict(ev), return_all=True).items():
        out['snr_' + k] = np.asarray(v)
    out['snr_net'] = np.asarray(net.SNR(dict(ev)))
    # the amplitude at the grid end, where the taper is 0 or 1 by rounding (same on every detector's grid)
    wf = WF.IMRPhenomD_NRTidalv2()
    evt = dict(ev)
    evt['LambdaTilde'], evt['deltaLambda'] = UT.Lamt_delLam_from_Lam12(ev['Lambda1'], ev['Lambda2'], ev['eta'])
    fc = wf.fcut(**evt)
    fg = np.geomspace(np.full(fc.shape, 10.), fc, num=1000)
    out['ampl_last'] = np.asarray(wf.Ampl(fg, **evt)[-1])
    F = net.FisherMatr(dict(ev))
    out['fisher_net'] = np.asarray(F)
    pn = WF.IMRPhenomD_NRTidalv2().ParNums
    Ff, pf = FT.fixParams(F, pn, ['deltaLambda'])
    cov, _ = FT.CovMatr(Ff)
    # gwfast's CovMatr returns long doubles, whose layout differs between x86 and Arm: store float64
    out['sky_area'] = np.asarray(FT.compute_localization_region(cov, pf, ev['theta']), dtype=np.float64)
    np.savez_compressed(os.path.join(OUT, 'kat_gw170817.npz'), **out)
    print('wrote kat_gw170817: SNR %.4f, sky area %.2f deg^2' % (out['snr_net'][0], out['sky_area'][0]))


def make_fishertools_helpers():
    """gwfast's fisherTools change-of-variable and prior helpers on Fisher and covariance matrices of the
    IMRPhenomD golden case (gwfast/fisherTools.py:378-823)."""
    import gwfast.fisherTools as FT
    g = np.load(os.path.join(OUT, 'phd_net_earth.npz'))
    F = np.asarray(g['fisher_L1'], dtype=np.float64)   # (11, 11, N)
    ev = {k: g['ev_' + k] for k in ('Mc', 'eta', 'dL')}
    pn = WF.IMRPhenomD().ParNums
    out = {'F': F, 'ev_Mc': ev['Mc'], 'ev_eta': ev['eta'], 'ev_dL': ev['dL']}
    out['prior'] = FT.addPrior(F, [1e2, 4e3], pn, ['psi', 'iota'])
    out['logdl_fish'] = np.asarray(FT.log_dL_to_dL_derivative_fish(F, pn, ev))
    out['logdl_cov'] = np.asarray(FT.log_dL_to_dL_derivative_cov(F, pn, ev))
    e0 = {k: float(v[0]) for k, v in ev.items()}
    F0 = F[:, :, 0]
    out['m1m2_to_Mceta_fish'] = FT.m1m2_to_Mceta_fish(F0, pn, e0)
    out['m1m2_to_Mceta_cov'] = FT.m1m2_to_Mceta_cov(F0, pn, e0)
    out['Mceta_to_m1m2_fish'] = FT.Mceta_to_m1m2_fish(F0, pn, e0)
    out['Mceta_to_m1m2_cov'] = FT.Mceta_to_m1m2_cov(F0, pn, e0)
    out['chi1chi2_to_chieffDeltachi_fish'] = FT.chi1chi2_to_chieffDeltachi_fish(F0, pn, e0)
    pns = WF.IMRPhenomD(is_chi1chi2=False).ParNums
    out['chiSchiA_to_chi1chi2_fish'] = FT.chiSchiA_to_chi1chi2_fish(F0, pns, e0)
    out['m1m2'] = np.array(FT.m1m2_from_Mceta(e0['Mc'], e0['eta']))
    np.savez_compressed(os.path.join(OUT, 'fishertools_helpers.npz'), **out)
    print('wrote fishertools_helpers')


def make_covariance():
    """fisherTools.CovMatr with its defaults (gwfast/fisherTools.py:32-212: equilibrated Cholesky in
    mpmath, inversion error) and CheckFisher (:216-279, mpmath eigh) on the network Fisher matrices
    of the IMRPhenomD (11 x 11) and IMRPhenomD_NRTidalv2 (13 x 13) golden cases."""
    import gwfast.fisherTools as FT
    out = {}
    for tag, src in (('phd', 'phd_net_earth'), ('nrt', 'nrt_net_earth')):
        g = np.load(os.path.join(OUT, src + '.npz'))
        F = np.asarray(g['fisher_net'], dtype=np.float64)
        cov, eps = FT.CovMatr(F)
        out[tag + '_F'] = F
        out[tag + '_cov'] = np.asarray(cov, dtype=np.float64)
        out[tag + '_eps'] = np.asarray(eps, dtype=np.float64)
        ev_, _, cond = FT.CheckFisher(F)
        out[tag + '_evals'] = np.asarray(ev_, dtype=np.float64)
        out[tag + '_cond'] = np.asarray(cond, dtype=np.float64)
    np.savez_compressed(os.path.join(OUT, 'covariance.npz'), **out)
    print('wrote covariance')


def make_overlap(res=300):
    """WFOverlap (gwfast/signal.py:1759-1921 per detector with return_separate, network.py:198-227 for
    the network): TaylorF2 against IMRPhenomD on the same BNS events, IMRPhenomD against itself with
    shifted masses and spins on BBH events; L1 and the ET triangle with Earth rotation."""
    dets = {'L1': (10., True), 'ETS': (5., True)}
    out = {'res': np.array(res)}
    ev_a = events_bns(np.random.default_rng(1010), 3)
    ev_b = events_bbh(np.random.default_rng(1011), 3)
    ev_b2 = dict(ev_b)
    ev_b2['Mc'] = ev_b['Mc'] * (1. + 2e-4)
    ev_b2['chi1z'] = ev_b['chi1z'] + 0.01
    import gwfast.gwfastUtils as UT
    ev_c = events_bns(np.random.default_rng(1017), 3)
    ev_c['chi1z'], ev_c['chi2z'] = np.array([0.2, -0.1, 0.05]), np.array([-0.15, 0.25, 0.1])
    ev_c['Lambda1'], ev_c['Lambda2'] = np.array([400., 900., 200.]), np.array([700., 300., 1100.])
    ev_c['LambdaTilde'], ev_c['deltaLambda'] = UT.Lamt_delLam_from_Lam12(ev_c['Lambda1'], ev_c['Lambda2'], ev_c['eta'])
    m1, m2 = np.array([6., 9., 12.]), np.array([1.35, 1.5, 1.4])
    ev_d = {'Mc': (m1 * m2) ** 0.6 / (m1 + m2) ** 0.2, 'eta': m1 * m2 / (m1 + m2) ** 2,
            'chi1z': np.array([0.5, -0.2, 0.1]), 'chi2z': np.zeros(3), 'dL': np.array([0.1, 0.2, 0.15])}
    ev_d = _angles(np.random.default_rng(1018), 3, ev_d)
    ev_d['Lambda1'], ev_d['Lambda2'] = np.zeros(3), np.array([1200., 500., 300.])
    ev_d['LambdaTilde'], ev_d['deltaLambda'] = UT.Lamt_delLam_from_Lam12(ev_d['Lambda1'], ev_d['Lambda2'], ev_d['eta'])
    ev_e = events_bbh(np.random.default_rng(1019), 3, mmax=150., qmin=0.1, chimax=0.9)
    cases = (('tf2_phd', WF.TaylorF2_RestrictedPN(), WF.IMRPhenomD(), ev_a, dict(ev_a)),
             ('phd_phd', WF.IMRPhenomD(), WF.IMRPhenomD(), ev_b, ev_b2),
             ('nrt_tf2t', WF.IMRPhenomD_NRTidalv2(), WF.TaylorF2_RestrictedPN(is_tidal=True), ev_c, dict(ev_c)),
             ('nsbh_phd', WF.IMRPhenomNSBH(verbose=False), WF.IMRPhenomD(), ev_d, dict(ev_d)),
             ('phm_phd', WF.IMRPhenomHM(), WF.IMRPhenomD(), ev_e, dict(ev_e)))
    for tag, wf1, wf2, ev1, ev2 in cases:
        for k in KEYS + (('Lambda1', 'Lambda2', 'LambdaTilde', 'deltaLambda') if wf1.is_tidal else ()):
            out['%s_ev1_%s' % (tag, k)] = np.asarray(ev1[k], dtype=np.float64)
            out['%s_ev2_%s' % (tag, k)] = np.asarray(ev2[k], dtype=np.float64)
        sigs = {}
        for dname, (fwall, earth) in dets.items():
            d = glob.detectors[dname]
            sigs[dname] = SIG.GWSignal(wf1, psd_path=psd_file(fwall), detector_shape=d['shape'], det_lat=d['lat'],
                                       det_long=d['long'], det_xax=d['xax'], verbose=False, is_ASD=False,
                                       useEarthMotion=earth, fmin=fwall)
            ov, s1, s2 = sigs[dname].WFOverlap(wf1, wf2, dict(ev1), dict(ev2), res=res, return_separate=True)
            out['%s_%s_ov' % (tag, dname)] = np.asarray(ov)
            out['%s_%s_snr1' % (tag, dname)] = np.asarray(s1)
            out['%s_%s_snr2' % (tag, dname)] = np.asarray(s2)
        net = NET.DetNet(sigs, verbose=False)
        out['%s_net' % tag] = np.asarray(net.WFOverlap(wf1, wf2, dict(ev1), dict(ev2), res=res))
    np.savez_compressed(os.path.join(OUT, 'overlap_net_earth.npz'), **out)
    print('wrote overlap_net_earth')


def make_snr_derivs(res=300):
    """DetNet.FisherMatr(return_SNR_derivatives=True) (gwfast/signal.py:938-945, :1016-1022,
    :1090-1094; network.py:124-145): per arm 4 trapz(Re(h conj(dh/dtheta)) / S, f) and the network sum
    divided by the network SNR, for TaylorF2 on the ET triangle with rotation and Virgo without, and
    tidal eccentric TaylorF2 (14 parameters) on ET. The derivatives are the finite-difference
    stand-in's. gwfast passes its complex128 parameters to GWstrain unchanged on this path, where
    IMRPhenomD calls np.fabs, which numpy refuses for complex input: the IMR models are not run here."""
    import gwfast.gwfastUtils as UT
    out = {'res': np.array(res)}
    evt = events_bns(np.random.default_rng(1015), 3)
    evt['Lambda1'], evt['Lambda2'] = np.array([300., 900., 150.]), np.array([500., 200., 700.])
    evt['LambdaTilde'], evt['deltaLambda'] = UT.Lamt_delLam_from_Lam12(evt['Lambda1'], evt['Lambda2'], evt['eta'])
    evt['ecc'] = np.array([0.02, 0.1, 0.05])
    cases = (('tf2', WF.TaylorF2_RestrictedPN(), {'ETS': (5., True), 'Virgo': (10., False)},
              events_bns(np.random.default_rng(1013), 3)),
             ('tf2te', WF.TaylorF2_RestrictedPN(is_tidal=True, is_eccentric=True), {'ETS': (5., True)}, evt))
    for tag, wf, dets, ev in cases:
        for k in KEYS + (('Lambda1', 'Lambda2', 'LambdaTilde', 'deltaLambda', 'ecc') if wf.is_tidal else ()):
            out['%s_ev_%s' % (tag, k)] = np.asarray(ev[k], dtype=np.float64)
        sigs = {}
        for dname, (fwall, earth) in dets.items():
            d = glob.detectors[dname]
            sigs[dname] = SIG.GWSignal(wf, psd_path=psd_file(fwall), detector_shape=d['shape'], det_lat=d['lat'],
                                       det_long=d['long'], det_xax=d['xax'], verbose=False, is_ASD=False,
                                       useEarthMotion=earth, fmin=fwall)
        net = NET.DetNet(sigs, verbose=False)
        snrs = net.SNR(dict(ev), res=res, return_all=True)
        F, D = net.FisherMatr(dict(ev), res=res, return_SNR_derivatives=True)
        for k in D:
            out['%s_sd_%s' % (tag, k)] = np.asarray(D[k])
            out['%s_fisher_%s' % (tag, k)] = np.asarray(F[k])
        for k, v in snrs.items():
            out['%s_snr_%s' % (tag, k)] = np.asarray(v)
        # the 'net' entry is divided by DetNet.SNR at its default resolution (network.py:139-143
        # passes no res), whatever res the Fisher used
        out['%s_snr_default_res' % tag] = np.asarray(net.SNR(dict(ev)))
    np.savez_compressed(os.path.join(OUT, 'snr_derivs.npz'), **out)
    print('wrote snr_derivs')


def make_derivs(res=200):
    """DetNet.FisherMatr(return_derivatives=True) (gwfast/signal.py:913-916, :938-939, :1057;
    network.py:124-137): per arm the (P, N, R) derivative arrays of the strain on the event grid
    (tcoal row per second), TaylorF2 on the ET triangle with rotation and on Virgo without, and
    tidal eccentric TaylorF2 (14 parameters) on ET. The intrinsic rows (Mc, eta, chi1z, chi2z and the
    tidal and ecc rows) are the finite-difference stand-in's, the others gwfast's closed forms."""
    import gwfast.gwfastUtils as UT
    out = {'res': np.array(res)}
    evt = events_bns(np.random.default_rng(1016), 3)
    evt['Lambda1'], evt['Lambda2'] = np.array([400., 800., 250.]), np.array([600., 300., 900.])
    evt['LambdaTilde'], evt['deltaLambda'] = UT.Lamt_delLam_from_Lam12(evt['Lambda1'], evt['Lambda2'], evt['eta'])
    evt['ecc'] = np.array([0.03, 0.08, 0.12])
    cases = (('', WF.TaylorF2_RestrictedPN(), {'ETS': (5., True), 'Virgo': (10., False)},
              events_bns(np.random.default_rng(1014), 3)),
             ('te_', WF.TaylorF2_RestrictedPN(is_tidal=True, is_eccentric=True), {'ETS': (5., True)}, evt))
    for pre, wf, dets, ev in cases:
        for k in KEYS + (('Lambda1', 'Lambda2', 'LambdaTilde', 'deltaLambda', 'ecc') if wf.is_tidal else ()):
            out[pre + 'ev_' + k] = np.asarray(ev[k], dtype=np.float64)
        sigs = {}
        for dname, (fwall, earth) in dets.items():
            d = glob.detectors[dname]
            sigs[dname] = SIG.GWSignal(wf, psd_path=psd_file(fwall), detector_shape=d['shape'], det_lat=d['lat'],
                                       det_long=d['long'], det_xax=d['xax'], verbose=False, is_ASD=False,
                                       useEarthMotion=earth, fmin=fwall)
        F, D = NET.DetNet(sigs, verbose=False).FisherMatr(dict(ev), res=res, return_derivatives=True)
        for k in D:
            out[pre + 'der_' + k] = np.asarray(D[k])
    np.savez_compressed(os.path.join(OUT, 'derivs_tf2.npz'), **out)
    print('wrote derivs_tf2')


def make_strain_caller(R=64):
    """GWstrain, GWAmplitudes and GWPhase at caller-given frequencies: per event an unsorted set,
    log-uniform from 3 Hz to 1.3 times the model's cut (so the models' reference frequency, the
    lowest of the given points, is not a detector's fmin, and the IMR models' cut is crossed)."""
    out = {}
    cases = (('phd', WF.IMRPhenomD(), {'L1': (10., True), 'ETS': (5., True)}, events_bbh(np.random.default_rng(1010), 3)),
             ('tf2', WF.TaylorF2_RestrictedPN(), {'Virgo': (10., False)}, events_bns(np.random.default_rng(1011), 3)),
             ('phm', WF.IMRPhenomHM(), {'ETS': (5., True)},
              events_bbh(np.random.default_rng(1012), 3, mmax=150., qmin=0.1, chimax=0.9)))
    for tag, wf, dets, ev in cases:
        ev = {k: np.array(v) for k, v in ev.items()}
        rng = np.random.default_rng(len(tag) * 7 + 3)
        fc = wf.fcut(**ev)
        f = np.exp(np.log(3.) + rng.uniform(0., 1., (R, len(fc))) * (np.log(1.3 * fc) - np.log(3.)))
        out[tag + '_f'] = f
        for k in KEYS:
            out['%s_ev_%s' % (tag, k)] = ev[k]
        for dname, (fwall, earth) in dets.items():
            d = glob.detectors[dname]
            s = SIG.GWSignal(wf, psd_path=psd_file(fwall), detector_shape=d['shape'], det_lat=d['lat'],
                             det_long=d['long'], det_xax=d['xax'], verbose=False, is_ASD=False, useEarthMotion=earth,
                             fmin=fwall)
            z = np.zeros_like(ev['Mc'])
            args = [f] + [ev[k] for k in ('Mc', 'eta', 'dL', 'theta', 'phi', 'iota', 'psi', 'tcoal', 'Phicoal',
                                           'chi1z', 'chi2z')]
            for r in ((0.,) if d['shape'] == 'L' else (0., 60., 120.)):
                t = '%s_%s_r%d' % (tag, dname, int(r))
                out[t + '_strain'] = s.GWstrain(*args, z, z, z, z, z, z, z, rot=r, is_chi1chi2=True)
                ap, ac = s.GWAmplitudes(dict(ev), f, rot=r)
                out[t + '_Ap'], out[t + '_Ac'] = np.asarray(ap), np.asarray(ac)
            if not wf.is_HigherModes:
                out[tag + '_GWPhase'] = np.asarray(s.GWPhase(dict(ev), f))
    np.savez_compressed(os.path.join(OUT, 'strain_caller.npz'), **out)
    print('wrote strain_caller', len(out), 'arrays')


def main():
    only = sys.argv[2:]
    if only:   # regenerate only the named parts: make_<part>()
        for part in only:
            globals()['make_' + part]()
        return
    import gwfast.gwfastUtils as UT
    rng = np.random.default_rng(1000)
    make_case('tf2_L_noearth', WF.TaylorF2_RestrictedPN(), {'Virgo': (10., False)}, events_bns(rng, 4), 400)
    rng = np.random.default_rng(1001)
    make_case('tf2_T_earth', WF.TaylorF2_RestrictedPN(use_3p5PN_SpinHO=True), {'ETS': (10., True)},
              events_bns(rng, 3), 300)
    rng = np.random.default_rng(1002)
    make_case('phd_net_earth', WF.IMRPhenomD(), {'L1': (10., True), 'H1': (10., True), 'ETS': (5., True)},
              events_bbh(rng, 4), 300)
    rng = np.random.default_rng(1003)
    make_case('phm_net_earth', WF.IMRPhenomHM(), {'L1': (10., True), 'ETS': (5., True)},
              events_bbh(rng, 3, mmax=150., qmin=0.1, chimax=0.9), 300)
    rng = np.random.default_rng(1004)
    ev = events_bns(rng, 3)
    ev['Lambda1'] = rng.uniform(100., 1000., 3)
    ev['Lambda2'] = rng.uniform(100., 1000., 3)
    ev['LambdaTilde'], ev['deltaLambda'] = UT.Lamt_delLam_from_Lam12(ev['Lambda1'], ev['Lambda2'], ev['eta'])
    make_case('tf2tidal_T_earth', WF.TaylorF2_RestrictedPN(is_tidal=True), {'ETS': (5., True), 'Virgo': (10., True)},
              ev, 300)
    # IMRPhenomD_NRTidalv2: spins up to 0.3 so that the quadrupole-moment terms matter, one event
    # with Lambda < 1 on one star (the polynomial branch of the quadrupole-moment relation)
    rng = np.random.default_rng(1005)
    ev = events_bns(rng, 4)
    ev['chi1z'] = rng.uniform(-.3, .3, 4)
    ev['chi2z'] = rng.uniform(-.3, .3, 4)
    ev['Lambda1'] = np.array([150., 800., 400., 0.6])
    ev['Lambda2'] = np.array([300., 1500., 0.4, 250.])
    ev['LambdaTilde'], ev['deltaLambda'] = UT.Lamt_delLam_from_Lam12(ev['Lambda1'], ev['Lambda2'], ev['eta'])
    _FD['lam_h'] = 2e-2
    make_case('nrt_net_earth', WF.IMRPhenomD_NRTidalv2(), {'L1': (10., True), 'ETS': (5., True)}, ev, 300)
    _FD['lam_h'] = None
    # TaylorF2 options: eccentricity (referenced at each detector's lowest grid frequency, so the two
    # detectors' fmin differ on purpose), then tidal + eccentric with the quadrupole moments, phiref_vlso
    # and fRef_ecc, then the Kerr-ISCO cut with the 3.5PN spin terms
    rng = np.random.default_rng(1006)
    ev = events_bns(rng, 4)
    ev['ecc'] = rng.uniform(0.01, 0.15, 4)
    make_case('tf2ecc_net_earth', WF.TaylorF2_RestrictedPN(is_eccentric=True), {'L1': (10., True), 'ETS': (5., True)},
              ev, 300)
    rng = np.random.default_rng(1007)
    ev = events_bns(rng, 3)
    ev['chi1z'] = rng.uniform(-.3, .3, 3)
    ev['chi2z'] = rng.uniform(-.3, .3, 3)
    ev['ecc'] = rng.uniform(0.01, 0.15, 3)
    ev['Lambda1'] = np.array([300., 900., 0.7])
    ev['Lambda2'] = np.array([500., 200., 400.])
    ev['LambdaTilde'], ev['deltaLambda'] = UT.Lamt_delLam_from_Lam12(ev['Lambda1'], ev['Lambda2'], ev['eta'])
    _FD['lam_h'] = 2e-2
    make_case('tf2tidalecc_opts', WF.TaylorF2_RestrictedPN(is_tidal=True, is_eccentric=True, use_QuadMonTid=True,
                                                           phiref_vlso=True, fRef_ecc=8.),
              {'Virgo': (10., True), 'ETS': (5., True)}, ev, 300)
    _FD['lam_h'] = None
    rng = np.random.default_rng(1008)
    make_case('tf2kerr_T', WF.TaylorF2_RestrictedPN(which_ISCO='Kerr', use_3p5PN_SpinHO=True), {'ETS': (5., True)},
              events_bbh(rng, 4, mmax=40., chimax=0.9), 300)
    # IMRPhenomNSBH: BH 1, NS 2 (Lambda1 = 0); disruptive with a torus, mildly disruptive, non-disruptive,
    # a NS with Lambda < 1 and a fast-spinning BH
    m1 = np.array([5., 8., 15., 6., 10.])
    m2 = np.array([1.4, 1.35, 1.5, 1.6, 1.3])
    ev = {'Mc': (m1 * m2) ** 0.6 / (m1 + m2) ** 0.2, 'eta': m1 * m2 / (m1 + m2) ** 2,
          'chi1z': np.array([0.8, 0.3, 0.0, -0.3, 0.95]), 'chi2z': np.zeros(5), 'dL': np.array([0.1, 0.2, 0.3, 0.15, 0.4])}
    ev = _angles(np.random.default_rng(1009), 5, ev)
    ev['Lambda1'] = np.zeros(5)
    ev['Lambda2'] = np.array([1500., 600., 300., 0.5, 2500.])
    ev['LambdaTilde'], ev['deltaLambda'] = UT.Lamt_delLam_from_Lam12(ev['Lambda1'], ev['Lambda2'], ev['eta'])
    # (smaller Lambda steps: one event lies within 0.1 in deltaLambda of a switch of the merger type)
    _FD['lam_h'] = 2e-3
    make_case('nsbh_net_earth', WF.IMRPhenomNSBH(verbose=False), {'L1': (10., True), 'ETS': (5., True)}, ev, 300)
    _FD['lam_h'] = None
    make_gw170817()
    make_fishertools_helpers()
    make_covariance()
    make_overlap()
    make_snr_derivs()
    make_derivs()
    make_strain_caller()
    # KAT from the reference tutorial: GW170817-like TF2 Schwarzschild cut frequency 1590.1 Hz
    z = 0.00980
    ev = {'Mc': np.array([1.1859 * (1. + z)]), 'eta': np.array([0.24786618323504223])}
    np.savez_compressed(os.path.join(OUT, 'kat_fcut.npz'), fcut=WF.TaylorF2_RestrictedPN().fcut(**ev),
                        Mc=ev['Mc'], eta=ev['eta'])


if __name__ == '__main__':
    main()
