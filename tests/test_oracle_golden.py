"""The oracle against golden vectors produced by gwfast's own sources (tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest
import torch

import oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
CASES = {
    'tf2_L_noearth': (O.Model('TF2'), {'Virgo': (10., False)}),
    'tf2_T_earth': (O.Model('TF2', spin_ho=True), {'ETS': (10., True)}),
    'phd_net_earth': (O.Model('PhenomD'), {'L1': (10., True), 'H1': (10., True), 'ETS': (5., True)}),
    'phm_net_earth': (O.Model('PhenomHM'), {'L1': (10., True), 'ETS': (5., True)}),
    'tf2tidal_T_earth': (O.Model('TF2', tidal=True), {'ETS': (5., True), 'Virgo': (10., True)}),
    'nrt_net_earth': (O.Model('PhenomD_NRTidalv2'), {'L1': (10., True), 'ETS': (5., True)}),
    'tf2ecc_net_earth': (O.Model('TF2', ecc=True), {'L1': (10., True), 'ETS': (5., True)}),
    'tf2tidalecc_opts': (O.Model('TF2', tidal=True, ecc=True, quadmon=True, vlso=True, fref_ecc=8.),
                         {'Virgo': (10., True), 'ETS': (5., True)}),
    'tf2kerr_T': (O.Model('TF2', spin_ho=True, kerr=True), {'ETS': (5., True)}),
    'nsbh_net_earth': (O.Model('PhenomNSBH'), {'L1': (10., True), 'ETS': (5., True)}),
}


def load(name):
    g = np.load(os.path.join(GOLD, name + '.npz'))
    params = CASES[name][0].params if name in CASES else O.PARAMS
    ev = {k: g['ev_' + k] for k in params}
    if name in CASES and CASES[name][0].name == 'PhenomD_NRTidalv2':
        # every grid of an event ends on the same fcut, where the Planck taper is 1 or 0 by the last
        # bit of M f - 1.2 f_merger: take the reference's outcome from its amplitude there
        CASES[name][0].taper_last = g['Ampl'][-1] != 0.
    return g, O.to_params(ev, params), int(g['res'])


def det_of(name, fw, earth):
    lat, lon, xax, sh = O.DETECTORS[name]
    f = np.geomspace(fw, 1e4, 2000)
    return O.Detector(lat, lon, xax, sh, fmin=fw, psd_f=f, psd_S=O.aligo_psd(f), earth=earth)


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def test_kat_tf2_fcut():
    # gwfast new_features_tutorial: TF2 Schwarzschild cut of the GW170817-like event is 1590.1 Hz
    g = np.load(os.path.join(GOLD, 'kat_fcut.npz'))
    fc = float(O.tf2_fcut(torch.tensor(g['Mc']), torch.tensor(g['eta']))[0])
    assert abs(fc - float(g['fcut'][0])) < 1e-9 * fc
    assert round(fc, 1) == 1590.1


@pytest.mark.parametrize('name', list(CASES))
def test_waveform_values(name):
    model, _ = CASES[name]
    g, p, res = load(name)
    f = torch.as_tensor(g['fgrid'].T.copy())
    assert rel(model.fcut_of(p).reshape(-1), g['fcut']) < 1e-14
    assert rel(O.tau_star(f, p['Mc'], p['eta']), g['tau_star'].T) < 1e-13
    if model.is_hm:
        hp, hc = model.hphc(f, p)
        assert rel(hp.numpy(), g['hp'].T) < 1e-10
        assert rel(hc.numpy(), g['hc'].T) < 1e-10
    else:
        assert rel(model.phase(f, p), g['Phi'].T) < 1e-13
        assert rel(model.ampl(f, p), g['Ampl'].T) < 1e-13


@pytest.mark.parametrize('name', list(CASES))
def test_strain_and_closed_form_derivatives(name):
    """Oracle AD derivatives equal gwfast's closed-form extrinsic derivatives (gwfast/signal.py:1303-1584).

    For the IMR models the last grid point sits at Mf = 0.2 within an ulp of the cut, where the two
    implementations can legitimately disagree on which side of the cut it falls; it is excluded.
    """
    model, dets = CASES[name]
    g, p, res = load(name)
    last = -1 if model.name != 'TF2' else None
    for dn, (fw, earth) in dets.items():
        det = det_of(dn, fw, earth)
        fg, S = O.event_grid(det, model, p, res)
        for rot in det.rots:
            tag = '%s_r%d' % (dn, int(rot))
            h = O.strain(det, model, fg, p, rot).numpy()[:, :last]
            assert rel(h, g['strain_' + tag].T[:, :last]) < 1e-7
            J = O.strain_jacobian(det, model, fg, p, rot)
            for i, nm in enumerate(O.PARAMS):
                k = 'dana_%s_%s' % (nm, tag)
                if k in g:
                    assert rel(J[i].numpy()[:, :last], g[k].T[:, :last]) < 2e-6, (tag, nm)


@pytest.mark.parametrize('name', list(CASES))
def test_snr(name):
    model, dets = CASES[name]
    g, p, res = load(name)
    tol = 1e-12 if not model.is_hm else 1e-10
    for dn, (fw, earth) in dets.items():
        det = det_of(dn, fw, earth)
        arms = O.snr_arms(det, model, p, res)
        if det.shape == 'L':
            assert rel(arms[0], g['snr_' + dn]) < tol
        else:
            for i in range(3):
                assert rel(arms[i], g['snr_%s_%d' % (dn, i)]) < tol


@pytest.mark.parametrize('name', list(CASES))
def test_fisher_against_reference_path(name):
    """Full reference FisherMatr path; its AD derivatives were replaced by 5-point finite differences,
    whose rounding through the 1e8-rad phase limits that golden to ~1e-4 of sqrt(F_aa F_bb)."""
    model, dets = CASES[name]
    g, p, res = load(name)
    for dn, (fw, earth) in dets.items():
        det = det_of(dn, fw, earth)
        Fa = O.fisher_arms(det, model, p, res)
        names = [dn] if det.shape == 'L' else ['%s_%d' % (dn, i) for i in range(3)]
        for nm, F in zip(names, Fa):
            Fr = np.moveaxis(g['fisher_' + nm], -1, 0)
            d = np.sqrt(np.abs(np.einsum('nii->ni', Fr)))
            err = np.abs(F.numpy() - Fr) / (d[:, :, None] * d[:, None, :])
            assert err.max() < 5e-4, (nm, err.max())


@pytest.mark.parametrize('name', ['tf2_L_noearth', 'phd_net_earth'])
def test_identities(name):
    """F_dLdL = (SNR/dL)^2 and F_PhicPhic = SNR^2 for 22-mode models (gwfast_tutorial cell 15)."""
    model, dets = CASES[name]
    g, p, res = load(name)
    dn, (fw, earth) = next(iter(dets.items()))
    det = det_of(dn, fw, earth)
    F = O.fisher(det, model, p, res)
    snr = O.snr(det, model, p, res)
    dL = p['dL'].reshape(-1)
    assert np.allclose(F[:, 2, 2], (snr / dL) ** 2, rtol=1e-12)
    assert np.allclose(F[:, 8, 8], snr ** 2, rtol=1e-12)


def gw170817():
    """The GW170817 example of gwfast's tutorial: event, O2 ASD tables, gwfast's own outputs."""
    g = np.load(os.path.join(GOLD, 'kat_gw170817.npz'))
    ev = {k[3:]: g[k] for k in g.files if k.startswith('ev_')}
    tabs = {}
    for d in ('L1', 'H1', 'Virgo'):
        f0, df, n = g['asd_grid_' + d]
        tabs[d] = (f0 + df * np.arange(int(n)), g['asd_' + d])
    return g, ev, tabs


def test_kat_gw170817_oracle():
    """Network SNR 33.16 and, with deltaLambda fixed, a 90 % sky area of 19.9 deg^2
    (gwfast_tutorial, IMRPhenomD_NRTidalv2, L1 + H1 + Virgo at O2 sensitivity, no Earth rotation).

    The grid ends where M f = 1.2 f_merger, and the taper there is 1 or 0 by rounding: gwfast's SNR
    path evaluates the amplitude with the Lambda1, Lambda2 it was given (for this event that point
    is 1, ``ampl_last``), its Fisher path with the pair recovered from (LambdaTilde, deltaLambda)
    (there it falls to 0). Both branches are checked against the matching output."""
    from gwfast_gb300 import fisherTools as FT
    from gwfast_gb300 import gwfastUtils as U
    from gwfast_gb300 import waveforms as W
    g, ev, tabs = gw170817()
    U.fill_tidal(ev)
    dets = []
    for d, (f, asd) in tabs.items():
        lat, lon, xax, sh = O.DETECTORS[d]
        dets.append(O.Detector(lat, lon, xax, sh, fmin=10., psd_f=f, psd_S=asd * asd, earth=False))
    m_snr = O.Model('PhenomD_NRTidalv2', taper_last=g['ampl_last'] != 0.)
    p = O.to_params(ev, m_snr.params)
    snrs = [float(O.snr(det, m_snr, p, 1000)[0]) for det in dets]
    for d, s in zip(tabs, snrs):
        assert abs(s - float(g['snr_' + d][0])) < 1e-12 * s, d
    net = float(np.sqrt(sum(s * s for s in snrs)))
    assert abs(net - float(g['snr_net'][0])) < 1e-12 * net
    assert round(net, 2) == 33.16
    Fr = g['fisher_net'][..., 0]
    dg = np.sqrt(np.abs(np.diag(Fr)))
    errs, areas = [], []
    for last in (False, True):
        model = O.Model('PhenomD_NRTidalv2', taper_last=np.array([last]))
        F = sum(O.fisher(det, model, p, 1000) for det in dets).numpy()[0]
        errs.append((np.abs(F - Fr) / np.outer(dg, dg)).max())
        Ff, pf = FT.fixParams(F[:, :, None], W.IMRPhenomD_NRTidalv2().ParNums, ['deltaLambda'])
        cov, _ = O.cov_matr_fast(np.moveaxis(Ff, -1, 0))
        areas.append(float(FT.compute_localization_region(np.moveaxis(cov, 0, -1), pf, ev['theta'])[0]))
    # finite-difference golden: ~1e-4 of sqrt(F_aa F_bb), as for the other Fisher goldens
    assert min(errs) < 5e-4, errs
    for a in areas:
        assert abs(a - float(g['sky_area'][0])) < 2e-3 * a
        assert round(a, 1) == 19.9


def _overlap_models(tag, last):
    if tag == 'nrt_tf2t':
        return O.Model('PhenomD_NRTidalv2', taper_last=np.full((1,), last)), O.Model('TF2', tidal=True)
    if tag == 'nsbh_phd':
        return O.Model('PhenomNSBH', cut_last=np.full((1,), last)), O.Model('PhenomD')
    names = {'tf2_phd': ('TF2', 'PhenomD'), 'phd_phd': ('PhenomD', 'PhenomD'), 'phm_phd': ('PhenomHM', 'PhenomD')}[tag]
    return O.Model(names[0]), O.Model(names[1])


@pytest.mark.parametrize('tag', ['tf2_phd', 'phd_phd', 'nrt_tf2t', 'nsbh_phd', 'phm_phd'])
def test_overlap_against_reference(tag):
    """WFOverlap: the oracle's per-detector parts ((h1|h2) and the two SNRs, return_separate=True) and
    the network overlap against gwfast's own (tests/golden/overlap_net_earth.npz): TaylorF2 against
    IMRPhenomD, IMRPhenomD against itself with shifted masses and spins, IMRPhenomD_NRTidalv2 against
    tidal TaylorF2, IMRPhenomNSBH against IMRPhenomD, IMRPhenomHM against IMRPhenomD. With the two
    tidal models the grid ends on a knife edge
    (the Planck taper's end, Mf = 0.2) that the last point falls on either side of by rounding, so
    each event is compared with the oracle taken both ways."""
    g = np.load(os.path.join(GOLD, 'overlap_net_earth.npz'))
    res = int(g['res'])
    lasts = (False, True) if tag in ('nrt_tf2t', 'nsbh_phd') else (None,)
    errs = []
    for last in lasts:
        om1, om2 = _overlap_models(tag, last)
        p1 = O.to_params({k: g['%s_ev1_%s' % (tag, k)] for k in om1.params}, om1.params)
        p2 = O.to_params({k: g['%s_ev2_%s' % (tag, k)] for k in om2.params}, om2.params)
        tot = [0., 0., 0.]
        e = 0.
        for name, fw in (('L1', 10.), ('ETS', 5.)):
            ov, n1, n2 = (x.numpy().reshape(-1) for x in O.overlap_parts(det_of(name, fw, True), om1, p1, om2, p2,
                                                                         res))
            ref = [g['%s_%s_%s' % (tag, name, q)] for q in ('ov', 'snr1', 'snr2')]
            e = np.maximum(e, np.abs(ov - ref[0]) / np.abs(ref[0]).max())
            e = np.maximum(e, np.abs(np.sqrt(n1) / ref[1] - 1.))
            e = np.maximum(e, np.abs(np.sqrt(n2) / ref[2] - 1.))
            tot = [t + x for t, x in zip(tot, (ov, n1, n2))]
        net = tot[0] / np.sqrt(tot[1] * tot[2])
        errs.append(np.maximum(e, np.abs(net - g['%s_net' % tag]) / np.abs(g['%s_net' % tag]).max()))
    assert np.all(np.min(errs, axis=0) < 1e-10), errs


@pytest.mark.parametrize('tag,model,dets', [
    ('tf2', O.Model('TF2'), (('ETS', 5., True), ('Virgo', 10., False))),
    ('tf2te', O.Model('TF2', tidal=True, ecc=True), (('ETS', 5., True),))])
def test_snr_derivatives_against_reference(tag, model, dets):
    """return_SNR_derivatives: the oracle's per-arm 4 trapz(Re(h conj(dh/dtheta)) / S, f) and the
    network sum over the network SNR against gwfast's own (tests/golden/snr_derivs.npz: TaylorF2 on
    ET with rotation and Virgo without; tidal eccentric TaylorF2, 14 parameters, on ET). gwfast's
    derivatives there are the golden generator's finite differences; measured against the
    Cauchy-Schwarz scale sqrt(F_aa) SNR_arm (which bounds |dS_a|) the two agree to ~4e-10, and the
    bound is 1e-8 of it. (Entries that vanish in exact arithmetic, such as the Phicoal row,
    Re(h conj(-i h)) = 0, differ by rounding only.)"""
    g = np.load(os.path.join(GOLD, 'snr_derivs.npz'))
    res = int(g['res'])
    p = O.to_params({k: g['%s_ev_%s' % (tag, k)] for k in model.params}, model.params)
    tot = 0.
    for name, fw, earth in dets:
        arms = O.snr_derivs_arms(det_of(name, fw, earth), model, p, res)
        keys = [name] if len(arms) == 1 else ['%s_%d' % (name, i) for i in range(3)]
        for k, a in zip(keys, arms):
            a = a.numpy()
            ref = g['%s_sd_%s' % (tag, k)]
            assert a.shape == ref.shape == (len(model.params), ref.shape[1]), k
            scale = np.sqrt(np.einsum('iin->in', g['%s_fisher_%s' % (tag, k)])) * g['%s_snr_%s' % (tag, k)][None]
            assert np.all(np.abs(a - ref) <= 1e-8 * scale), k
            tot = tot + a
    # gwfast divides the network entry by DetNet.SNR at its default resolution (1000 points), not at
    # the Fisher's res
    snr_def = g[tag + '_snr_default_res']
    odets = [det_of(n, fw, e) for n, fw, e in dets]
    assert rel(O.network_snr(odets, model, p, 1000).numpy(), snr_def) < 1e-12
    net = tot / snr_def
    scale = np.sqrt(np.einsum('iin->in', g[tag + '_fisher_net']))
    assert np.all(np.abs(net - g[tag + '_sd_net']) <= 1e-8 * scale)


@pytest.mark.parametrize('pre,model,dets', [
    ('', O.Model('TF2'), (('ETS', 5., True), ('Virgo', 10., False))),
    ('te_', O.Model('TF2', tidal=True, ecc=True), (('ETS', 5., True),))], ids=['tf2', 'tf2_tidal_ecc'])
def test_strain_derivative_arrays_against_reference(pre, model, dets):
    """return_derivatives: the oracle's per-arm (P, N, R) derivative arrays (tcoal row per second,
    triangle arms 0, 60 degrees and minus their sum) against gwfast's own (tests/golden/derivs_tf2.npz:
    TaylorF2 on ET with rotation and Virgo without; tidal eccentric TaylorF2, 14 parameters, on ET).
    Per (arm, parameter, event) row, relative to the row's maximum: the closed-form rows agree to
    ~1e-8 (bound 3e-7); the intrinsic rows are the generator's finite differences, ~1e-5 at worst
    (bound 5e-5), deltaLambda's (a step of 10) ~6e-5 (bound 2e-4)."""
    g = np.load(os.path.join(GOLD, 'derivs_tf2.npz'))
    res = int(g['res'])
    p = O.to_params({k: g[pre + 'ev_' + k] for k in model.params}, model.params)
    P = len(model.params)
    tol = np.full(P, 3e-7)
    tol[[0, 1, 9, 10]] = 5e-5   # Mc, eta, chi1z, chi2z
    tol[11:] = 5e-5             # LambdaTilde, deltaLambda, ecc
    if model.tidal:
        tol[12] = 2e-4
    for name, fw, earth in dets:
        arms = O.strain_derivs_arms(det_of(name, fw, earth), model, p, res)
        keys = [name] if len(arms) == 1 else ['%s_%d' % (name, i) for i in range(3)]
        for k, a in zip(keys, arms):
            r = g[pre + 'der_' + k]
            assert a.shape == r.shape and r.shape[0] == P, k
            e = np.abs(a.numpy() - r).max(axis=2) / np.abs(r).max(axis=2)
            assert np.all(e.max(axis=1) < tol), (k, e.max(axis=1))


@pytest.mark.parametrize('tag', ['phd', 'nrt'])
def test_covariance_against_reference(tag):
    """fisherTools.CovMatr with its defaults (mpmath equilibrated Cholesky) on the IMRPhenomD
    (11 x 11) and IMRPhenomD_NRTidalv2 (13 x 13) network Fishers of the golden cases: the oracle's
    float64 equilibrated Cholesky inverse gives the same marginalised errors within
    max(1e-9, 1e-14 cond) (measured: at most 2e-17 cond; cond 2e7 to 2e11 here)."""
    g = np.load(os.path.join(GOLD, 'covariance.npz'))
    F = np.moveaxis(g[tag + '_F'], -1, 0)
    cov, _ = O.cov_matr_fast(F)
    s = np.sqrt(np.einsum('nii->ni', cov))
    sr = np.sqrt(np.einsum('iin->ni', g[tag + '_cov']))
    d = 1. / np.sqrt(np.einsum('nii->ni', F))
    w = np.linalg.eigvalsh(F * d[:, :, None] * d[:, None, :])
    cond = w[:, -1] / w[:, 0]
    err = (np.abs(s - sr) / sr).max(axis=1)
    assert np.all(err < np.maximum(1e-9, 1e-14 * cond)), (err, cond)
    # the full matrices too, entry by entry against sqrt(C_aa C_bb)
    cr = np.moveaxis(g[tag + '_cov'], -1, 0)
    e2 = (np.abs(cov - cr) / (sr[:, :, None] * sr[:, None, :])).max(axis=(1, 2))
    assert np.all(e2 < np.maximum(1e-9, 1e-14 * cond)), (e2, cond)


@pytest.mark.parametrize('tag,model,dets', [
    ('phd', 'PhenomD', {'L1': (10., True), 'ETS': (5., True)}),
    ('tf2', 'TF2', {'Virgo': (10., False)}),
    ('phm', 'PhenomHM', {'ETS': (5., True)})])
def test_strain_at_caller_frequencies(tag, model, dets):
    """GWstrain, GWAmplitudes and GWPhase of gwfast at unsorted caller frequencies up to 1.3 times the
    model's cut (tests/golden/make_golden.py, make_strain_caller) against the oracle: the models'
    reference frequency is the lowest of each event's points. Strain to 1e-7 of its largest modulus (the
    2 pi f tcoal term reaches ~1e9 rad, rounded differently in the two), amplitudes to 1e-10, GWPhase
    within 1e-6 rad."""
    g = np.load(os.path.join(GOLD, 'strain_caller.npz'))
    ev = {k: g['%s_ev_%s' % (tag, k)] for k in O.PARAMS}
    p = O.to_params(ev)
    om = O.Model(model)
    f = torch.as_tensor(np.ascontiguousarray(g[tag + '_f'].T), dtype=O.DT)   # (N, R)
    for dn, (fw, earth) in dets.items():
        det = det_of(dn, fw, earth)
        for rot in ((0.,) if det.shape == 'L' else (0., 60., 120.)):
            t = '%s_%s_r%d' % (tag, dn, int(rot))
            h = O.strain(det, om, f, p, rot).numpy().T
            assert rel(h, g[t + '_strain']) < 1e-7, t
            ap, ac = (x.detach().numpy().T for x in O.amplitudes(det, om, f, p, rot))
            assert rel(ap, g[t + '_Ap']) < 1e-10 and rel(ac, g[t + '_Ac']) < 1e-10, t
    if tag + '_GWPhase' in g:
        ph = (2. * np.pi * f * (p['tcoal'] * O.DAY_S) - p['Phicoal'] - om.phase(f, p)).detach().numpy().T
        assert np.max(np.abs(ph - g[tag + '_GWPhase'])) < 1e-6
