"""Host-side logic that needs no GPU: parameter handling, reparametrisation, duty cycle, sharding."""
import os

import numpy as np
import pytest
import torch

import oracle as O
from gwfast_gb300 import gwfastUtils as U
from gwfast_gb300 import shard, synthetic
from gwfast_gb300.signal import GWSignal, event_array, reparametrise


def test_event_array_order_and_broadcast():
    ev = synthetic.bbh_events(5, seed=1)
    ev['tcoal'] = 0.25
    p = event_array(ev)
    assert p.shape == (11, 5) and p.flags.c_contiguous
    assert np.all(p[7] == 0.25)
    assert np.all(p[0] == ev['Mc']) and np.all(p[10] == ev['chi2z'])


def test_check_evparams_mutates_and_raises():
    ev = {'m1': np.array([30.]), 'm2': np.array([20.]), 'ra': np.array([1.]), 'dec': np.array([0.2]),
          'thetaJN': np.array([0.4]), 'tcoal': np.array([0.1])}
    U.check_evparams(ev)
    Mc, eta = U.Mceta_from_m1m2(30., 20.)
    assert np.isclose(ev['Mc'][0], Mc) and np.isclose(ev['eta'][0], eta)
    assert np.isclose(ev['theta'][0], np.pi / 2 - 0.2) and ev['iota'][0] == 0.4
    with pytest.raises(ValueError):
        U.check_evparams({'Mc': 1.})
    with pytest.raises(ValueError):
        U.fill_spins({})
    e2 = {'chiS': np.array([0.1]), 'chiA': np.array([0.05])}
    U.fill_spins(e2)
    assert np.isclose(e2['chi1z'][0], 0.15) and np.isclose(e2['chi2z'][0], 0.05)


def test_tcoal_from_tgps():
    """tcoal (GMST, fraction of a day) from tGPS, as gwfast/gwfastUtils.py:972-981 fills it.

    Known answer: gwfast's tutorial event GW170817 (tGPS 1187008882.4) carries the GMST that gwfast's
    astropy conversion printed, 0.43432288 (stored in tests/golden/kat_gw170817.npz). This conversion
    evaluates the same IAU 2006 formula with UTC for UT1, so it may differ by |UT1 - UTC| <= 0.9 s,
    i.e. 1.05e-5 of a day (it differs by 0.34 s here). J2000.0 (2000-01-01 12:00 UTC): GMST
    18.697374558 h (the published IAU 1982 value; IAU 2006 differs by < 1e-6 h). gwfast's linear
    approximation GPSt_to_GMST_alt ignores leap seconds and precession and stays within 3 s over
    2001-2036."""
    kat = np.load(os.path.join(os.path.dirname(__file__), 'golden', 'kat_gw170817.npz'))
    t = np.array([1187008882.4])
    g = U.GPSt_to_LMST(t, lat=0., long=0.)
    assert abs(g[0] - kat['ev_tcoal'][0]) <= 0.9 / 86400. + 1e-8
    assert abs(U.GPSt_to_GMST(630763213.) * 24. - 18.697374558) < 1e-6 * 24.
    ts = np.linspace(1.0e9, 1.8e9, 101)
    d = (U.GPSt_to_GMST(ts) - U.GPSt_to_GMST_alt(ts) + 0.5) % 1.0 - 0.5
    assert np.max(np.abs(d)) * 86400. < 3.0
    assert np.allclose(U.GPSt_to_LMST(t, 40., 90.), (g + 0.25) % 1.0)
    assert U.leap_seconds(1187008882.4) == 18 and U.leap_seconds(1.0e8) == 2
    ev = {'Mc': np.array([1.2]), 'eta': np.array([0.25]), 'theta': np.array([1.]), 'phi': np.array([2.]),
          'iota': np.array([0.5]), 'tGPS': t}
    U.check_evparams(ev)
    assert ev['tcoal'][0] == g[0]


def test_mass_conversions_roundtrip():
    m1, m2 = U.m1m2_from_Mceta(*U.Mceta_from_m1m2(np.array([35.]), np.array([12.])))
    assert np.allclose([m1[0], m2[0]], [35., 12.])


def _oracle_jacobian_new(det, model, f, p, kind):
    """d h / d(m1, m2) or d(chiS, chiA) by forward AD through the conversion (independent of reparametrise)."""
    out = []
    if kind == 'm1m2':
        m1, m2 = U.m1m2_from_Mceta(p['Mc'].numpy(), p['eta'].numpy())
        m1, m2 = torch.tensor(m1), torch.tensor(m2)
        for j in range(2):
            def fn(x, j=j):
                a, b = (x, m2) if j == 0 else (m1, x)
                q = dict(p)
                q['Mc'] = (a * b) ** 0.6 / (a + b) ** 0.2
                q['eta'] = a * b / (a + b) ** 2
                return O.strain_parts(det, model, f, q)
            prim = (m1 if j == 0 else m2,)
            _, (re, im) = torch.func.jvp(fn, prim, (torch.ones_like(prim[0]),))
            out.append(torch.complex(re, im))
    else:
        cs, ca = 0.5 * (p['chi1z'] + p['chi2z']), 0.5 * (p['chi1z'] - p['chi2z'])
        for j in range(2):
            def fn(x, j=j):
                s, a = (x, ca) if j == 0 else (cs, x)
                q = dict(p)
                q['chi1z'], q['chi2z'] = s + a, s - a
                return O.strain_parts(det, model, f, q)
            prim = (cs if j == 0 else ca,)
            _, (re, im) = torch.func.jvp(fn, prim, (torch.ones_like(prim[0]),))
            out.append(torch.complex(re, im))
    return out


@pytest.mark.parametrize('kind', ['m1m2', 'chiSchiA'])
def test_reparametrise_matches_direct_derivatives(kind):
    ev = synthetic.bbh_events(3, seed=4)
    p = O.to_params(ev)
    f0 = np.geomspace(10., 1e4, 500)
    det = O.Detector(30.563, -90.774, 242.7, 'L', fmin=10., psd_f=f0, psd_S=O.aligo_psd(f0), earth=False)
    model = O.Model('PhenomD')
    f, S = O.event_grid(det, model, p, 300)
    D = O.strain_jacobian(det, model, f, p)
    D[O.TC_INDEX] /= O.DAY_S
    F = O._gram(D, S, f).numpy()
    Fr = reparametrise(F, ev, use_m1m2=(kind == 'm1m2'), use_chi1chi2=(kind == 'm1m2'))
    new = _oracle_jacobian_new(det, model, f, p, kind)
    idx = (0, 1) if kind == 'm1m2' else (9, 10)
    D2 = D.clone()
    D2[idx[0]], D2[idx[1]] = new
    Fd = O._gram(D2, S, f).numpy()
    d = np.sqrt(np.abs(np.einsum('nii->ni', Fd)))
    assert (np.abs(Fr - Fd) / (d[:, :, None] * d[:, None, :])).max() < 1e-10


def test_duty_factor_draws_follow_reference_sequence():
    """Masks are drawn after np.random.seed(seedUse), one choice([0,1], N) per arm (gwfast/signal.py:729-765)."""
    s = GWSignal.__new__(GWSignal)
    s.DutyFactor = 0.7
    s.seedUse = np.array([12345])
    arms = np.ones((3, 50))
    got = s._apply_duty(arms)
    np.random.seed(s.seedUse)
    want = np.stack([np.random.choice([0, 1], 50, p=[0.3, 0.7]) for _ in range(3)])
    assert np.array_equal(got, want)
    F = np.ones((1, 50, 11, 11))
    gotF = s._apply_duty(F)
    np.random.seed(s.seedUse)
    m = np.random.choice([0, 1], 50, p=[0.3, 0.7])
    assert np.array_equal(gotF[0, :, 0, 0], m)


def test_synthetic_catalogues_are_seeded_and_in_range():
    a, b = synthetic.bbh_events(1000, seed=1001), synthetic.bbh_events(1000, seed=1001)
    assert all(np.array_equal(a[k], b[k]) for k in a)
    m1, m2 = U.m1m2_from_Mceta(a['Mc'], a['eta'])
    assert m1.min() >= 5. - 1e-9 and m1.max() <= 80. + 1e-9
    assert np.all(m2 / m1 >= 0.2 - 1e-9) and np.all(a['eta'] <= 0.25)
    bn = synthetic.bns_events(200, seed=1000)
    m1, m2 = U.m1m2_from_Mceta(bn['Mc'], bn['eta'])
    assert np.all(m1 >= m2 - 1e-12) and m2.min() >= 1.1 - 1e-9 and m1.max() <= 2.0 + 1e-9


def test_shard_slices_cover_everything():
    for n in (0, 1, 7, 10, 1001):
        for w in (1, 2, 3, 8):
            sl = [shard.shard_slice(n, r, w) for r in range(w)]
            assert sl[0][0] == 0 and sl[-1][1] == n
            assert all(sl[i][1] == sl[i + 1][0] for i in range(w - 1))
            assert max(b - a for a, b in sl) - min(b - a for a, b in sl) <= 1


def test_fix_params_and_sky_area():
    from gwfast_gb300 import fisherTools
    rng = np.random.default_rng(3)
    A = rng.standard_normal((5, 11, 11))
    F = np.moveaxis(A @ np.swapaxes(A, 1, 2) + 11 * np.eye(11), 0, -1)
    pn = {'Mc': 0, 'eta': 1, 'dL': 2, 'theta': 3, 'phi': 4, 'iota': 5, 'psi': 6, 'tcoal': 7, 'Phicoal': 8,
          'chi1z': 9, 'chi2z': 10}
    Fr, pr = fisherTools.fixParams(F, pn, ['psi', 'Phicoal'])
    assert Fr.shape == (9, 9, 5)
    assert pr == {'Mc': 0, 'eta': 1, 'dL': 2, 'theta': 3, 'phi': 4, 'iota': 5, 'tcoal': 6, 'chi1z': 7, 'chi2z': 8}
    keep = [0, 1, 2, 3, 4, 5, 7, 9, 10]
    assert np.array_equal(Fr, F[np.ix_(keep, keep)])
    # sky area from a diagonal (theta, phi) block: 2 pi sqrt(det) |sin theta| (-ln 0.1) sr
    C = np.zeros((11, 11, 1))
    C[3, 3], C[4, 4] = 1e-4, 4e-4
    a = fisherTools.compute_localization_region(C, pn, np.array([np.pi / 2]), units='Sterad')
    assert np.isclose(a[0], 2 * np.pi * 2e-4 * np.log(10.))


def test_mlp_oracle_gradient_matches_finite_differences():
    """The CPU model's analytic backward pass against central differences (weights kept exactly
    representable in bfloat16 so the rounding does not move under the perturbation)."""
    from oracle import mlp_oracle as M
    rng = np.random.default_rng(5)
    hidden, layers = 8, 2
    n_w = 11 * 8 + 8 * 8 + 8 + 8 + 8 + 1
    w = M.bf16(rng.normal(0., 0.3, n_w).astype(np.float32))
    p = np.stack([rng.uniform(5, 50, 20), rng.uniform(0.1, 0.25, 20), rng.uniform(0.5, 10, 20),
                  rng.uniform(0, np.pi, 20), rng.uniform(0, 2 * np.pi, 20), rng.uniform(0, np.pi, 20),
                  rng.uniform(0, np.pi, 20), rng.uniform(0, 1, 20), rng.uniform(0, 2 * np.pi, 20),
                  rng.uniform(-.5, .5, 20), rng.uniform(-.5, .5, 20)])
    norm = np.concatenate([np.zeros(11), np.ones(11)])
    t = rng.normal(2., 1., 20)
    loss, g = M.forward_backward(w, norm, p, t, hidden, layers)
    # biases are not rounded: check them by central differences
    Ws, _ = M.unpack(w, hidden, layers)
    nW = sum(W.size for W in Ws)
    for i in range(nW, n_w):
        d = np.zeros(n_w)
        d[i] = 1e-6
        fd = (M.forward_backward(w + d, norm, p, t, hidden, layers)[0]
              - M.forward_backward(w - d, norm, p, t, hidden, layers)[0]) / 2e-6
        assert abs(fd - g[i]) < 1e-6 * max(1., abs(g[i]))


def test_tidal_parameters_and_descriptor():
    """LambdaTilde/deltaLambda from Lambda1/Lambda2 and back (gwfast/gwfastUtils.py:398-446); the tidal
    TaylorF2 descriptor has 13 parameters and model id 3."""
    from gwfast_gb300 import gwfastUtils as U
    from gwfast_gb300 import waveforms as W
    rng = np.random.default_rng(3)
    eta = rng.uniform(0.2, 0.25, 50)
    l1, l2 = rng.uniform(0., 3000., 50), rng.uniform(0., 3000., 50)
    lt, dl = U.Lamt_delLam_from_Lam12(l1, l2, eta)
    r1, r2 = U.Lam12_from_Lamt_delLam(lt, dl, eta)
    np.testing.assert_allclose(r1, l1, rtol=1e-9, atol=1e-8)
    np.testing.assert_allclose(r2, l2, rtol=1e-9, atol=1e-8)
    # equal masses, equal deformabilities: LambdaTilde = Lambda, deltaLambda = 0
    lt0, dl0 = U.Lamt_delLam_from_Lam12(np.array([400.]), np.array([400.]), np.array([0.25]))
    np.testing.assert_allclose(lt0, 400., rtol=1e-14)
    np.testing.assert_allclose(dl0, 0., atol=1e-12)
    wf = W.TaylorF2_RestrictedPN(is_tidal=True)
    assert wf.nParams == 13 and wf.params[-2:] == ('LambdaTilde', 'deltaLambda')
    assert wf.gpu_desc().model == 3 and wf.objType == 'BNS'
    ev = {'Mc': np.array([1.2]), 'eta': np.array([0.24])}
    with pytest.raises(ValueError):
        U.fill_tidal(ev)
    with pytest.raises(NotImplementedError):
        W.IMRPhenomD(is_tidal=True)


def test_fishertools_helpers_against_gwfast():
    """Priors, log(dL) and mass/spin changes of variables against gwfast's own fisherTools
    (tests/golden/make_golden.py: make_fishertools_helpers)."""
    import os
    from gwfast_gb300 import fisherTools as FT
    from gwfast_gb300 import waveforms as W
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden', 'fishertools_helpers.npz'))
    F = g['F']
    ev = {'Mc': g['ev_Mc'], 'eta': g['ev_eta'], 'dL': g['ev_dL']}
    pn = W.IMRPhenomD().ParNums
    close = lambda a, b: np.testing.assert_allclose(a, b, rtol=1e-13, atol=0)
    close(FT.addPrior(F, [1e2, 4e3], pn, ['psi', 'iota']), g['prior'])
    close(FT.log_dL_to_dL_derivative_fish(F, pn, ev), g['logdl_fish'])
    close(FT.log_dL_to_dL_derivative_cov(F, pn, ev), g['logdl_cov'])
    e0 = {k: float(v[0]) for k, v in ev.items()}
    F0 = F[:, :, 0]
    for name in ('m1m2_to_Mceta_fish', 'm1m2_to_Mceta_cov', 'Mceta_to_m1m2_fish', 'Mceta_to_m1m2_cov',
                 'chi1chi2_to_chieffDeltachi_fish'):
        close(getattr(FT, name)(F0, pn, e0), g[name])
    close(FT.chiSchiA_to_chi1chi2_fish(F0, W.IMRPhenomD(is_chi1chi2=False).ParNums, e0), g['chiSchiA_to_chi1chi2_fish'])
    close(np.array(FT.m1m2_from_Mceta(e0['Mc'], e0['eta'])), g['m1m2'])
    Mc, eta = FT.Mceta_from_m1m2(*g['m1m2'])
    close(np.array([Mc, eta]), np.array([e0['Mc'], e0['eta']]))


def test_check_fisher_against_gwfast(capsys):
    """fisherTools.CheckFisher against gwfast's own (mpmath eigh, tests/golden/covariance.npz): the
    eigenvalues agree to 1e-14 of the largest; the condition numbers, whose smallest eigenvalue is
    only as good as 1e-16 of the largest, within 1e-15 cond for the IMRPhenomD matrices (cond up to
    1e12; the 13 x 13 ones sit at 1e16, at the rounding floor, where gwfast itself reports negative
    eigenvalues, as does this one). An all-NaN matrix gives NaN rows, as there."""
    import os
    from gwfast_gb300 import fisherTools as FT
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden', 'covariance.npz'))
    for tag in ('phd', 'nrt'):
        ev, vec, cond = FT.CheckFisher(g[tag + '_F'])
        er = g[tag + '_evals']
        assert ev.shape == er.shape and vec.shape == (ev.shape[0],) + ev.shape[1:] * 2
        assert np.all(np.abs(ev - er).max(axis=1) <= 1e-14 * np.abs(er).max(axis=1)), tag
        if tag == 'phd':
            assert np.all(np.abs(cond / g['phd_cond'] - 1.) <= 1e-15 * g['phd_cond'])
    F = g['phd_F'].copy()
    F[:, :, 1] = np.nan
    ev, vec, cond = FT.CheckFisher(F, verbose=True)
    assert np.all(np.isnan(ev[1])) and np.all(np.isnan(vec[1])) and np.isnan(cond[1])
    assert np.all(np.isfinite(cond[[0, 2, 3]]))
    assert 'Fisher is nan at position 1' in capsys.readouterr().out


def test_batch_files_roundtrip(tmp_path):
    """Per-batch output files of the catalogue driver under gwfast's names and shapes, read back."""
    from gwfast_gb300 import pipeline
    rng = np.random.default_rng(3)
    det = np.array([True, False, True, True])
    F = rng.normal(size=(11, 11, 3))
    out = {'snr': rng.uniform(5, 20, 4), 'detected': det, 'fisher': F, 'cov': F * 2, 'eps': rng.uniform(size=3),
           'cond': rng.uniform(size=3), 'cond_numbers': rng.uniform(size=3), 'errors': rng.uniform(size=(11, 3)),
           'sky_area_90': rng.uniform(size=3)}
    pipeline.batch_to_file(out, 40, str(tmp_path))
    back = pipeline.batch_from_file(str(tmp_path), 40, 44)
    assert np.allclose(back['snrs'], out['snr']) and np.array_equal(back['fishers'], F)
    assert np.array_equal(back['idxs_det'].astype(int), [40, 42, 43])
    assert back['errors'].shape == (11, 3) and np.allclose(back['cond_numbers'], out['cond_numbers'])
    none = dict(out, detected=np.zeros(4, bool), fisher=None)
    pipeline.batch_to_file(none, 0, str(tmp_path))
    assert set(pipeline.batch_from_file(str(tmp_path), 0, 4)) == {'snrs'}


def test_f32_rounding_matches_casts(tmp_path):
    """The integer FP64 -> FP32 rounding of the FP32 record set-up (gwfast_gb300/csrc/gwf_f32conv.cuh,
    compiled here as host C++) gives the bit patterns of the casts it replaces on 12 M values: random
    bit patterns, normal values across and beyond the FP32 range, round-to-nearest-even ties and
    near-ties, mantissa carries into the exponent, and the special values."""
    import shutil
    import subprocess
    gxx = shutil.which('g++')
    if gxx is None:
        pytest.skip('g++ not found')
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    exe = str(tmp_path / 'f32conv_check')
    subprocess.run([gxx, '-O2', '-std=c++17', '-I', os.path.join(root, 'gwfast_gb300', 'csrc'),
                    os.path.join(root, 'tests', 'f32conv_check.cpp'), '-o', exe], check=True)
    r = subprocess.run([exe, '4000000'], capture_output=True, text=True)
    print(r.stdout)
    assert r.returncode == 0, r.stdout
