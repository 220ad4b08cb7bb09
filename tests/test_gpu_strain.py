"""GWstrain, GWAmplitudes and GWPhase at caller-given frequencies (gwfast/signal.py:425-655) through
the C ABI (gwf_strain) against the oracle's restatement of the same methods.

Frequencies: an unsorted set per event, log-uniform from 3 Hz to 1.3 times the model's cut (beyond
the IMR models' Mf = 0.2 their amplitudes are zero, as in gwfast), so the models' reference
frequency (the lowest of the event's points, as gwfast takes it) differs from the detector's fmin.

Tolerances: amplitudes relative to the event's largest amplitude <= 1e-10; GWPhase within 1e-6 rad
(2 pi f tcoal reaches ~1e9 rad, whose FP64 rounding differs between the two evaluation orders by
~1e-7 rad); the strain relative to its largest modulus <= 1e-6 (the same phase rounding).
"""
import numpy as np
import pytest

import oracle as O
from gwfast_gb300 import synthetic
from gwfast_gb300 import waveforms as W
from gwfast_gb300.signal import GWSignal

pytestmark = pytest.mark.gpu

MODELS = {'IMRPhenomD': ('PhenomD', synthetic.bbh_events), 'TaylorF2_RestrictedPN': ('TF2', synthetic.bns_events),
          'IMRPhenomHM': ('PhenomHM', synthetic.bbh_events)}


def signal_and_oracle(model, name, fmin, earth):
    spec = synthetic.detector_spec(name, fmin)
    sig = GWSignal(getattr(W, model)(), useEarthMotion=earth, verbose=False, **spec)
    f, S = spec['psd_path']
    od = O.Detector(spec['det_lat'], spec['det_long'], spec['det_xax'], spec['detector_shape'], fmin=fmin, psd_f=f,
                    psd_S=S, earth=earth)
    return sig, od


def caller_freqs(om, p, R, seed):
    fc = om.fcut_of(p).reshape(-1).detach().numpy()
    rng = np.random.default_rng(seed)
    u = rng.random((len(fc), R))
    return np.exp(np.log(3.) + u * (np.log(1.3 * fc) - np.log(3.))[:, None])   # (N, R), unsorted


def strain_args(ev):
    return dict(Mc=ev['Mc'], eta=ev['eta'], dL=ev['dL'], theta=ev['theta'], phi=ev['phi'], iota=ev['iota'],
                psi=ev['psi'], tcoal=ev['tcoal'], Phicoal=ev['Phicoal'], chiS=ev['chi1z'], chiA=ev['chi2z'],
                is_chi1chi2=True)


def rel(a, b):
    """max |a - b| per event over the event's max |b| (events along the last axis)"""
    return np.max(np.abs(a - b).max(axis=0) / np.abs(b).max(axis=0))


@pytest.mark.parametrize('model,name,fmin,earth', [
    ('IMRPhenomD', 'L1', 10., True),
    ('IMRPhenomD', 'ETS', 5., True),
    ('TaylorF2_RestrictedPN', 'Virgo', 10., False),
    ('IMRPhenomHM', 'ETS', 5., True)])
def test_strain_amplitudes_phase(gpu_lib, model, name, fmin, earth):
    oname, maker = MODELS[model]
    ev = maker(5, seed=41)
    sig, od = signal_and_oracle(model, name, fmin, earth)
    om = O.Model(oname)
    p = O.to_params(ev)
    fo = caller_freqs(om, p, 96, seed=42)
    f = np.ascontiguousarray(fo.T)                      # gwfast's grids are (R, N)
    ft = O.torch.as_tensor(fo, dtype=O.DT)
    worst = {}
    for rot in ((0.,) if name != 'ETS' else (0., 60., 120.)):
        h = sig.GWstrain(f, rot=rot, **strain_args(ev))
        ho = O.strain(od, om, ft, p, rot).numpy().T
        Ap, Ac = sig.GWAmplitudes(dict(ev), f, rot=rot)
        Apo, Aco = (x.detach().numpy().T for x in O.amplitudes(od, om, ft, p, rot))
        amax = np.maximum(np.abs(Apo).max(axis=0), np.abs(Aco).max(axis=0))
        worst['h'] = max(worst.get('h', 0.), rel(h, ho))
        worst['A'] = max(worst.get('A', 0.), np.max(np.maximum(np.abs(Ap - Apo).max(axis=0),
                                                               np.abs(Ac - Aco).max(axis=0)) / amax))
    if model != 'IMRPhenomHM':
        ph = sig.GWPhase(dict(ev), f)
        pho = (2. * np.pi * ft * (p['tcoal'] * O.DAY_S) - p['Phicoal'] - om.phase(ft, p)).detach().numpy().T
        worst['phase'] = np.max(np.abs(ph - pho))
        # the strain's own phase: Psi = GWPhase + 2 pi f Delta t_loc, so h = (Ap + i Ac) e^{i Psi}
        psi = sig.GWstrain(f, return_single_comp='Psip', **strain_args(ev))
        Ap0, Ac0 = sig.GWAmplitudes(dict(ev), f)
        h0 = sig.GWstrain(f, **strain_args(ev))
        worst['Psi'] = rel((Ap0 + 1j * Ac0) * np.exp(1j * psi), h0)
    print('%s on %s: %s' % (model, name, ', '.join('%s %.2e' % kv for kv in worst.items())))
    assert worst['h'] < 1e-6
    assert worst['A'] < 1e-10
    if 'phase' in worst:
        assert worst['phase'] < 1e-6
        assert worst['Psi'] < 1e-6


def test_strain_shapes_and_parametrisations(gpu_lib):
    """One event with a shared (R,) frequency array gives (R,) outputs; (chiS, chiA) and (m1, m2)
    inputs give the strain of the equivalent (chi1z, chi2z) and (Mc, eta)."""
    from gwfast_gb300 import gwfastUtils as utils
    ev = synthetic.bbh_events(1, seed=43)
    sig, _ = signal_and_oracle('IMRPhenomD', 'L1', 10., True)
    f = np.geomspace(8., 300., 50)
    args = {k: np.asarray(v)[0] for k, v in strain_args(ev).items() if k != 'is_chi1chi2'}
    h = sig.GWstrain(f, is_chi1chi2=True, **args)
    assert h.shape == (50,) and np.all(np.isfinite(h))
    c1, c2 = args['chiS'], args['chiA']
    hs = sig.GWstrain(f, **dict(args, chiS=0.5 * (c1 + c2), chiA=0.5 * (c1 - c2)))
    assert np.max(np.abs(hs - h)) <= 1e-12 * np.max(np.abs(h))
    m1, m2 = utils.m1m2_from_Mceta(args['Mc'], args['eta'])
    hm = sig.GWstrain(f, is_chi1chi2=True, is_m1m2=True, **dict(args, Mc=m1, eta=m2))
    assert np.max(np.abs(hm - h)) <= 1e-9 * np.max(np.abs(h))
    with pytest.raises(NotImplementedError):
        sig.GWstrain(f, rot=60., is_chi1chi2=True, **args)


@pytest.mark.parametrize('tag,model,dets', [
    ('phd', 'IMRPhenomD', {'L1': (10., True), 'ETS': (5., True)}),
    ('tf2', 'TaylorF2_RestrictedPN', {'Virgo': (10., False)}),
    ('phm', 'IMRPhenomHM', {'ETS': (5., True)})])
def test_strain_against_gwfast_golden(gpu_lib, tag, model, dets):
    """The library against gwfast's own GWstrain, GWAmplitudes and GWPhase at unsorted caller
    frequencies (tests/golden/strain_caller.npz, made by tests/golden/make_golden.py from gwfast 1.1.2):
    strain to 1e-6 of its largest modulus, amplitudes to 1e-10, GWPhase within 1e-6 rad."""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden', 'strain_caller.npz'))
    keys = ('Mc', 'eta', 'dL', 'theta', 'phi', 'iota', 'psi', 'tcoal', 'Phicoal', 'chi1z', 'chi2z')
    ev = {k: g['%s_ev_%s' % (tag, k)] for k in keys}
    f = g[tag + '_f']
    for dn, (fw, earth) in dets.items():
        sig, _ = signal_and_oracle(model, dn, fw, earth)
        for rot in ((0.,) if sig.detector_shape == 'L' else (0., 60., 120.)):
            t = '%s_%s_r%d' % (tag, dn, int(rot))
            h = sig.GWstrain(f, rot=rot, **strain_args(ev))
            Ap, Ac = sig.GWAmplitudes(dict(ev), f, rot=rot)
            eh, ea = rel(h, g[t + '_strain']), max(rel(Ap, g[t + '_Ap']), rel(Ac, g[t + '_Ac']))
            print('%s: strain %.2e, amplitudes %.2e' % (t, eh, ea))
            assert eh < 1e-6
            assert ea < 1e-10
        if tag + '_GWPhase' in g:
            assert np.max(np.abs(sig.GWPhase(dict(ev), f) - g[tag + '_GWPhase'])) < 1e-6
