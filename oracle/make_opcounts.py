"""Count the algorithmic floating-point work per frequency point (test/bench infrastructure).

Runs the oracle's value path (waveform, tau_star, pattern functions, delay) under a torch
function mode that adds the number of output elements of every arithmetic or
transcendental call (each +, -, *, /, pow, exp, log, sin, cos, atan, sqrt ... counts 1
per element).  Per-point work is isolated by evaluating R = 1000 and R = 2000 points
and differencing, so per-event set-up cancels.

Fisher work per (event, arm, point) = 5 x waveform (value + 4 forward tangents over
Mc, eta, chi1z, chi2z) + projection + 264 (66-entry Gram update) + 4 (trapezoid weight
and 1/S), following the cost model stated for the benchmark roofline.  SNR work per
(event, arm, point) = waveform + projection + 4.

Writes profiles/opcounts.json.  Run:  python oracle/make_opcounts.py
"""
import json
import os
import sys

import numpy as np
import torch
from torch.overrides import TorchFunctionMode

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import oracle as O  # noqa: E402

COUNTED = {'add', 'sub', 'mul', 'div', 'true_divide', 'pow', 'exp', 'log', 'sin', 'cos', 'atan', 'sqrt', 'neg',
           'abs', 'where', 'rsub', 'radd', 'rmul', 'rtruediv', 'rpow', '__add__', '__sub__', '__mul__',
           '__truediv__', '__pow__', '__radd__', '__rsub__', '__rmul__', '__rtruediv__', '__rpow__', '__neg__',
           'cbrt', 'square', 'reciprocal', 'atan2', 'log10', 'exp2', 'expm1', 'log1p', 'sinh', 'cosh'}


class Counter(TorchFunctionMode):
    def __init__(self):
        super().__init__()
        self.n = 0

    def __torch_function__(self, func, types, args=(), kwargs=None):
        out = func(*args, **(kwargs or {}))
        name = getattr(func, '__name__', '')
        if name in COUNTED and isinstance(out, torch.Tensor):
            self.n += out.numel()
        return out


def count(fn):
    c = Counter()
    with c:
        fn()
    return c.n


def per_point(model, earth, det):
    ev = {'Mc': np.array([25.]), 'eta': np.array([0.22]), 'dL': np.array([2.]), 'theta': np.array([1.]),
          'phi': np.array([2.]), 'iota': np.array([0.7]), 'psi': np.array([0.3]), 'tcoal': np.array([0.4]),
          'Phicoal': np.array([1.1]), 'chi1z': np.array([0.3]), 'chi2z': np.array([-0.2])}
    if model.name == 'TF2':
        ev['Mc'], ev['eta'] = np.array([1.2]), np.array([0.2485])
    p = O.to_params(ev)
    out = {}
    for R in (1000, 2000):
        f, _ = O.event_grid(det, model, p, R)

        def wave():
            if model.is_hm:
                model.hphc(f, p)
            else:
                model.ampl(f, p)
                model.phase(f, p)

        def proj():
            if earth:
                O.tau_star(f, p['Mc'], p['eta'])
            t = p['tcoal'] + 0. * f
            dl = O.delt_loc(det, p['theta'], p['phi'], t)
            O.pattern(det, p['theta'], p['phi'], t + dl / O.DAY_S, p['psi'], 0.)
        out[R] = (count(wave), count(proj))
    w = (out[2000][0] - out[1000][0]) / 1000.
    pr = (out[2000][1] - out[1000][1]) / 1000.
    return w, pr


def main():
    lat, lon, xax, sh = O.DETECTORS['L1']
    fr = np.geomspace(5., 1e4, 2000)
    res = {}
    for name, model in (('TaylorF2_RestrictedPN', O.Model('TF2')), ('IMRPhenomD', O.Model('PhenomD')),
                        ('IMRPhenomHM', O.Model('PhenomHM'))):
        for earth in (False, True):
            det = O.Detector(lat, lon, xax, sh, fmin=10., psd_f=fr, psd_S=O.aligo_psd(fr), earth=earth)
            w, pr = per_point(model, earth, det)
            key = '%s/%s' % (name, 'earth' if earth else 'fixed')
            res[key] = {'waveform_value': w, 'projection': pr,
                        'fisher_per_arm_point': 5. * w + pr + 264. + 4.,
                        'snr_per_arm_point': w + pr + 4.}
    path = os.path.join(os.path.dirname(HERE), 'profiles', 'opcounts.json')
    with open(path, 'w') as fh:
        json.dump({'units': 'flop per (event, arm, frequency point)', 'source': 'oracle/make_opcounts.py',
                   'counts': res}, fh, indent=1)
    print(json.dumps(res, indent=1))


if __name__ == '__main__':
    main()
