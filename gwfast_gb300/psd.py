"""Analytic aLIGO noise fit used by the synthetic workloads.

S(f) = 1e-49 [x^-4.14 - 5 x^-2 + 111 (1 - x^2 + x^4/2) / (1 + x^2/2)], x = f / 215 Hz,
tabulated on log-spaced rows from the detector's low-frequency wall to 10 kHz.  Through
gwfast's np.interp(..., left=1, right=1) convention (gwfast/signal.py:723) a PSD of 1
below the first row makes everything under the wall negligible.
"""
import numpy as np


def aligo_psd(f):
    x = np.asarray(f, dtype=np.float64) / 215.
    return 1e-49 * (x ** -4.14 - 5. * x ** -2 + 111. * (1. - x * x + 0.5 * x ** 4) / (1. + 0.5 * x * x))


def aligo_table(fwall, fmax=1e4, rows=20000):
    f = np.geomspace(fwall, fmax, rows)
    return f, aligo_psd(f)
