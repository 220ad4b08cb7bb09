"""Pack the Kerr (l=2, m=2, n=0) quasi-normal-mode table used by IMRPhenomD.

IMRPhenomD evaluates the ringdown and damping frequencies of the remnant by
linear interpolation in the final spin on a fixed table (gwfast
``gwfast/waveforms.py:988-990``, ``:1034-1035``; data ``WFfiles/QNMData_*.txt``).
Parity needs exactly that table, so this script packs the three published
columns (spin, ringdown frequency, damping frequency, the latter two in units
of 1/M) into one file, ``qnm_220.txt``.  It only runs where the gwfast sources
are available; the packed file is what the library reads.
"""
import os
import sys

import numpy as np


def main(src_dir):
    cols = [np.loadtxt(os.path.join(src_dir, 'QNMData_%s.txt' % c)) for c in ('a', 'fring', 'fdamp')]
    tab = np.stack(cols, axis=1)
    assert tab.shape[1] == 3 and np.all(np.diff(tab[:, 0]) > 0)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'qnm_220.txt')
    np.savetxt(out, tab, fmt='%.18e', header='spin fring*M fdamp*M (Kerr 220 QNM table used by IMRPhenomD)')
    print('wrote', out, tab.shape)


if __name__ == '__main__':
    if len(sys.argv) != 2:
        sys.exit('usage: python make_qnm_table.py <gwfast checkout>/WFfiles')
    main(sys.argv[1])
