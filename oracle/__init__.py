"""CPU float64 oracle for the gwfast Fisher-forecast hot path.

TEST INFRASTRUCTURE ONLY.  This package restates, in plain torch float64 on the
CPU, the reference algorithm (gwfast 1.1.2: ``gwfast/waveforms.py``,
``gwfast/signal.py``, ``gwfast/network.py``, ``gwfast/fisherTools.py``).  It is
the checker: only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` may import it.  The product (``gwfast_gb300``) never routes
through it.

Parity pinning: ``tests/golden/make_golden.py`` runs the reference's own
Python sources (with a numpy stand-in for ``jax.numpy``) on seeded events and
stores their outputs; ``tests/test_oracle_golden.py`` checks this oracle
against those fixtures.
"""
from .gwf_oracle import *  # noqa: F401,F403
from .gwf_oracle import _gram, _trapz  # noqa: F401,E402
