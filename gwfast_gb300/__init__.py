"""GB300-native Fisher-forecast hot path with gwfast's events-dict API.

Submodules mirror gwfast's: ``signal.GWSignal``, ``network.DetNet``,
``waveforms.{TaylorF2_RestrictedPN, IMRPhenomD, IMRPhenomHM}``,
``fisherTools.CovMatr``, ``gwfastGlobals``, ``gwfastUtils``.
"""
__version__ = '0.1.0'

from . import gwfastGlobals, gwfastUtils, psd, waveforms  # noqa: F401


def __getattr__(name):
    if name in ('signal', 'network', 'fisherTools', 'synthetic'):
        import importlib
        return importlib.import_module('.' + name, __name__)
    raise AttributeError(name)
