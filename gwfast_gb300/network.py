"""DetNet: a network of GWSignal detectors (gwfast/network.py:17-343).

All detectors of the network are evaluated in one library call (one fused kernel
launch per detector on one stream), and the network Fisher is accumulated on the
device.
"""
import numpy as np

from . import gwfastUtils as utils
from .signal import (fisher_batch, overlap_batch, reparametrise, reparametrise_derivs, reparametrise_vec, snr_batch,
                     strain_derivs_batch)


class DetNet:
    """gwfast/network.py:17-31."""

    def __init__(self, signals, verbose=True):
        self.signals = signals
        self.verbose = verbose

    def _list(self):
        return list(self.signals.keys()), list(self.signals.values())

    def _update_all_seeds(self, seeds=[], verbose=True):
        if seeds == []:
            seeds = [None for _ in self.signals]
        for i, d in enumerate(self.signals):
            self.signals[d]._update_seed(seed=seeds[i])

    def SNR(self, evParams, res=1000, return_all=False, precision='fp64', res_per_event=None):
        """Network SNR (gwfast/network.py:53-82); precision='fp32' selects the FP32 SNR kernel."""
        utils.check_evparams(evParams)
        names, sigs = self._list()
        arms = snr_batch(sigs, evParams, res, device=sigs[0].device, precision=precision, res_per_event=res_per_event)
        snrs = {}
        for name, s, a in zip(names, sigs, arms):
            if s.detector_shape == 'T' and return_all:
                for i in range(3):
                    snrs['%s_%s' % (name, i)] = a[i]
            elif s.detector_shape == 'T':
                snrs[name] = np.sqrt((a ** 2).sum(axis=0))
            else:
                snrs[name] = a[0]
        net = np.sqrt(np.array([snrs[k] ** 2 for k in snrs]).sum(axis=0))
        if return_all:
            snrs['net'] = net
            return snrs
        return net

    def FisherMatr(self, evParams, return_all=False, return_derivatives=False, return_SNR_derivatives=False, **kwargs):
        """Network Fisher matrix, (11, 11, N) (gwfast/network.py:84-153).

        return_SNR_derivatives=True returns (allF, allDer) as gwfast: per-arm Fisher matrices and
        per-arm SNR-derivative integrals (11, N) keyed by detector (name_0..2 for triangles), plus
        'net': the Fisher total and dSNR/dtheta = sum of the integrals / network SNR (SNRs from
        kwargs['SNRs'] if given, else DetNet.SNR at its default resolution of 1000 points whatever
        res the Fisher uses, as gwfast/network.py:139-143 calls it)."""
        utils.check_evparams(evParams)
        names, sigs = self._list()
        res = kwargs.get('res', 1000)
        if res is None:
            res = max(s._resolve_res(evParams, None, kwargs.get('df')) for s in sigs)
        spacing = kwargs.get('spacing', 'geom')
        use_m1m2 = kwargs.get('use_m1m2', False)
        use_chi1chi2 = kwargs.get('use_chi1chi2', True)
        if kwargs.get('computeDerivFinDiff', False):
            raise NotImplementedError('finite-difference derivatives are not used on the GPU path')
        precision = kwargs.get('precision', 'fp64')
        if return_derivatives and not return_SNR_derivatives:
            # gwfast/network.py:126-137: per-arm Fisher matrices plus 'net', per-arm (P, N, R) derivatives
            allF, allDer = {}, {}
            for name, s in zip(names, sigs):
                Fa, Da = s.FisherMatr(evParams, res=res, spacing=spacing, use_m1m2=use_m1m2, use_chi1chi2=use_chi1chi2,
                                      return_derivatives=True, precision=precision,
                                      refine_cond=kwargs.get('refine_cond'))
                keys = ['%s_%s' % (name, i) for i in range(3)] if s.detector_shape == 'T' else [name]
                for i, k in enumerate(keys):
                    allF[k] = Fa[i]
                    allDer[k] = Da[i]
            allF['net'] = np.array([allF[k] for k in allF]).sum(axis=0)
            return allF, allDer
        if return_SNR_derivatives:
            per, der = fisher_batch(sigs, evParams, res, per_arm=True, spacing=spacing, device=sigs[0].device,
                                    precision=precision, refine_cond=kwargs.get('refine_cond'),
                                    res_per_event=kwargs.get('res_per_event'), snr_derivs=True)
            allF, allDer = {}, {}
            for name, s, Fa, Da in zip(names, sigs, per, der):
                Fa = reparametrise(Fa, evParams, use_m1m2, use_chi1chi2)
                Da = reparametrise_vec(Da, evParams, use_m1m2, use_chi1chi2)
                keys = ['%s_%s' % (name, i) for i in range(3)] if s.detector_shape == 'T' else [name]
                for i, k in enumerate(keys):
                    allF[k] = np.moveaxis(Fa[i], 0, -1)
                    allDer[k] = np.moveaxis(Da[i], 0, -1)
            snrs = kwargs['SNRs'] if 'SNRs' in kwargs else self.SNR(evParams, precision='fp64' if precision == 'fp64'
                                                                    else 'fp32')
            allF['net'] = np.array([allF[k] for k in allF]).sum(axis=0)
            allDer['net'] = np.array([allDer[k] for k in allDer]).sum(axis=0) / snrs
            return allF, allDer
        if not return_all:
            F = fisher_batch(sigs, evParams, res, per_arm=False, spacing=spacing, device=sigs[0].device,
                             precision=precision, refine_cond=kwargs.get('refine_cond'),
                             res_per_event=kwargs.get('res_per_event'))
            F = reparametrise(F, evParams, use_m1m2, use_chi1chi2)
            return np.moveaxis(F, 0, -1)
        per = fisher_batch(sigs, evParams, res, per_arm=True, spacing=spacing, device=sigs[0].device,
                           precision=precision, refine_cond=kwargs.get('refine_cond'),
                           res_per_event=kwargs.get('res_per_event'))
        allF = {}
        for name, s, Fa in zip(names, sigs, per):
            Fa = reparametrise(Fa, evParams, use_m1m2, use_chi1chi2)
            if s.detector_shape == 'T':
                for i in range(3):
                    allF['%s_%s' % (name, i)] = np.moveaxis(Fa[i], 0, -1)
            else:
                allF[name] = np.moveaxis(Fa[0], 0, -1)
        allF['net'] = np.array([allF[k] for k in allF]).sum(axis=0)
        return allF

    def WFOverlap(self, WF1, WF2, evParams1, evParams2, res=1000, **kwargs):
        """Network overlap of two waveforms on two parameter sets (gwfast/network.py:198-227):
        sum_d (h1|h2)_d / sqrt(sum_d SNR1_d^2 sum_d SNR2_d^2)."""
        names, sigs = self._list()
        ov, n1, n2 = overlap_batch(sigs, WF1, WF2, evParams1, evParams2, res)
        return ov.sum(axis=0) / np.sqrt(n1.sum(axis=0) * n2.sum(axis=0))
