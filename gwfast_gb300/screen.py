"""Learned SNR screen for the forecast pipeline (a method-level addition; gwfast has no
counterpart).

A small MLP (library kernels, gwf_mlp_*) predicts ln(network SNR) from the event parameters for one
fixed network. It is trained on SNRs from the exact kernel. In a forecast, only events whose
predicted ln SNR lies within `band` of ln(threshold) get the exact SNR; events predicted well above
the band are taken as detected, events predicted well below are skipped, and a random `audit_frac`
of the skipped ones still get the exact SNR, so that missed detections are measured, not assumed.
"""
import numpy as np

from . import _lib
from .signal import event_array, _prep


class SNRScreen:
    def __init__(self, net, hidden=256, layers=4, seed=0, device=0):
        self.net = net
        self.mlp = _lib.MLP(hidden=hidden, layers=layers, seed=seed, device=device)
        self.train_loss = None
        self.res = None

    def fit(self, events, snr=None, res=1000, epochs=30, batch=4096, lr=2e-3, seed=0, snr_precision='fp32',
            res_per_event=None):
        """Train on the events' exact network SNRs (computed here unless given, on res points or on
        the per-event grid lengths res_per_event). Returns the mean squared error in ln SNR over the
        last epoch."""
        p = _prep(events)
        if snr is None:
            snr = self.net.SNR(events, res=res, precision=snr_precision, res_per_event=res_per_event)
        self.res = res
        self.train_loss = self.mlp.train(p, np.log(np.maximum(np.asarray(snr, dtype=np.float64), 1e-30)),
                                         epochs=epochs, batch=batch, lr=lr, seed=seed)
        return self.train_loss

    def predict_ln_snr(self, events):
        return self.mlp.predict(_prep(events))

    def split(self, events, snr_th=12., band=0.3, audit_frac=0.01, seed=0, pred=None):
        """Masks (sure_detected, uncertain, skipped, audit) over the events; audit is a subset of skipped."""
        pred = self.predict_ln_snr(events) if pred is None else pred
        lt = np.log(snr_th)
        sure = pred > lt + band
        skipped = pred < lt - band
        uncertain = ~sure & ~skipped
        rng = np.random.default_rng(seed)
        audit = skipped & (rng.random(len(pred)) < audit_frac)
        return sure, uncertain, skipped, audit


__all__ = ['SNRScreen', 'event_array']
