"""Batch forecast: SNR of every event, detection threshold, network Fisher matrices of the
detected events, covariances, 1-sigma errors and sky areas, the core of gwfast's catalogue driver
(compute_errs, gwfast/run/calculate_forecasts_from_catalog.py:410-635) on the GPU path.

Not reproduced from the driver: duty factors applied after the fact (set DutyFactor on the
GWSignal objects instead), derivative outputs and the h5 catalogue I/O.
"""
import time

import numpy as np

from . import fisherTools
from .gwfastUtils import check_evparams


def _subset(events, mask):
    return {k: (np.asarray(v)[mask] if np.ndim(v) else v) for k, v in events.items()}


def compute_errs(net, events, snr_th=12., res=1000, precision='mixed', snr_precision='fp32', params_fix=(),
                 refine_cond=None, res_per_event=None, sky_area=True, timings=None, screen=None, band=0.3,
                 audit_frac=0.01, audit_seed=0):
    """Forecast for one batch of events.

    net: DetNet; events: the gwfast events dict (completed in place like gwfast does).
    precision: Fisher form ('fp64', 'fp32' or 'mixed'); snr_precision: SNR form ('fp64' or 'fp32').
    Returns a dict: snr (N,), detected (N,) bool, fisher / cov (P, P, N_det), eps, cond and
    errors (P, N_det) (sqrt of the covariance diagonal), sky_area_90 (N_det,) in deg^2 and the
    parameter numbering par_nums. timings, if a dict, receives the wall time of each stage.

    screen: an SNRScreen trained for this network. Then only the events whose predicted ln SNR is
    within `band` of ln(snr_th), plus a random `audit_frac` of those predicted below the band, get
    the exact SNR; those predicted above the band count as detected (their 'snr' entry is the
    prediction). out['screen'] reports the fractions and the audit: events of the audit sample
    with exact SNR above the threshold are missed detections.
    """
    t0 = time.perf_counter()
    check_evparams(events)
    screen_info = None
    if screen is None:
        snr = net.SNR(events, res=res, precision=snr_precision, res_per_event=res_per_event)
        detected = np.atleast_1d(snr > snr_th)
    else:
        pred = screen.predict_ln_snr(events)
        sure, uncertain, skipped, audit = screen.split(events, snr_th, band, audit_frac, audit_seed, pred=pred)
        exact = uncertain | audit
        snr = np.exp(pred)
        if exact.any():
            rex = None if res_per_event is None else np.asarray(res_per_event)[exact]
            snr[exact] = net.SNR(_subset(events, exact), res=res, precision=snr_precision, res_per_event=rex)
        detected = sure | (exact & (snr > snr_th))   # audit events above threshold are kept (and counted as missed)
        missed = int(np.sum(audit & (snr > snr_th)))
        screen_info = {'sure_detected': float(sure.mean()), 'uncertain': float(uncertain.mean()),
                       'skipped': float(skipped.mean()), 'exact_snr_fraction': float(exact.mean()),
                       'audit_events': int(audit.sum()), 'audit_missed_detections': missed}
    t1 = time.perf_counter()
    detected = np.atleast_1d(detected)
    det = _subset(events, detected)
    rdet = None if res_per_event is None else np.asarray(res_per_event)[detected]
    sigs = list(net.signals.values())
    par_nums = dict(sigs[0].wf_model.ParNums)
    out = {'snr': snr, 'detected': detected, 'par_nums': par_nums, 'screen': screen_info}
    if not detected.any():
        out.update(fisher=None, cov=None, eps=None, cond=None, errors=None, sky_area_90=None)
        return out
    F = net.FisherMatr(det, res=res, precision=precision, refine_cond=refine_cond, res_per_event=rdet)
    t2 = time.perf_counter()
    if params_fix:
        F, par_nums = fisherTools.fixParams(F, par_nums, list(params_fix))
        out['par_nums'] = par_nums
    cov, eps, cond = fisherTools.CovMatr(F, return_cond=True, device=sigs[0].device)
    t3 = time.perf_counter()
    out.update(fisher=F, cov=cov, eps=eps, cond=cond, errors=np.sqrt(np.abs(np.einsum('iin->in', cov))))
    out['sky_area_90'] = (fisherTools.compute_localization_region(cov, par_nums, np.asarray(det['theta']))
                          if sky_area and 'theta' in par_nums and 'phi' in par_nums else None)
    if timings is not None:
        timings.update(snr=t1 - t0, fisher=t2 - t1, cov=t3 - t2, total=time.perf_counter() - t0)
    return out
