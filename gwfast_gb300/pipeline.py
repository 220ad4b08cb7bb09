"""Batch forecast: SNR of every event, detection threshold, network Fisher matrices of the
detected events, CheckFisher, covariances, 1-sigma errors and sky areas, the core of gwfast's
catalogue driver (compute_errs, run/calculate_forecasts_from_catalog.py:410-635) on the GPU path,
and the driver's loop over batches with per-batch output files and resume (:224-290, :700-770).

Not reproduced from the driver: duty factors applied after the fact (set DutyFactor on the
GWSignal objects instead), derivative outputs and the h5 catalogue I/O (h5py is not a dependency of
this package; catalogues come in as the events dict).
"""
import os
import time

import numpy as np

from . import fisherTools
from .gwfastUtils import check_evparams


def _subset(events, mask):
    return {k: (np.asarray(v)[mask] if np.ndim(v) else v) for k, v in events.items()}


def compute_errs(net, events, snr_th=12., res=1000, precision='mixed', snr_precision='fp32', params_fix=(),
                 refine_cond=None, res_per_event=None, sky_area=True, timings=None, screen=None, band=0.3,
                 audit_frac=0.01, audit_seed=0, check_fisher=False):
    """Forecast for one batch of events.

    net: DetNet; events: the gwfast events dict (completed in place like gwfast does).
    precision: Fisher form ('fp64', 'fp32' or 'mixed'); snr_precision: SNR form ('fp64' or 'fp32').
    Returns a dict: snr (N,), detected (N,) bool, fisher / cov (P, P, N_det), eps, cond and
    errors (P, N_det) (sqrt of the covariance diagonal), sky_area_90 (N_det,) in deg^2 and the
    parameter numbering par_nums. timings, if a dict, receives the wall time of each stage.
    check_fisher: also run fisherTools.CheckFisher on the Fisher matrices of the detected events, as
    the driver does before the inversion (:604): out['cond_numbers'] are its condition numbers of the
    matrices as they are (the driver's output), out['cond'] those of the equilibrated matrices.

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
    if check_fisher:
        _, _, out['cond_numbers'] = fisherTools.CheckFisher(F, use_mpmath=True)
    cov, eps, cond = fisherTools.CovMatr(F, return_cond=True, device=sigs[0].device)
    t3 = time.perf_counter()
    out.update(fisher=F, cov=cov, eps=eps, cond=cond, errors=np.sqrt(np.abs(np.einsum('iin->in', cov))))
    out['sky_area_90'] = (fisherTools.compute_localization_region(cov, par_nums, np.asarray(det['theta']))
                          if sky_area and 'theta' in par_nums and 'phi' in par_nums else None)
    if timings is not None:
        timings.update(snr=t1 - t0, fisher=t2 - t1, cov=t3 - t2, total=time.perf_counter() - t0)
    return out


_BATCH_FILES = ('snrs', 'fishers', 'covs', 'sky_area', 'errors', 'inversion_errors', 'cond_numbers', 'idxs_det')


def _suffix(i_in, i_f):
    return '_%d_to_%d' % (i_in, i_f)


def batch_to_file(out, i_in, out_path):
    """One batch's outputs under the names and formats of the driver's to_file
    (run/calculate_forecasts_from_catalog.py:224-247): snrs (all events) as text; fishers and covs
    (P, P, N_det) as .npy; sky areas, errors (P, N_det), inversion errors, condition numbers and the
    global indices of the detected events as text. Without detected events only the SNRs are written,
    as the driver does."""
    n = len(np.atleast_1d(out['snr']))
    suff = _suffix(i_in, i_in + n)
    np.savetxt(os.path.join(out_path, 'snrs' + suff + '.txt'), np.atleast_1d(out['snr']))
    if out['fisher'] is None:
        return
    idxs = np.arange(i_in, i_in + n)[np.argwhere(out['detected'])]
    sky = out['sky_area_90'] if out['sky_area_90'] is not None else np.full(out['fisher'].shape[-1], np.nan)
    cond = out['cond_numbers'] if out.get('cond_numbers') is not None else out['cond']
    np.save(os.path.join(out_path, 'fishers' + suff + '.npy'), out['fisher'])
    np.save(os.path.join(out_path, 'covs' + suff + '.npy'), out['cov'])
    np.savetxt(os.path.join(out_path, 'sky_area' + suff + '.txt'), np.atleast_1d(sky))
    np.savetxt(os.path.join(out_path, 'errors' + suff + '.txt'), out['errors'])
    np.savetxt(os.path.join(out_path, 'inversion_errors' + suff + '.txt'), np.atleast_1d(out['eps']))
    np.savetxt(os.path.join(out_path, 'cond_numbers' + suff + '.txt'), np.atleast_1d(cond))
    np.savetxt(os.path.join(out_path, 'idxs_det' + suff + '.txt'), idxs)


def batch_from_file(out_path, i_in, i_f):
    """Read one batch back (run/calculate_forecasts_from_catalog.py:250-290): a dict with snrs and, when
    the batch had detections, fishers, covs, sky_area, errors (P, N_det), inversion_errors,
    cond_numbers and idxs_det, single-event batches given their array dimensions back."""
    suff = _suffix(i_in, i_f)
    res = {'snrs': np.atleast_1d(np.loadtxt(os.path.join(out_path, 'snrs' + suff + '.txt')))}
    if not os.path.exists(os.path.join(out_path, 'fishers' + suff + '.npy')):
        return res
    res['fishers'] = np.load(os.path.join(out_path, 'fishers' + suff + '.npy'))
    res['covs'] = np.load(os.path.join(out_path, 'covs' + suff + '.npy'))
    for k in ('sky_area', 'inversion_errors', 'cond_numbers', 'idxs_det'):
        res[k] = np.atleast_1d(np.loadtxt(os.path.join(out_path, k + suff + '.txt')))
    err = np.loadtxt(os.path.join(out_path, 'errors' + suff + '.txt'))
    res['errors'] = err[:, np.newaxis] if np.ndim(err) == 1 else err
    return res


def run_catalogue(net, events, out_path, batch_size=10000, resume=True, idx_in=0, **kwargs):
    """The catalogue driver's loop (run/calculate_forecasts_from_catalog.py:700-770) on one GPU: the
    events in consecutive batches of batch_size, each through compute_errs (CheckFisher on) and written
    with batch_to_file under the suffix _<first>_to_<last> (global indices from idx_in); with resume, a
    batch whose SNR file already exists is skipped (:738-741), so an interrupted run continues where it
    stopped. Returns the concatenation of all batches as read back from the files: snrs (N,), and over
    the detected events fishers and covs (P, P, N_det), errors (P, N_det), sky_area, inversion_errors,
    cond_numbers and idxs_det. kwargs go to compute_errs."""
    os.makedirs(out_path, exist_ok=True)
    n = len(np.atleast_1d(np.asarray(events[next(iter(events))])))
    kwargs.setdefault('check_fisher', True)
    rpe = kwargs.pop('res_per_event', None)
    bounds = [(i, min(i + batch_size, n)) for i in range(0, n, batch_size)]
    for a, b in bounds:
        if resume and os.path.exists(os.path.join(out_path, 'snrs' + _suffix(idx_in + a, idx_in + b) + '.txt')):
            continue
        ev = _subset(events, slice(a, b))
        out = compute_errs(net, ev, res_per_event=None if rpe is None else np.asarray(rpe)[a:b], **kwargs)
        batch_to_file(out, idx_in + a, out_path)
    parts = [batch_from_file(out_path, idx_in + a, idx_in + b) for a, b in bounds]
    tot = {'snrs': np.concatenate([p['snrs'] for p in parts])}
    det = [p for p in parts if 'fishers' in p]
    if det:
        tot['fishers'] = np.concatenate([p['fishers'] for p in det], axis=-1)
        tot['covs'] = np.concatenate([p['covs'] for p in det], axis=-1)
        tot['errors'] = np.concatenate([p['errors'] for p in det], axis=-1)
        for k in ('sky_area', 'inversion_errors', 'cond_numbers', 'idxs_det'):
            tot[k] = np.concatenate([p[k] for p in det])
    return tot
