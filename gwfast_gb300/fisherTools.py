"""Fisher-matrix inversion and checks (gwfast/fisherTools.py:32-279).

CovMatr runs the equilibrated Cholesky inversion as one batched FP64 CUDA kernel
(one thread per event) instead of gwfast's per-event mpmath loop.
"""
import numpy as np

from . import _lib


def CovMatr(FisherMatrix, invMethodIn='cho', condNumbMax=1e50, truncate=False, svals_thresh=1e-15, verbose=False,
            alt_method='svd', device=0, return_cond=False):
    """Covariance matrices (P, P, N) and inversion errors (N,) (gwfast/fisherTools.py:32-196).

    Only the default 'cho' method (with the SVD-equivalent fallback for matrices that
    are not positive definite) is implemented.
    """
    if invMethodIn != 'cho':
        raise NotImplementedError("only invMethodIn='cho' is implemented on the GPU path")
    if truncate:
        raise NotImplementedError('singular-value truncation is not implemented on the GPU path')
    F = np.ascontiguousarray(np.moveaxis(np.asarray(FisherMatrix, dtype=np.float64), -1, 0))
    P = F.shape[1]
    if F.shape[1:] != (P, P) or P > 14:
        raise NotImplementedError('the GPU inversion handles up to 14x14 matrices')
    K = 11 if P <= 11 else (13 if P <= 13 else 14)   # the kernel sizes (11, 13 tidal, 14 tidal eccentric)
    if P < K:
        # block-diagonal embedding with an identity block (e.g. after fixParams): the inverse of
        # the leading block is the leading block of the inverse; an equilibrated matrix has
        # eigenvalues on both sides of 1, so the condition number is unchanged, and the identity
        # block adds no inversion error
        Fp = np.broadcast_to(np.eye(K), (F.shape[0], K, K)).copy()
        Fp[:, :P, :P] = F
        F = Fp
    N = F.shape[0]
    cov = np.empty_like(F)
    eps = np.empty(N)
    cond = np.empty(N)
    _lib.context(device).cov(F, cov=cov, eps=eps, cond=cond, n_params=K)
    out = np.moveaxis(np.ascontiguousarray(cov[:, :P, :P]), 0, -1)
    if return_cond:
        return out, eps, cond
    return out, eps


def compute_inversion_error(Fisher, Cov):
    """max |Cov F - 1| per event (gwfast/fisherTools.py:199-212)."""
    F = np.moveaxis(Fisher, -1, 0)
    C = np.moveaxis(Cov, -1, 0)
    return np.abs(C @ F - np.eye(F.shape[-1])).max(axis=(1, 2))


def CheckFisher(FisherM, condNumbMax=1.0e15, use_mpmath=True, verbose=False):
    """Eigenvalues, eigenvectors and condition numbers (gwfast/fisherTools.py:216-279), float64 on the host."""
    evals, evecs = np.linalg.eigh(np.moveaxis(FisherM, -1, 0))
    cond = np.abs(evals).max(axis=1) / np.abs(evals).min(axis=1)
    if verbose and np.any(cond > condNumbMax):
        print('WARNING: the condition number is too large at positions %s' % np.where(cond > condNumbMax)[0])
    return evals, evecs, cond


def fixParams(MatrIn, ParNums_inp, ParMarg):
    """Drop the rows and columns of the fixed parameters (gwfast/fisherTools.py:340-375).

    MatrIn: (P, P, N). Returns the reduced (P', P', N) matrices and the renumbered ParNums."""
    drop = sorted(ParNums_inp[p] for p in ParMarg)
    out = np.delete(np.delete(np.asarray(MatrIn), drop, axis=0), drop, axis=1)
    keep = sorted((i, k) for k, i in ParNums_inp.items() if k not in ParMarg)
    return out, {k: j for j, (_, k) in enumerate(keep)}


def compute_localization_region(Cov, parNum, thFid, perc_level=90, units='SqDeg'):
    """Sky area of the perc_level credible ellipse from the (theta, phi) covariance block
    (gwfast/fisherTools.py:830-866; Barack & Cutler, PRD 69, 082005, 2004):
    dOmega = -2 pi |sin theta| sqrt(C_thth C_phph - C_thph^2) ln(1 - perc_level / 100)."""
    cth = Cov[parNum['theta'], parNum['theta']]
    cph = Cov[parNum['phi'], parNum['phi']]
    cx = Cov[parNum['phi'], parNum['theta']]
    area = -2. * np.pi * np.sqrt(cth * cph - cx ** 2) * np.abs(np.sin(thFid)) * np.log(1. - perc_level / 100.)
    if units == 'Sterad':
        return area
    if units == 'SqDeg':
        return (180. / np.pi) ** 2 * area
    raise ValueError("units must be 'SqDeg' or 'Sterad'")
