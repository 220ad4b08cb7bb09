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
    if F.shape[1:] != (11, 11):
        raise NotImplementedError('the GPU inversion handles 11x11 matrices')
    N = F.shape[0]
    cov = np.empty_like(F)
    eps = np.empty(N)
    cond = np.empty(N)
    _lib.context(device).cov(F, cov=cov, eps=eps, cond=cond)
    out = np.moveaxis(cov, 0, -1)
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
