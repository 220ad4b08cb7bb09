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
    """Eigenvalues (N, P), eigenvectors (N, P, P) and condition numbers (N,) of (P, P, N) Fisher
    matrices (gwfast/fisherTools.py:216-279). The decomposition is LAPACK's in float64 on the host
    (use_mpmath is accepted for the signature: gwfast's mpmath eigh runs at its default 53-bit
    precision too). As there, an all-NaN matrix gives NaN rows, a matrix whose decomposition fails
    gives NaN rows, and negative eigenvalues are reported."""
    F = np.moveaxis(np.asarray(FisherM, dtype=np.float64), -1, 0)
    evals = np.full(F.shape[:2], np.nan)
    evecs = np.full(F.shape, np.nan)
    ok = ~np.all(np.isnan(F), axis=(1, 2))
    if verbose:
        for k in np.where(~ok)[0]:
            print('Fisher is nan at position %s. ' % k)
    idx = np.where(ok)[0]
    try:
        if idx.size:
            evals[idx], evecs[idx] = np.linalg.eigh(F[idx])
    except np.linalg.LinAlgError:
        for k in idx:
            try:
                evals[k], evecs[k] = np.linalg.eigh(F[k])
            except np.linalg.LinAlgError as e:
                print(e)
                print('Event is number %s' % k)
    if np.any(evals <= 0.):
        print('WARNING: one or more eigenvalues are negative at position(s) %s' % str(np.unique(np.where(evals < 0)[0])))
    cond = np.abs(evals).max(axis=1) / np.abs(evals).min(axis=1)
    if np.any(cond > condNumbMax) and verbose:
        print('WARNING: the condition number is too large (%s>%s)' % (cond, condNumbMax))
        print('Unreliable covariance at positions ' + str(cond > condNumbMax))
    elif verbose:
        print('Condition number= %s . Ok. ' % cond)
    return evals, evecs, cond


def fixParams(MatrIn, ParNums_inp, ParMarg):
    """Drop the rows and columns of the fixed parameters (gwfast/fisherTools.py:340-375).

    MatrIn: (P, P, N). Returns the reduced (P', P', N) matrices and the renumbered ParNums."""
    drop = sorted(ParNums_inp[p] for p in ParMarg)
    out = np.delete(np.delete(np.asarray(MatrIn), drop, axis=0), drop, axis=1)
    keep = sorted((i, k) for k, i in ParNums_inp.items() if k not in ParMarg)
    return out, {k: j for j, (_, k) in enumerate(keep)}


def perturb_Fisher(totF, eps=1e-10, **kwargs):
    """Invert the Fisher matrices and again after adding uniform random perturbations of size eps, and
    print the relative change of each covariance (infinity norm), as a stability check
    (gwfast/fisherTools.py:282-299). Returns those relative changes."""
    Cov_base, _ = CovMatr(totF, **kwargs)
    Cov, _ = CovMatr(np.asarray(totF) + np.random.rand(*np.shape(totF)) * eps, **kwargs)
    err = [np.linalg.norm(Cov_base[..., i] / Cov[..., i] - 1., ord=np.inf) for i in range(Cov.shape[-1])]
    print('Relative errors when perturbing at the %s level: %s' % (eps, err))
    return err


def check_covariance(FisherM, Cov, tol=1e-10):
    """Products Cov F per event with the inversion error, the diagonal minus one, the largest
    off-diagonal element and the mask of off-diagonal elements above tol printed, as
    gwfast/fisherTools.py:302-336. Returns the list of (P, P) products."""
    prods = [Cov[:, :, i] @ FisherM[:, :, i] for i in range(Cov.shape[-1])]
    print('Inversion errors: %s' % compute_inversion_error(FisherM, Cov))
    print('diagonal-1 = %s' % str([m.diagonal() - 1. for m in prods]))
    off = [m[~np.eye(m.shape[0], dtype=bool)] for m in prods]
    print('Max off diagonal: %s' % str([o.max() for o in off]))
    print('\nmask: where F*S(off-diagonal)>%s (--> problematic if True off diagonal)' % tol)
    print([m > tol for m in prods])
    return prods


def addPrior(Matr, vals, ParNums, ParAdd):
    """Gaussian priors: vals added to the diagonal at the parameters ParAdd (gwfast/fisherTools.py:378-407).
    As there, the values go to the positions in increasing parameter order."""
    idx = np.sort(np.array([ParNums[p] for p in ParAdd]))
    P = Matr.shape[0]
    diag = np.zeros(P)
    diag[idx] = vals
    prior = np.diag(diag)
    return prior + Matr if Matr.ndim == 2 else prior[:, :, None] + Matr


def log_dL_to_dL_derivative_fish(or_matrix, ParNums, evParams):
    """Fisher matrices in log(dL) -> in dL: row and column dL divided by dL (gwfast/fisherTools.py:435-458)."""
    m = np.array(or_matrix, dtype=np.float64, copy=True)
    i = ParNums['dL']
    m[:, i, :] /= np.asarray(evParams['dL'], dtype=np.float64)
    m[i, :, :] /= np.asarray(evParams['dL'], dtype=np.float64)
    return m


def log_dL_to_dL_derivative_cov(or_matrix, ParNums, evParams):
    """Covariance matrices in log(dL) -> in dL: row and column dL times dL (gwfast/fisherTools.py:410-432)."""
    m = np.array(or_matrix, dtype=np.float64, copy=True)
    i = ParNums['dL']
    m[:, i, :] *= np.asarray(evParams['dL'], dtype=np.float64)
    m[i, :, :] *= np.asarray(evParams['dL'], dtype=np.float64)
    return m


# component masses <-> (Mc, eta) (gwfast/fisherTools.py:461-617): m_{1,2} = (1 +- sqrt(1 - 4 eta)) / 2 Mc eta^(-3/5)
def dm1_dMc(eta):
    return (1. + np.sqrt(1. - 4. * eta)) * eta ** (-3. / 5.) / 2.


def dm2_dMc(eta):
    return (1. - np.sqrt(1. - 4. * eta)) * eta ** (-3. / 5.) / 2.


def dm1_deta(Mc, eta):
    s = np.sqrt(1. - 4. * eta)
    return -Mc * (3. - 2. * eta + 3. * s) / (10. * s * eta ** (8. / 5.))


def dm2_deta(Mc, eta):
    s = np.sqrt(1. - 4. * eta)
    return -Mc * (-3. + 2. * eta + 3. * s) / (10. * s * eta ** (8. / 5.))


def dMc_dm1(m1, m2):
    return m2 * (2. * m1 + 3. * m2) / (5. * (m1 * m2) ** (2. / 5.) * (m1 + m2) ** (6. / 5.))


def dMc_dm2(m1, m2):
    return dMc_dm1(m2, m1)


def deta_dm1(m1, m2):
    return m2 * (m2 - m1) / (m1 + m2) ** 3


def deta_dm2(m1, m2):
    return deta_dm1(m2, m1)


def J_m1m2_Mceta(Mc, eta):
    """d(m1, m2) / d(Mc, eta)."""
    return np.array([[dm1_dMc(eta), dm1_deta(Mc, eta)], [dm2_dMc(eta), dm2_deta(Mc, eta)]])


def J_Mceta_m1m2(m1, m2):
    """d(Mc, eta) / d(m1, m2)."""
    return np.array([[dMc_dm1(m1, m2), dMc_dm2(m1, m2)], [deta_dm1(m1, m2), deta_dm2(m1, m2)]])


def m1m2_from_Mceta(Mc, eta):
    s = np.sqrt(1. - 4. * eta)
    return (1. + s) / 2. * Mc / eta ** (3. / 5.), (1. - s) / 2. * Mc / eta ** (3. / 5.)


def Mceta_from_m1m2(m1, m2):
    """Chirp mass and symmetric mass ratio. (gwfast's fisherTools copy of this function,
    :606-617, writes (m1*m2)**3/5/(m1+m2)**1/5, which Python reads as ((m1 m2)^3 / 5) / ((m1 + m2) / 5);
    this returns the chirp mass, as its gwfastUtils.Mceta_from_m1m2 does.)"""
    return (m1 * m2) ** (3. / 5.) / (m1 + m2) ** (1. / 5.), (m1 * m2) / (m1 + m2) ** 2


def _rotate(or_matrix, ParNums, names, J, transpose_left):
    R = np.identity(or_matrix.shape[0])
    i = [ParNums[n] for n in names]
    R[np.ix_(i, i)] = J
    return (R.T if transpose_left else R) @ or_matrix @ R


def m1m2_to_Mceta_fish(or_matrix, ParNums, evParams):
    """One event's (P, P) Fisher matrix from (m1, m2) to (Mc, eta), as gwfast/fisherTools.py:620-640
    writes it (R F R with R = d(m1, m2)/d(Mc, eta) in the Mc, eta block)."""
    return _rotate(or_matrix, ParNums, ('Mc', 'eta'), J_m1m2_Mceta(evParams['Mc'], evParams['eta']), False)


def m1m2_to_Mceta_cov(or_matrix, ParNums, evParams):
    """One event's (P, P) covariance from (m1, m2) to (Mc, eta), as gwfast/fisherTools.py:643-663."""
    return _rotate(or_matrix, ParNums, ('Mc', 'eta'), J_Mceta_m1m2(*m1m2_from_Mceta(evParams['Mc'], evParams['eta'])),
                   False)


def Mceta_to_m1m2_fish(or_matrix, ParNums, evParams):
    """One event's (P, P) Fisher matrix from (Mc, eta) to (m1, m2): R^T F R, R = d(Mc, eta)/d(m1, m2)
    (gwfast/fisherTools.py:666-687)."""
    m1, m2 = m1m2_from_Mceta(evParams['Mc'], evParams['eta'])
    return _rotate(or_matrix, ParNums, ('Mc', 'eta'), J_Mceta_m1m2(m1, m2), True)


def Mceta_to_m1m2_cov(or_matrix, ParNums, evParams):
    """One event's (P, P) covariance from (Mc, eta) to (m1, m2): R^T C R, R = d(m1, m2)/d(Mc, eta)
    (gwfast/fisherTools.py:690-709)."""
    return _rotate(or_matrix, ParNums, ('Mc', 'eta'), J_m1m2_Mceta(evParams['Mc'], evParams['eta']), True)


def dchi1_dchieff(m1, m2):
    return 1.


def dchi2_dchieff(m1, m2):
    return 1.


def dchi1_dDelchi(m1, m2):
    return m2 / (m1 + m2)


def dchi2_dDelchi(m1, m2):
    return -m1 / (m1 + m2)


def J_chi1chi2_chieffDeltachi(m1, m2):
    """d(chi1z, chi2z) / d(chi_eff, Delta chi) (gwfast/fisherTools.py:764-775)."""
    return np.array([[1., dchi1_dDelchi(m1, m2)], [1., dchi2_dDelchi(m1, m2)]])


def chi1chi2_to_chieffDeltachi_fish(or_matrix, ParNums, evParams):
    """One event's (P, P) Fisher matrix from (chi1z, chi2z) to (chi_eff, Delta chi): R^T F R
    (gwfast/fisherTools.py:778-799)."""
    return _rotate(or_matrix, ParNums, ('chi1z', 'chi2z'),
                   J_chi1chi2_chieffDeltachi(*m1m2_from_Mceta(evParams['Mc'], evParams['eta'])), True)


def chiSchiA_to_chi1chi2_fish(or_matrix, ParNums, evParams):
    """One event's (P, P) Fisher matrix from (chiS, chiA) to (chi1z, chi2z) (gwfast/fisherTools.py:802-823)."""
    return _rotate(or_matrix, ParNums, ('chiS', 'chiA'), np.array([[.5, .5], [.5, -.5]]), False)


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
