"""FP64 restatement of the reference two-site DMRG (test infrastructure only).

Each function follows the reference line by line in FP64; the reference's
device arithmetic is FP32 (src/m_tensor/dense_tensor.mojo:1320-1328) and its
Lanczos / SVD arithmetic FP64 on the host.  Index conventions:

* MPS site  A[Dl, s, Dr]                  (src/state/mps_state.mojo:13-49)
* MPO site  W[wl, s_in, s_out, wr]        (src/state/mpo_state.mojo:10-54)
* env       L[w, D_ket, D_bra], R[w, D_ket, D_bra]
            (index 1 contracts with the ket, index 2 is the bra/output index,
            src/state/environments.mojo:110-131, :320-327)
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import scipy.linalg

DBL_EPSILON = 2.2204460492503131e-16


@dataclass
class DMRGParams:
    """src/algorithms/dmrg.mojo:22-36."""
    num_sweeps: int
    chi_max: int
    eps_trunc: float
    max_krylov_iter: int
    krylov_tol: float
    energy_tol: float
    two_site: bool = True
    verbose: bool = False


# ----------------------------------------------------------------------------
# contractions
# ----------------------------------------------------------------------------

def build_two_site_theta(A_i, A_ip1):
    """dmrg.mojo:93-140: theta[Dl,d,d,Dr] = A_i[Dl*d, Dm] @ A_ip1[Dm, d*Dr]."""
    Dl, d, Dm = A_i.shape
    Dm2, d2, Dr = A_ip1.shape
    if Dm2 != Dm:
        raise ValueError("Bond dimension mismatch in build_two_site_theta")
    if d != d2:
        raise ValueError("Physical dimensions must match")
    return (A_i.reshape(Dl * d, Dm) @ A_ip1.reshape(Dm, d * Dr)).reshape(Dl, d, d, Dr)


def apply_two_site_heff(theta, L, R, W1, W2):
    """dmrg.mojo:254-374, same four-step order.

    out[Dl', t1, t2, Dr'] = sum L[wL,Dl,Dl'] theta[Dl,s1,s2,Dr] W1[wL,s1,t1,wM]
                                W2[wM,s2,t2,wR] R[wR,Dr,Dr']
    """
    T1 = np.tensordot(L, theta, axes=([1], [0]))            # [wL, Dl', s1, s2, Dr]
    T2 = np.tensordot(T1, W1, axes=([0, 2], [0, 1]))        # [Dl', s2, Dr, t1, wM]
    T3 = np.tensordot(T2, W2, axes=([4, 1], [0, 1]))        # [Dl', Dr, t1, t2, wR]
    return np.tensordot(T3, R, axes=([4, 1], [0, 1]))       # [Dl', t1, t2, Dr']


def update_left_environment(L, A, W):
    """environments.mojo:99-201.

    L_next[wR, Dr, Dr'] = sum L[wL,Dl,Dl'] A[Dl,s,Dr] W[wL,s,s',wR] A[Dl',s',Dr']
    """
    T1 = np.tensordot(L, A, axes=([1], [0]))                # [wL, Dl', s, Dr]
    T2 = np.tensordot(T1, W, axes=([0, 2], [0, 1]))         # [Dl', Dr, s', wR]
    T3 = np.tensordot(T2, A, axes=([0, 2], [0, 1]))         # [Dr, wR, Dr']
    return np.ascontiguousarray(T3.transpose(1, 0, 2))


def update_right_environment(R, A, W):
    """environments.mojo:309-417.

    R_prev[wL, Dl, Dl'] = sum R[wR,Dr,Dr'] A[Dl,s,Dr] W[wL,s,s',wR] A[Dl',s',Dr']
    """
    T1 = np.tensordot(R, A, axes=([1], [2]))                # [wR, Dr', Dl, s]
    T2 = np.tensordot(T1, W, axes=([0, 3], [3, 1]))         # [Dr', Dl, wL, s']
    T3 = np.tensordot(T2, A, axes=([0, 3], [2, 1]))         # [Dl, wL, Dl']
    return np.ascontiguousarray(T3.transpose(1, 0, 2))


def identity_env(w: int, D: int):
    """Boundary environment: identity in (D, D) for every channel
    (dmrg.mojo:74-84, environments.mojo:445-455)."""
    E = np.zeros((w, D, D))
    for k in range(w):
        E[k] = np.eye(D)
    return E


def build_right_environments(mps, mpo):
    """environments.mojo:420-472: R[N] = identity, R[i] = update_right(R[i+1])."""
    N = len(mps)
    envs = [None] * (N + 1)
    envs[N] = identity_env(mpo[N - 1].shape[3], mps[N - 1].shape[2])
    for i in range(N - 1, -1, -1):
        envs[i] = update_right_environment(envs[i + 1], mps[i], mpo[i])
    return envs


# ----------------------------------------------------------------------------
# Lanczos + classical Jacobi (dmrg.mojo:486-756)
# ----------------------------------------------------------------------------

def jacobi_smallest_eigpair(T, tol, max_rotations=200):
    """dmrg.mojo:507-598: classical Jacobi with at most ``max_rotations`` rotations.

    Pivot = largest |A[i][j]| (i<j, row-major scan, strict '>'), starting from
    A[0][1].  Returns (smallest diagonal, normalised eigenvector column).
    """
    A = [list(map(float, row)) for row in T]
    n = len(A)
    if n == 0:
        raise ValueError("Empty matrix in Jacobi eigensolver")
    if n == 1:
        return A[0][0], np.array([1.0])
    V = [[1.0 if i == j else 0.0 for j in range(n)] for i in range(n)]
    for _ in range(max_rotations):
        p, q = 0, 1
        max_val = abs(A[0][1])
        for i in range(n):
            for j in range(i + 1, n):
                v = abs(A[i][j])
                if v > max_val:
                    max_val = v
                    p, q = i, j
        if max_val < tol:
            break
        app, aqq, apq = A[p][p], A[q][q], A[p][q]
        phi = 0.5 * math.atan2(2.0 * apq, aqq - app)
        c = math.cos(phi)
        s = math.sin(phi)
        for k in range(n):
            if k != p and k != q:
                aik = A[k][p]
                akq = A[k][q]
                nkp = c * aik - s * akq
                nkq = s * aik + c * akq
                A[k][p] = nkp
                A[p][k] = nkp
                A[k][q] = nkq
                A[q][k] = nkq
        npp = c * c * app - 2.0 * s * c * apq + s * s * aqq
        nqq = s * s * app + 2.0 * s * c * apq + c * c * aqq
        A[p][p] = npp
        A[q][q] = nqq
        A[p][q] = 0.0
        A[q][p] = 0.0
        for k in range(n):
            vip = V[k][p]
            viq = V[k][q]
            V[k][p] = c * vip - s * viq
            V[k][q] = s * vip + c * viq
    min_i = 0
    min_val = A[0][0]
    for i in range(1, n):
        if A[i][i] < min_val:
            min_val = A[i][i]
            min_i = i
    vec = np.array([V[i][min_i] for i in range(n)])
    nrm = math.sqrt(float(np.dot(vec, vec)))
    if nrm > 0.0:
        vec = vec / nrm
    return min_val, vec


@dataclass
class LanczosTrace:
    alpha: list = field(default_factory=list)
    beta: list = field(default_factory=list)
    numiter: int = 0


def lanczos_two_site_optimize(theta, L, R, W1, W2, max_iter, tol,
                              eig="jacobi", trace: LanczosTrace | None = None,
                              reorth: bool = False):
    """dmrg.mojo:486-756 (plain Lanczos, no reorthogonalisation, beta threshold
    100*n*eps, final alpha-only step, capped Jacobi, Ritz vector, normalise).

    ``eig="exact"`` replaces the capped Jacobi by LAPACK dstev (converged mode);
    ``reorth=True`` adds full FP64 reorthogonalisation (not in the reference).
    """
    shape = theta.shape
    v0 = theta.reshape(-1).astype(np.float64)
    dim = v0.size
    norm0 = math.sqrt(float(np.dot(v0, v0)))
    if norm0 < 1e-14:
        raise ValueError("Initial vector has zero norm")
    v0 = v0 / norm0
    krylov = [v0]
    alpha, beta = [], []
    beta_threshold = 100.0 * dim * DBL_EPSILON
    numiter = max_iter
    v = v0
    for j in range(max_iter - 1):
        w = apply_two_site_heff(v.reshape(shape), L, R, W1, W2).reshape(-1)
        a = float(np.dot(krylov[j], w))
        alpha.append(a)
        w = w - a * krylov[j]
        if j > 0:
            w = w - beta[j - 1] * krylov[j - 1]
        if reorth:
            for vk in krylov:
                w = w - float(np.dot(vk, w)) * vk
        b = math.sqrt(float(np.dot(w, w)))
        if b < beta_threshold:
            numiter = j + 1
            break
        beta.append(b)
        v = w / b
        krylov.append(v)
    if numiter == max_iter:
        j = max_iter - 1
        w = apply_two_site_heff(krylov[j].reshape(shape), L, R, W1, W2).reshape(-1)
        alpha.append(float(np.dot(krylov[j], w)))
    nK = numiter
    T = np.zeros((nK, nK))
    for i in range(nK):
        T[i, i] = alpha[i]
    for i in range(nK - 1):
        T[i, i + 1] = beta[i]
        T[i + 1, i] = beta[i]
    if eig == "jacobi":
        E0, coeffs = jacobi_smallest_eigpair(T, tol)
    else:
        if nK == 1:
            E0, coeffs = alpha[0], np.array([1.0])
        else:
            ev, vecs = scipy.linalg.eigh_tridiagonal(np.array(alpha[:nK]), np.array(beta[:nK - 1]))
            E0, coeffs = float(ev[0]), vecs[:, 0]
    out = np.zeros(dim)
    for i in range(nK):
        out += coeffs[i] * krylov[i]
    on = math.sqrt(float(np.dot(out, out)))
    if on > 0.0:
        out = out / on
    if trace is not None:
        trace.alpha = list(alpha)
        trace.beta = list(beta[:nK - 1])
        trace.numiter = nK
    return E0, out.reshape(shape)


# ----------------------------------------------------------------------------
# truncated SVD + split (dense_tensor.mojo:1483-1623, dmrg.mojo:143-252)
# ----------------------------------------------------------------------------

def truncation_rank(S, chi_max, eps_trunc):
    """chi_kept rule of dense_tensor.mojo:1528-1548 (FP64)."""
    k = len(S)
    chi_kept = min(k, chi_max)
    if eps_trunc > 0.0 and k > 0:
        total = 0.0
        for i in range(k):
            total += float(S[i]) * float(S[i])
        if total <= 0.0:
            chi_kept = 0
        else:
            kept = 0.0
            limit = min(k, chi_max)
            chi_kept = limit
            for trial in range(1, limit + 1):
                s = float(S[trial - 1])
                kept += s * s
                if (total - kept) / total <= eps_trunc:
                    chi_kept = trial
                    break
    return chi_kept


def svd_trunc(M, chi_max, eps_trunc):
    """dense_tensor_svd_trunc_lapack_f64: dgesdd thin SVD + chi rule."""
    m, n = M.shape
    if m == 0 or n == 0:
        return np.zeros((m, 0)), np.zeros(0), np.zeros((0, n)), 0
    U, S, Vt = scipy.linalg.svd(M, full_matrices=False, lapack_driver="gesdd")
    chi = truncation_rank(S, chi_max, eps_trunc)
    return U[:, :chi].copy(), S[:chi].copy(), Vt[:chi].copy(), chi


@dataclass
class SplitInfo:
    chi: int
    discarded_weight: float
    S: np.ndarray


def split_two_site_theta_svd(theta, chi_max, eps_trunc, left_to_right=True):
    """dmrg.mojo:143-252: S absorbed right (L->R) or left (R->L)."""
    Dl, d, _, Dr = theta.shape
    total = float(np.dot(theta.reshape(-1), theta.reshape(-1)))
    U, S, Vt, chi = svd_trunc(theta.reshape(Dl * d, d * Dr), chi_max, eps_trunc)
    kept = float(np.dot(S, S))
    disc = (total - kept) / total if total > 0.0 else 0.0
    if left_to_right:
        A = U.reshape(Dl, d, chi)
        B = (S[:, None] * Vt).reshape(chi, d, Dr)
    else:
        A = (U * S[None, :]).reshape(Dl, d, chi)
        B = Vt.reshape(chi, d, Dr)
    return A, B, SplitInfo(chi, disc, S)


# ----------------------------------------------------------------------------
# sweep driver (dmrg.mojo:377-483, :759-844)
# ----------------------------------------------------------------------------

@dataclass
class SweepLog:
    energies: list = field(default_factory=list)       # per sweep (bond-0 R->L value)
    local_energies: list = field(default_factory=list)  # every local update
    discarded: list = field(default_factory=list)
    chis: list = field(default_factory=list)
    spectra: list = field(default_factory=list)


def dmrg_two_site(mpo, mps, params: DMRGParams, eig="jacobi", log: SweepLog | None = None,
                  keep_spectra=False, reorth=False):
    """dmrg.mojo:377-483.  Returns (energy, mps) with a fresh list of sites."""
    if not params.two_site:
        raise ValueError("Only two-site DMRG is currently implemented")
    N = len(mps)
    if N < 2:
        raise ValueError("DMRG requires at least 2 sites")
    if len(mpo) != N:
        raise ValueError("MPS and MPO must have the same number of sites")
    mps = [np.array(a, dtype=np.float64, copy=True) for a in mps]
    R_env = build_right_environments(mps, mpo)
    L_env = [None] * (N + 1)
    L_env[0] = identity_env(mpo[0].shape[0], mps[0].shape[0])
    energy = 0.0
    prev = 0.0

    def local(i, l2r):
        theta = build_two_site_theta(mps[i], mps[i + 1])
        E, th = lanczos_two_site_optimize(theta, L_env[i], R_env[i + 2], mpo[i], mpo[i + 1],
                                          params.max_krylov_iter, params.krylov_tol,
                                          eig=eig, reorth=reorth)
        A, B, info = split_two_site_theta_svd(th, params.chi_max, params.eps_trunc, l2r)
        mps[i], mps[i + 1] = A, B
        if l2r:
            L_env[i + 1] = update_left_environment(L_env[i], A, mpo[i])
        else:
            R_env[i + 1] = update_right_environment(R_env[i + 2], B, mpo[i + 1])
        if log is not None:
            log.local_energies.append(E)
            log.discarded.append(info.discarded_weight)
            log.chis.append(info.chi)
            if keep_spectra:
                log.spectra.append(info.S.copy())
        return E

    for sweep in range(params.num_sweeps):
        for i in range(N - 1):
            energy = local(i, True)
        for i in range(N - 2, -1, -1):
            energy = local(i, False)
        if log is not None:
            log.energies.append(energy)
        if sweep > 0 and abs(energy - prev) < params.energy_tol:
            break
        prev = energy
    return energy, mps


# ----------------------------------------------------------------------------
# helpers used by tests / configs
# ----------------------------------------------------------------------------

def right_normalize(mps):
    """Right-canonical form by QR from the right; site 0 normalised to 1.

    The reference's generic canonicaliser is dead code (mps_state.mojo:204
    calls a method that does not exist); the configs ask for a right-normalised
    random start, so this is the plain textbook LQ sweep.
    """
    mps = [np.array(a, dtype=np.float64, copy=True) for a in mps]
    for i in range(len(mps) - 1, 0, -1):
        Dl, d, Dr = mps[i].shape
        M = mps[i].reshape(Dl, d * Dr)
        Q, Rm = np.linalg.qr(M.T)                 # M^T = Q R -> M = R^T Q^T
        k = Q.shape[1]
        mps[i] = Q.T.reshape(k, d, Dr)
        mps[i - 1] = np.tensordot(mps[i - 1], Rm.T, axes=([2], [0]))
    nrm = np.linalg.norm(mps[0])
    mps[0] = mps[0] / nrm
    return mps


def mps_to_statevector(mps):
    """mps_state.mojo:454-492 (row-major contraction; first site most significant)."""
    psi = mps[0].reshape(-1, mps[0].shape[2])
    for A in mps[1:]:
        psi = (psi @ A.reshape(A.shape[0], -1)).reshape(-1, A.shape[2])
    return psi.reshape(-1)


def expectation(mps, mpo):
    """<psi|H|psi> through left environments (environments.mojo:475-532)."""
    L = identity_env(mpo[0].shape[0], mps[0].shape[0])
    for A, W in zip(mps, mpo):
        L = update_left_environment(L, A, W)
    return float(L.reshape(-1)[0])


def norm_sq(mps):
    L = np.ones((1, 1))
    for A in mps:
        L = np.tensordot(np.tensordot(L, A, axes=([0], [0])), A, axes=([0, 1], [0, 1]))
    return float(L[0, 0])


def heff_flops(chi_l, chi_r, D, d, D2=None):
    """Algorithmic FLOPs of one two-site H_eff apply in the reference order (dmrg.mojo:254-374):
    L . theta 2 D d^2 chi_l^2 chi_r, the two MPO steps 2 D D2 d^3 chi_l chi_r each, . R
    2 D d^2 chi_l chi_r^2 (D2: the MPO bond between the two sites).  At chi_l = chi_r = chi and
    D2 = D: 4 D d^2 chi^3 + 4 D^2 d^3 chi^2."""
    D2 = D if D2 is None else D2
    return (2 * D * d * d * chi_l * chi_l * chi_r + 4 * D * D2 * d ** 3 * chi_l * chi_r
            + 2 * D * d * d * chi_l * chi_r * chi_r)


def env_flops(chi_l, chi_r, D, d):
    return 2 * D * d * chi_l * chi_l * chi_r + 2 * D * D * d * d * chi_l * chi_r + 2 * D * d * chi_l * chi_r * chi_r
