"""FP64 restatement of the reference's MPS observables (test infrastructure only).

Follows src/state/environments.mojo:535-1189, src/state/mpo_state.mojo:196-310 and
src/algorithms/dmrg_utils.mojo:18-91.  Sites are numpy arrays in the reference
layouts (MPS A[Dl, s, Dr], MPO W[wl, s_in, s_out, wr]); environments with two
different states are L[w, D_ket, D_bra].
"""
from __future__ import annotations

import numpy as np

from .dmrg import update_left_environment


def update_left_environment_two_mps(L, A_bra, A_ket, W):
    """environments.mojo:535-590.

    L_next[wR, Dr, Dr'] = sum L[wL,Dl,Dl'] A_ket[Dl,s,Dr] W[wL,s,s',wR] A_bra[Dl',s',Dr']
    """
    T1 = np.tensordot(L, A_ket, axes=([1], [0]))            # [wL, Dl', s, Dr]
    T2 = np.tensordot(T1, W, axes=([0, 2], [0, 1]))         # [Dl', Dr, s', wR]
    T3 = np.tensordot(T2, A_bra, axes=([0, 2], [0, 1]))     # [Dr, wR, Dr']
    return np.ascontiguousarray(T3.transpose(1, 0, 2))


def expectation_value_two_mps(bra, mpo, ket):
    """environments.mojo:698-730: <bra|mpo|ket>; the boundary is the identity in
    (Dl0, Dl0) with Dl0 the bra's left bond, and the result is element 0."""
    N = len(bra)
    if len(mpo) != N or len(ket) != N:
        raise ValueError("expectation_value_two_mps: length mismatch")
    wL0 = mpo[0].shape[0]
    Dl0 = bra[0].shape[0]
    L = np.zeros((wL0, Dl0, Dl0))
    for w in range(wL0):
        L[w] = np.eye(Dl0)
    for i in range(N):
        L = update_left_environment_two_mps(L, bra[i], ket[i], mpo[i])
    if L.size != 1:
        raise ValueError("Unexpected final environment size in expectation_value_two_mps")
    return float(L.reshape(-1)[0])


def mps_contraction_step_left(A_bra, A_ket, L):
    """environments.mojo:767-862: L[Dl_ket, Dl_bra] -> L[Dr_ket, Dr_bra] (no MPO)."""
    temp = np.tensordot(L, A_ket, axes=([0], [0]))          # [Dl_bra, d, Dr_ket]
    return np.tensordot(temp, A_bra, axes=([0, 1], [0, 1]))  # [Dr_ket, Dr_bra]


def mps_vdot_direct(bra, ket):
    """environments.mojo:971-1016: <bra|ket>, boundary identity of min(Dl_ket, Dl_bra)."""
    N = len(bra)
    if len(ket) != N:
        raise ValueError("mps_vdot_direct: length mismatch")
    if N == 0:
        return 0.0
    Dk, Db = ket[0].shape[0], bra[0].shape[0]
    L = np.zeros((Dk, Db))
    for i in range(min(Dk, Db)):
        L[i, i] = 1.0
    for i in range(N):
        L = mps_contraction_step_left(bra[i], ket[i], L)
    if L.size != 1:
        raise ValueError("mps_vdot_direct: final L is not scalar")
    return float(L.reshape(-1)[0])


def mps_overlap(bra, ket):
    """environments.mojo:1018-1025."""
    return mps_vdot_direct(bra, ket)


def expectation_value(mps, mpo):
    """environments.mojo:475-518 (identity boundary over the MPS's left bond)."""
    wL0, Dl0 = mpo[0].shape[0], mps[0].shape[0]
    L = np.zeros((wL0, Dl0, Dl0))
    for w in range(wL0):
        L[w] = np.eye(Dl0)
    for A, W in zip(mps, mpo):
        L = update_left_environment(L, A, W)
    if L.size != 1:
        raise ValueError("Unexpected final environment size in expectation_value")
    return float(L.reshape(-1)[0])


def expectation_value_normalized(mps, mpo):
    """environments.mojo:521-532: <H> / <I> with the identity MPO."""
    num = expectation_value(mps, mpo)
    den = expectation_value(mps, create_identity_mpo(len(mps), mps[0].shape[1]))
    if abs(den) < 1e-20:
        raise ValueError("MPS norm is ~0 in expectation_value_normalized")
    return num / den


def mpo_compose(mpo_a, mpo_b):
    """environments.mojo:1086-1132.

    W[(al, bl), i, o, (ar, br)] = sum_m Wa[al, i, m, ar] Wb[bl, m, o, br]
    """
    if len(mpo_a) != len(mpo_b):
        raise ValueError("MPO compose: length mismatch")
    out = []
    for Wa, Wb in zip(mpo_a, mpo_b):
        wLa, d_in, d_mid, wRa = Wa.shape
        wLb, d_mid2, d_out, wRb = Wb.shape
        if d_mid2 != d_mid:
            raise ValueError("MPO compose: physical dim mismatch")
        C = np.tensordot(Wa, Wb, axes=([2], [1]))            # [wLa, d_in, wRa, wLb, d_out, wRb]
        C = C.transpose(0, 3, 1, 4, 2, 5)
        out.append(np.ascontiguousarray(C).reshape(wLa * wLb, d_in, d_out, wRa * wRb))
    return out


def variance(mps, mpo):
    """environments.mojo:1071-1083: <H^2> - <H>^2 with H^2 = mpo_compose(H, H)."""
    E = expectation_value_normalized(mps, mpo)
    E2 = expectation_value_normalized(mps, mpo_compose(mpo, mpo))
    return E2 - E * E


def apply_mpo(mpo, mps):
    """environments.mojo:1135-1189.

    out[(w, a), t, (v, b)] = sum_s A[a, s, b] W[w, s, t, v]
    """
    if len(mpo) != len(mps):
        raise ValueError("apply_mpo: MPS and MPO must have same number of sites")
    out = []
    for A, W in zip(mps, mpo):
        Dl, d, Dr = A.shape
        wL, d_in, d_out, wR = W.shape
        if d_in != d:
            raise ValueError("apply_mpo: physical dim mismatch")
        C = np.tensordot(A, W, axes=([1], [1]))              # [Dl, Dr, wL, d_out, wR]
        C = C.transpose(2, 0, 3, 4, 1)                       # [wL, Dl, d_out, wR, Dr]
        out.append(np.ascontiguousarray(C).reshape(wL * Dl, d_out, wR * Dr))
    return out


# ---- MPO builders (mpo_state.mojo:196-310) -------------------------------------

def create_identity_mpo(num_sites: int, physical_dim: int):
    """mpo_state.mojo:196-241: bond dimension 1, identity on every site."""
    if num_sites < 1 or physical_dim < 1:
        raise ValueError("invalid identity MPO")
    return [np.eye(physical_dim).reshape(1, physical_dim, physical_dim, 1) for _ in range(num_sites)]


def create_single_site_op_mpo(num_sites: int, site_idx: int, op_data):
    """mpo_state.mojo:243-272: 2x2 row-major op on one site, identity elsewhere."""
    if num_sites < 1 or site_idx < 0 or site_idx >= num_sites:
        raise ValueError("create_single_site_op_mpo: invalid site_idx")
    if len(op_data) != 4:
        raise ValueError("create_single_site_op_mpo: op_data must be 4 elements (2x2)")
    sites = create_identity_mpo(num_sites, 2)
    sites[site_idx] = np.asarray(op_data, dtype=np.float64).reshape(1, 2, 2, 1)
    return sites


def create_two_site_op_mpo(num_sites: int, site_i: int, site_j: int, op_i_data, op_j_data):
    """mpo_state.mojo:275-310: O_i O_j with site_i < site_j, identity elsewhere."""
    if num_sites < 2 or site_i < 0 or site_j >= num_sites or site_i >= site_j:
        raise ValueError("create_two_site_op_mpo: invalid sites")
    if len(op_i_data) != 4 or len(op_j_data) != 4:
        raise ValueError("create_two_site_op_mpo: op data must be 4 elements each")
    sites = create_identity_mpo(num_sites, 2)
    sites[site_i] = np.asarray(op_i_data, dtype=np.float64).reshape(1, 2, 2, 1)
    sites[site_j] = np.asarray(op_j_data, dtype=np.float64).reshape(1, 2, 2, 1)
    return sites


# ---- dmrg_utils.mojo:18-91 -------------------------------------------------------

PAULI_Z = [1.0, 0.0, 0.0, -1.0]
PAULI_X = [0.0, 1.0, 1.0, 0.0]


def energy(mps, mpo):
    return expectation_value_normalized(mps, mpo)


def variance_op(mps, mpo):
    return variance(mps, mpo)


def fidelity(mps1, mps2):
    return abs(mps_overlap(mps1, mps2))


def observe_sz(mps, i):
    return 0.5 * expectation_value_normalized(mps, create_single_site_op_mpo(len(mps), i, PAULI_Z))


def observe_sz_sz(mps, i, j):
    return 0.25 * expectation_value_normalized(mps, create_two_site_op_mpo(len(mps), i, j, PAULI_Z, PAULI_Z))


def observe_sx_sx(mps, i, j):
    return 0.25 * expectation_value_normalized(mps, create_two_site_op_mpo(len(mps), i, j, PAULI_X, PAULI_X))


# ---- bond entropies (the JSON schema's reserved "entropy", main.mojo:662) -----

def bond_entropies_statevector(psi, L, d):
    """-sum p ln p of the Schmidt values across each inner bond of a dense state."""
    out = []
    v = np.asarray(psi, dtype=np.float64).reshape(-1)
    for i in range(1, L):
        s = np.linalg.svd(v.reshape(d ** i, -1), compute_uv=False)
        p = s * s / np.sum(s * s)
        p = p[p > 0]
        out.append(float(-np.sum(p * np.log(p))))
    return out
