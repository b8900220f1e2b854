"""Pins of the oracle's MPS observables (no GPU) against dense state-vector algebra.

The reference's own checks (src/tests/state/mps/test_mps_observables.mojo) are
range checks plus <psi|psi> = ||psi||^2; here every observable is compared with
the same quantity formed from the dense state vectors and the dense MPO matrix
M[s_in, s_out] (oracle.ed.mpo_to_sparse), which also fixes the index roles:
the ket contracts with s_in, the bra with s_out, apply_mpo returns M^T psi and
mpo_compose(a, b) is M_a M_b.
"""
import numpy as np
import pytest

from oracle import dmrg as od
from oracle import ed
from oracle import hamiltonians as oh
from oracle import observables as ob


def random_mps(L, d, chi, seed):
    rng = np.random.default_rng(seed)
    dims = [1] + [min(chi, d ** min(k, L - k)) for k in range(1, L)] + [1]
    return [rng.standard_normal((dims[i], d, dims[i + 1])) / np.sqrt(dims[i] * d) for i in range(L)]


def random_mpo(L, d, D, seed):
    rng = np.random.default_rng(seed)
    dims = [1] + [D] * (L - 1) + [1]
    return [rng.standard_normal((dims[i], d, d, dims[i + 1])) for i in range(L)]


def dense(mpo):
    return ed.mpo_to_sparse(mpo).toarray()


def statevector_to_mps(psi, L, d):
    """exact MPS by successive SVDs (no truncation)"""
    sites = []
    rest = psi.reshape(1, -1)
    Dl = 1
    for _ in range(L - 1):
        M = rest.reshape(Dl * d, -1)
        U, S, Vt = np.linalg.svd(M, full_matrices=False)
        k = int(np.sum(S > 1e-14 * S[0]))
        sites.append(U[:, :k].reshape(Dl, d, k))
        rest = S[:k, None] * Vt[:k]
        Dl = k
    sites.append(rest.reshape(Dl, d, 1))
    return sites


@pytest.mark.parametrize("L,d,chi,D", [(5, 2, 4, 3), (4, 3, 5, 2), (6, 2, 8, 4)])
def test_two_mps_expectation_and_overlap(L, d, chi, D):
    bra, ket = random_mps(L, d, chi, 1), random_mps(L, d, chi + 1, 2)
    mpo = random_mpo(L, d, D, 3)
    sb, sk = od.mps_to_statevector(bra), od.mps_to_statevector(ket)
    M = dense(mpo)
    assert ob.expectation_value_two_mps(bra, mpo, ket) == pytest.approx(sb @ (M.T @ sk), rel=1e-12, abs=1e-14)
    assert ob.mps_overlap(bra, ket) == pytest.approx(sb @ sk, rel=1e-12, abs=1e-14)
    assert ob.mps_overlap(ket, ket) == pytest.approx(sk @ sk, rel=1e-12)
    # the two-MPS environment with bra == ket is the one-MPS environment
    assert ob.expectation_value_two_mps(ket, mpo, ket) == pytest.approx(od.expectation(ket, mpo), rel=1e-12)


def test_apply_mpo_and_compose():
    L, d = 5, 2
    psi = random_mps(L, d, 4, 7)
    a, b = random_mpo(L, d, 3, 8), random_mpo(L, d, 2, 9)
    out = ob.apply_mpo(a, psi)
    assert [s.shape for s in out] == [(a[i].shape[0] * psi[i].shape[0], d, a[i].shape[3] * psi[i].shape[2])
                                      for i in range(L)]
    np.testing.assert_allclose(od.mps_to_statevector(out), dense(a).T @ od.mps_to_statevector(psi), rtol=1e-12,
                               atol=1e-13)
    comp = ob.mpo_compose(a, b)
    np.testing.assert_allclose(dense(comp), dense(a) @ dense(b), rtol=1e-12, atol=1e-12)


def test_variance_and_utilities():
    L = 6
    mpo = oh.heisenberg_xxz(L, J=1.0, D=0.7, h=0.1)
    H = dense(mpo)
    psi = random_mps(L, 2, 8, 11)
    v = od.mps_to_statevector(psi)
    n2 = v @ v
    E = v @ H @ v / n2
    assert ob.energy(psi, mpo) == pytest.approx(E, rel=1e-12)
    assert ob.variance_op(psi, mpo) == pytest.approx(v @ H @ H @ v / n2 - E * E, rel=1e-10)
    # an eigenstate has zero variance
    w, U = np.linalg.eigh(0.5 * (H + H.T))
    gs = statevector_to_mps(U[:, 0], L, 2)
    assert abs(ob.variance(gs, mpo)) < 1e-10
    assert ob.energy(gs, mpo) == pytest.approx(w[0], rel=1e-12)
    assert ob.fidelity(gs, gs) == pytest.approx(1.0, rel=1e-12)
    # single- and two-site spin observables against the dense operators
    Z = np.diag([1.0, -1.0])
    X = np.array([[0.0, 1.0], [1.0, 0.0]])

    def op_at(ops):
        out = np.ones((1, 1))
        for k in range(L):
            out = np.kron(out, ops.get(k, np.eye(2)))
        return out
    assert ob.observe_sz(psi, 2) == pytest.approx(0.5 * v @ op_at({2: Z}).T @ v / n2, rel=1e-12, abs=1e-14)
    assert ob.observe_sz_sz(psi, 1, 4) == pytest.approx(0.25 * v @ op_at({1: Z, 4: Z}) @ v / n2, rel=1e-12,
                                                        abs=1e-14)
    assert ob.observe_sx_sx(psi, 0, 5) == pytest.approx(0.25 * v @ op_at({0: X, 5: X}) @ v / n2, rel=1e-12,
                                                        abs=1e-14)


def test_builders_and_errors():
    idm = ob.create_identity_mpo(3, 4)
    np.testing.assert_array_equal(dense(idm), np.eye(64))
    with pytest.raises(ValueError):
        ob.create_single_site_op_mpo(3, 3, ob.PAULI_Z)
    with pytest.raises(ValueError):
        ob.create_two_site_op_mpo(4, 2, 2, ob.PAULI_Z, ob.PAULI_Z)
    with pytest.raises(ValueError):
        ob.mps_overlap(random_mps(3, 2, 2, 0), random_mps(4, 2, 2, 0))
    with pytest.raises(ValueError):
        ob.apply_mpo(random_mpo(3, 3, 2, 0), random_mps(3, 2, 2, 0))
    assert ob.mps_vdot_direct([], []) == 0.0
