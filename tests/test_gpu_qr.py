"""Device thin QR (ct_qr, dense_tensor_qr) and the QR canonicalisers against the oracle.

* the reference's fixtures (test_dense_tensor_qr.mojo: LCG data, 6x4, 5x5, 4x6, 2x2) and larger
  random shapes, tall and wide: Q^T Q = I and Q R = A to 1e-13 relative, R exactly zero below
  the diagonal, and Q, R equal LAPACK's (NumPy) up to the signs of Q's columns / R's rows;
* rank-deficient inputs (a zero column, repeated and dependent columns, a product state): the
  completed columns keep Q orthonormal and Q R = A;
* non-2D input raises, as in the reference;
* mps_orthogonalize_qr rebuilds a dense state; left/right canonicalisation keeps the state and
  makes the sites left/right-orthonormal.
"""
import numpy as np
import pytest

from oracle import dmrg as od
from oracle import qr as oq

pytestmark = pytest.mark.gpu


def ct_mod():
    import chemtensor_mojo_gb300 as ct
    return ct


def lcg_data(nelem, seed):
    state = seed
    out = []
    for _ in range(nelem):
        state = (1664525 * state + 1013904223) % (1 << 32)
        out.append(np.float32(state / float(1 << 32) - 0.5))
    return np.array(out, dtype=np.float64)


def device_qr(ctx, A):
    ct = ct_mod()
    Q, R = ct.dense_tensor_qr(ct.create_dense_tensor_from_data(ctx, A, A.shape), ctx)
    return Q.to_numpy(), R.to_numpy()


def check_qr(A, Q, R, tol=1e-13):
    m, n = A.shape
    k = min(m, n)
    assert Q.shape == (m, k) and R.shape == (k, n)
    assert np.abs(Q.T @ Q - np.eye(k)).max() < tol
    assert np.all(np.tril(R, -1) == 0.0)
    assert np.linalg.norm(Q @ R - A) <= tol * max(np.linalg.norm(A), 1e-300)


@pytest.mark.parametrize("m,n,seed", [(6, 4, 100), (5, 5, 101), (4, 6, 103), (5, 5, 104), (2, 2, 105)])
def test_reference_fixtures(ctx, m, n, seed):
    A = lcg_data(m * n, seed).reshape(m, n)
    Q, R = device_qr(ctx, A)
    check_qr(A, Q, R)
    Qr, Rr = oq.dense_tensor_qr(A)
    s = np.sign(np.diag(Rr))
    np.testing.assert_allclose(Q * s, Qr, rtol=0, atol=1e-13)
    np.testing.assert_allclose(R * s[:, None], Rr, rtol=0, atol=1e-13)


@pytest.mark.parametrize("m,n", [(1000, 700), (300, 900), (2048, 1024), (129, 65)])
def test_random_shapes(ctx, m, n):
    rng = np.random.default_rng(m + n)
    A = rng.standard_normal((m, n))
    Q, R = device_qr(ctx, A)
    check_qr(A, Q, R, tol=2e-13)
    Qr, Rr = oq.dense_tensor_qr(A)
    s = np.sign(np.diag(Rr))
    np.testing.assert_allclose(R * s[:, None], Rr, rtol=0, atol=1e-10 * np.abs(Rr).max())


def test_rank_deficient(ctx):
    rng = np.random.default_rng(9)
    A = rng.standard_normal((200, 60))
    A[:, 7] = 0.0                                   # zero column
    A[:, 20] = A[:, 3]                              # repeated column
    A[:, 41] = 2.0 * A[:, 5] - 0.5 * A[:, 30]       # dependent column
    Q, R = device_qr(ctx, A)
    check_qr(A, Q, R, tol=2e-13)
    # the product state |0...0> as a dense vector: one nonzero per column block
    psi = np.zeros((2,) * 6)
    psi[(0,) * 6] = 1.0
    M = psi.reshape(8, 8)
    Q, R = device_qr(ctx, M)
    check_qr(M, Q, R)


def test_non_2d_raises(ctx):
    ct = ct_mod()
    with pytest.raises(ValueError, match="2D matrix"):
        ct.dense_tensor_qr(ct.create_dense_tensor_from_data(ctx, np.ones(6), [6]), ctx)


def test_orthogonalize_and_canonicalise(ctx):
    ct = ct_mod()
    rng = np.random.default_rng(4)
    L = 8
    psi = rng.standard_normal((2,) * L)
    mps = ct.mps_orthogonalize_qr(ctx, ct.create_dense_tensor_from_data(ctx, psi, psi.shape))
    sites = mps.to_numpy()
    ref = oq.mps_orthogonalize_qr(psi)
    assert [a.shape for a in sites] == [a.shape for a in ref]
    np.testing.assert_allclose(od.mps_to_statevector(sites), psi.reshape(-1) / np.linalg.norm(psi), rtol=1e-12,
                               atol=1e-13)
    for A in sites[:-1]:
        M = A.reshape(-1, A.shape[2])
        assert np.abs(M.T @ M - np.eye(M.shape[1])).max() < 1e-13
    # random MPS: left- and right-canonical forms keep the (normalised) state
    dims = [1, 2, 4, 8, 16, 8, 4, 2, 1]
    arrays = [rng.standard_normal((dims[i], 2, dims[i + 1])) for i in range(L)]
    v0 = od.mps_to_statevector(arrays)
    v0 = v0 / np.linalg.norm(v0)
    for how in ("left", "right"):
        m2 = ct.mps_from_arrays(ctx, arrays)
        getattr(m2, f"{how}_canonicalize")(ctx)
        s2 = m2.to_numpy()
        v = od.mps_to_statevector(s2)
        assert abs(abs(v @ v0) - 1.0) < 1e-12 and abs(np.linalg.norm(v) - 1.0) < 1e-12
        inner = s2[:-1] if how == "left" else s2[1:]
        for A in inner:
            M = A.reshape(-1, A.shape[2]) if how == "left" else A.reshape(A.shape[0], -1)
            G = M.T @ M if how == "left" else M @ M.T
            assert np.abs(G - np.eye(G.shape[0])).max() < 1e-13
