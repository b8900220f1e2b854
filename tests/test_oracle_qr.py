"""The oracle's QR path (no GPU), on the reference's own fixtures: test_dense_tensor_qr.mojo
uses make_host_data_f32 (src/tests/test_utils.mojo:13-21) with seeds 100-104 and checks Q^T Q = I,
R upper triangular and Q R = A; mps_orthogonalize_qr must rebuild the state."""
import numpy as np
import pytest

from oracle import dmrg as od
from oracle import qr as oq


def lcg_data(nelem, seed):
    state = seed
    out = []
    for _ in range(nelem):
        state = (1664525 * state + 1013904223) % (1 << 32)
        out.append(np.float32(state / float(1 << 32) - 0.5))
    return np.array(out, dtype=np.float64)


@pytest.mark.parametrize("m,n,seed", [(6, 4, 100), (5, 5, 101), (4, 6, 103), (5, 5, 104), (2, 2, 105)])
def test_reference_qr_fixtures(m, n, seed):
    A = lcg_data(m * n, seed).reshape(m, n)
    Q, R = oq.dense_tensor_qr(A)
    k = min(m, n)
    assert Q.shape == (m, k) and R.shape == (k, n)
    assert np.abs(Q.T @ Q - np.eye(k)).max() < 1e-14
    assert np.abs(np.tril(R, -1)).max() == 0.0
    assert np.abs(Q @ R - A).max() < 1e-14


def test_non_2d_raises():
    with pytest.raises(ValueError, match="2D matrix"):
        oq.dense_tensor_qr(np.ones(6))


def test_orthogonalize_rebuilds_state():
    rng = np.random.default_rng(3)
    psi = rng.standard_normal((2,) * 7)
    sites = oq.mps_orthogonalize_qr(psi)
    v = od.mps_to_statevector(sites)
    np.testing.assert_allclose(v, psi.reshape(-1) / np.linalg.norm(psi), rtol=1e-12, atol=1e-14)
    for A in sites[:-1]:
        M = A.reshape(-1, A.shape[2])
        assert np.abs(M.T @ M - np.eye(M.shape[1])).max() < 1e-13
