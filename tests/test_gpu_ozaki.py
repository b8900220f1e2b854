"""FP64 GEMM emulated on the BF16 tensor cores (ct_gemm with CT_PREC_FP64_TC).

Each operand row is cut into 8 exact 7-bit slices after a power-of-two row
scaling; 36 slice products per FP64 product are summed exactly in FP32 per 512
of K and combined in FP64.  The error bound checked is elementwise against
sum_k |A_ik||B_kj| (the scale of an FP64 GEMM's own rounding): 2e-14, with the
plain FP64 GEMM of the same data held to the same bound for comparison.  The
reference products are formed in extended precision (NumPy longdouble).
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TC = 2


def _lib():
    from chemtensor_mojo_gb300 import _lib as L
    return L


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def _p(t):
    return C.c_void_p(t.data_ptr())


@pytest.fixture(scope="module")
def handle():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    L = _lib()
    lib = L.load()
    torch.cuda.set_device(0)
    h = C.c_void_p()
    L.check(lib.ct_create(0, None, C.byref(h)), "ct_create")
    yield lib, h
    lib.ct_destroy(h)


def _gemm(lib, h, prec, A, B, trans_a, trans_b, alpha=1.0, beta=0.0, C0=None):
    L = _lib()
    opA = A.T if trans_a else A
    opB = B.T if trans_b else B
    m, k = opA.shape
    n = opB.shape[1]
    dA, dB = _dev(A), _dev(B)
    dC = _dev(C0 if C0 is not None else np.zeros((m, n)))
    L.check(lib.ct_gemm(h, prec, trans_a, trans_b, m, n, k, C.c_double(alpha), _p(dA), A.shape[1], _p(dB),
                        B.shape[1], C.c_double(beta), _p(dC), n), "ct_gemm")
    # the handle's own stream: wait for it before reading C, and check the device status word
    L.check(lib.ct_synchronize(h), "ct_synchronize")
    st = C.c_int()
    L.check(lib.ct_get_status(h, C.byref(st)), "ct_get_status")
    assert st.value == 0
    return dC.cpu().numpy()


def _ref(A, B, trans_a, trans_b, alpha=1.0, beta=0.0, C0=None):
    opA = (A.T if trans_a else A).astype(np.longdouble)
    opB = (B.T if trans_b else B).astype(np.longdouble)
    r = alpha * (opA @ opB)
    if C0 is not None:
        r = r + beta * C0.astype(np.longdouble)
    scale = np.abs(alpha) * (np.abs(A.T if trans_a else A) @ np.abs(B.T if trans_b else B))
    if C0 is not None:
        scale = scale + abs(beta) * np.abs(C0)
    return r, scale


@pytest.mark.parametrize("m,n,k,ta,tb", [(1, 1, 1, 0, 0), (5, 7, 3, 0, 1), (128, 32, 32, 0, 0),
                                         (200, 100, 300, 1, 0), (130, 33, 257, 1, 1), (384, 320, 1000, 0, 1)])
def test_fp64_tc_gemm_matches_extended_precision(handle, m, n, k, ta, tb):
    lib, h = handle
    rng = np.random.default_rng(m * 1000 + n * 10 + k)
    A = rng.standard_normal((k, m) if ta else (m, k))
    B = rng.standard_normal((n, k) if tb else (k, n))
    got = _gemm(lib, h, FP64_TC, A, B, ta, tb)
    ref, scale = _ref(A, B, ta, tb)
    err = np.abs(got - ref.astype(np.float64)) / scale
    assert err.max() <= 2e-14
    plain = _gemm(lib, h, 0, A, B, ta, tb)
    assert (np.abs(plain - ref.astype(np.float64)) / scale).max() <= 2e-14


def test_fp64_tc_gemm_graded_and_zero_rows(handle):
    """Rows spanning 1e-150..1e150, columns decaying over 40 orders inside a row, an all-zero
    row of A and of B, alpha and beta: the power-of-two row scaling keeps every row's own
    relative accuracy."""
    lib, h = handle
    rng = np.random.default_rng(3)
    m, n, k = 150, 70, 400
    A = rng.standard_normal((m, k)) * 10.0 ** rng.uniform(-150, 150, (m, 1)) * np.exp(-0.23 * np.arange(k))
    B = rng.standard_normal((n, k)) * 10.0 ** rng.uniform(-20, 20, (n, 1))
    A[17] = 0.0
    B[3] = 0.0
    C0 = rng.standard_normal((m, n)) * (np.abs(A) @ np.abs(B).T)
    got = _gemm(lib, h, FP64_TC, A, B, 0, 1, alpha=-0.75, beta=0.5, C0=C0)
    ref, scale = _ref(A, B, 0, 1, alpha=-0.75, beta=0.5, C0=C0)
    scale = np.where(scale > 0, scale, 1.0)
    assert np.all(np.isfinite(got))
    assert (np.abs(got - ref.astype(np.float64)) / scale).max() <= 2e-14
    assert np.all(got[17] == 0.5 * C0[17])


def test_fp64_tc_gemm_gram_of_nearly_dependent_rows(handle):
    """The Gram matrix Z Z^T of rows that are nearly parallel (the subspace split's first
    CholeskyQR pass): its Cholesky pivots are ~1e-10 and survive only with FP64-level
    products.  The smallest pivot agrees with the one from the extended-precision Gram to
    1e-3 relative."""
    lib, h = handle
    rng = np.random.default_rng(11)
    c, ln = 64, 512
    base = rng.standard_normal((8, ln))
    Z = rng.standard_normal((c, 8)) @ base + 1e-5 * rng.standard_normal((c, ln))
    Z /= np.linalg.norm(Z, axis=1, keepdims=True)
    G = _gemm(lib, h, FP64_TC, Z, Z, 0, 1)
    Gr, scale = _ref(Z, Z, 0, 1)
    assert (np.abs(G - Gr.astype(np.float64)) / scale).max() <= 2e-14
    piv = np.diag(np.linalg.cholesky(0.5 * (G + G.T))) ** 2
    piv_r = np.diag(np.linalg.cholesky(Gr.astype(np.float64))) ** 2
    assert piv_r.min() < 1e-8
    assert abs(piv.min() - piv_r.min()) <= 1e-3 * piv_r.min()


def test_expectation_fp64_tc_matches_fp64(ctx):
    """<psi|H|psi> / <psi|psi> of a 14-site Heisenberg chain state with bonds up to 128 (environment
    GEMMs above the tensor-core threshold): the FP64 tensor-core chain agrees with the FP64 SIMT
    chain to 1e-13 relative."""
    import chemtensor_mojo_gb300 as ct
    from oracle import dmrg as od
    from oracle import hamiltonians as oh
    L = 14
    arrays, _ = ct.random_mps_c_compatible_arrays(L, 2, 128, 5)
    sites = od.right_normalize(arrays)
    mpo_a = oh.spin_half_xxz(L, 1.0)
    mps = ct.mps_from_arrays(ctx, sites)
    mpo = ct.mpo_from_arrays(ctx, mpo_a)
    e64 = ct.expectation_value_normalized(mps, mpo, ctx, prec="fp64")
    etc = ct.expectation_value_normalized(mps, mpo, ctx, prec="fp64_tc")
    assert abs(etc - e64) <= 1e-13 * abs(e64)
