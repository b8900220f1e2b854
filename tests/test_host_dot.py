"""dense_tensor_dot's host logic on the CPU (no device): axis pairing, the leading/trailing
inference of dense_tensor.mojo:1141-1167, output shapes and the ct_gemm arguments it derives.

The C ABI call is replaced by a stand-in context whose ``ct_gemm`` applies the documented
contract (row-major C[m,n] = alpha op(A) op(B) + beta C with leading dimensions lda, ldb, ldc)
with NumPy, so every case of the reference's test_dense_tensor_dot.mojo (DT-DOT-001 to 008) is
checked against the aligned-pairing tensordot without a GPU.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from chemtensor_mojo_gb300 import dense_tensor as dtm


class FakeCtx:
    """Resolves the pointers ct_gemm receives to the CPU arrays behind them."""

    def __init__(self):
        self.arrays = {}
        self.calls = []

    def tensor(self, a, shape):
        t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64).reshape(-1).copy())
        d = dtm.DenseTensor.__new__(dtm.DenseTensor)
        d.storage = t
        d.shape = [int(s) for s in shape]
        self.arrays[t.data_ptr()] = t.numpy()
        return d

    def call(self, name, *args):
        assert name == "ct_gemm"
        prec, ta, tb, m, n, k, alpha, pa, lda, pb, ldb, beta, pc, ldc = args
        v = lambda x: x.value if hasattr(x, "value") else x  # noqa: E731
        m, n, k, lda, ldb, ldc = (v(x) for x in (m, n, k, lda, ldb, ldc))
        A, B, Cm = self.arrays[v(pa)], self.arrays[v(pb)], self.arrays[v(pc)]
        Am = A[: (k if ta else m) * lda].reshape(k if ta else m, lda)[:, : (m if ta else k)]
        Bm = B[: (n if tb else k) * ldb].reshape(n if tb else k, ldb)[:, : (k if tb else n)]
        opA = Am.T if ta else Am
        opB = Bm.T if tb else Bm
        Cv = Cm[: m * ldc].reshape(m, ldc)[:, :n]
        Cv[...] = v(alpha) * (opA @ opB) + v(beta) * Cv
        self.calls.append(dict(ta=ta, tb=tb, m=m, n=n, k=k, lda=lda, ldb=ldb, ldc=ldc))


def expected(A, B, nm, axrange_A, axrange_B):
    """aligned (non-reversed) pairing: A[offA + i] <-> B[offB + i]"""
    offA = 0 if axrange_A else A.ndim - nm
    offB = 0 if axrange_B else B.ndim - nm
    return np.tensordot(A, B, axes=(list(range(offA, offA + nm)), list(range(offB, offB + nm))))


CASES = [  # (shape A, shape B, ndim_mult, axrange_A, axrange_B, inferred B side when both False)
    ((3, 4), (4, 5), 1, False, True, None),            # DT-DOT-001
    ((3, 4), (4, 5), 1, False, False, True),           # DT-DOT-002: default = B leading
    ((2, 3, 4), (4, 5, 6), 1, False, True, None),      # DT-DOT-003
    ((2, 3, 4, 5), (4, 5, 6, 7), 2, False, True, None),  # DT-DOT-004
    ((4, 3), (4, 5), 1, True, True, None),             # DT-DOT-005A
    ((4, 3), (5, 4), 1, True, False, None),            # DT-DOT-005B
    ((3, 4), (5, 4), 1, False, False, False),          # DT-DOT-005C: inferred B trailing
    ((2, 3, 4, 5), (4, 5, 6, 7), 2, False, False, True),   # DT-DOT-007: inferred B leading
    ((2, 3, 4, 5), (6, 7, 4, 5), 2, False, False, False),  # DT-DOT-008: inferred B trailing
    ((6, 40, 33), (33, 7, 9), 1, False, True, None),
    ((5, 6, 7), (5, 6, 8), 2, True, True, None),
]


@pytest.mark.parametrize("sa,sb,nm,ara,arb,infer", CASES)
def test_reference_dot_cases(sa, sb, nm, ara, arb, infer):
    rng = np.random.default_rng(len(sa) * 31 + len(sb) + nm)
    A = rng.standard_normal(sa)
    B = rng.standard_normal(sb)
    eff_b = arb if (ara or arb) else infer
    ref = expected(A, B, nm, ara, eff_b)
    ctx = FakeCtx()
    out = ctx.tensor(np.zeros(ref.shape), list(ref.shape))
    dtm.dense_tensor_dot(out, ctx.tensor(A, sa), ctx.tensor(B, sb), ctx, ndim_mult=nm, axrange_A=ara,
                         axrange_B=arb)
    np.testing.assert_allclose(out.storage.numpy().reshape(ref.shape), ref, rtol=1e-13, atol=1e-13)
    assert len(ctx.calls) == 1


def test_scalar_result():
    """DT-DOT-006: A [7] . B [7] -> scalar stored in a [1] tensor."""
    rng = np.random.default_rng(6)
    a, b = rng.standard_normal(7), rng.standard_normal(7)
    ctx = FakeCtx()
    out = ctx.tensor(np.zeros(1), [1])
    dtm.dense_tensor_dot(out, ctx.tensor(a, [7]), ctx.tensor(b, [7]), ctx, ndim_mult=1, axrange_A=False,
                         axrange_B=True)
    assert out.storage.numpy()[0] == pytest.approx(float(a @ b), rel=1e-14)


def test_shape_errors():
    ctx = FakeCtx()
    A, B = ctx.tensor(np.ones((3, 4)), [3, 4]), ctx.tensor(np.ones((5, 6)), [5, 6])
    with pytest.raises(ValueError):
        dtm.dense_tensor_dot(ctx.tensor(np.zeros(15), [3, 5]), A, B, ctx)
    B2 = ctx.tensor(np.ones((4, 5)), [4, 5])
    with pytest.raises(ValueError):
        dtm.dense_tensor_dot(ctx.tensor(np.zeros(12), [3, 4]), A, B2, ctx)   # wrong output shape
    with pytest.raises(ValueError):
        dtm.dense_tensor_dot(ctx.tensor(np.zeros(1), [1]), A, B2, ctx, ndim_mult=3)
