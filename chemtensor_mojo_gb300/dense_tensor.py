"""Dense tensor core: the host side of src/m_tensor/dense_tensor.mojo.

``DenseTensor`` holds a contiguous FP64 CUDA buffer (a torch tensor used only
as device memory) plus a row-major shape; every operation on it calls
libctdmrg through the C ABI.  Names, argument meaning and error behaviour
follow the reference:

* ``DenseTensor``                 dense_tensor.mojo:264-763
* ``create_dense_tensor*``        dense_tensor.mojo:815-961
* ``dense_tensor_dot``            dense_tensor.mojo:963-1328 (axis inference,
                                  aligned pairing, leading/trailing ranges)
* ``dense_tensor_svd_trunc``      dense_tensor.mojo:1595-1623 (device Jacobi SVD
                                  instead of the host LAPACK round trip)
"""
from __future__ import annotations

import ctypes as C
import math
import threading
from typing import List, Sequence

import numpy as np
import torch

from . import _lib
from ._lib import check

_ctx_lock = threading.Lock()
_contexts = {}


class DeviceContext:
    """One libctdmrg handle per (device, host thread), bound to torch's stream.

    Mirrors the role of MAX's ``DeviceContext`` in the reference signatures.
    """

    def __init__(self, device: int | None = None):
        if not torch.cuda.is_available():
            raise RuntimeError("chemtensor_mojo_gb300 needs a CUDA device (there is no CPU fallback)")
        self.lib = _lib.load()
        self.device = torch.cuda.current_device() if device is None else int(device)
        self.torch_device = torch.device("cuda", self.device)
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            check(self.lib.ct_create(self.device, C.c_void_p(self._torch_stream()), C.byref(h)), "ct_create")
        self.handle = h
        self._bound = self._torch_stream()

    def _torch_stream(self) -> int:
        s = torch.cuda.current_stream(self.device).cuda_stream
        return s if s != 0 else 1  # 1 = cudaStreamLegacy (torch's default stream)

    def bind(self) -> "DeviceContext":
        s = self._torch_stream()
        if s != self._bound:
            check(self.lib.ct_set_stream(self.handle, C.c_void_p(s)), "ct_set_stream", self.handle)
            self._bound = s
        return self

    def call(self, name: str, *args):
        self.bind()
        st = getattr(self.lib, name)(self.handle, *args)
        check(st, name, self.handle)

    def synchronize(self):
        self.call("ct_synchronize")

    def workspace_bytes(self) -> int:
        v = C.c_int64()
        self.call("ct_workspace_bytes", C.byref(v))
        return v.value

    def set_workspace_limit(self, nbytes: int):
        self.call("ct_set_workspace_limit", C.c_int64(int(nbytes)))

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            if getattr(self, "handle", None):
                self.lib.ct_destroy(self.handle)
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False


def get_context(device: int | None = None) -> DeviceContext:
    dev = torch.cuda.current_device() if device is None else int(device)
    key = (dev, threading.get_ident())
    with _ctx_lock:
        ctx = _contexts.get(key)
        if ctx is None:
            ctx = DeviceContext(dev)
            _contexts[key] = ctx
        return ctx


def _ptr(t: torch.Tensor) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


def compute_row_major_strides(shape: Sequence[int]) -> List[int]:
    st = [1] * len(shape)
    for i in range(len(shape) - 2, -1, -1):
        st[i] = st[i + 1] * int(shape[i + 1])
    return st


class DenseTensor:
    """Contiguous row-major FP64 tensor on the device (dense_tensor.mojo:264-310)."""

    def __init__(self, storage: torch.Tensor, shape: Sequence[int]):
        if storage.dtype != torch.float64 or not storage.is_cuda:
            raise TypeError("DenseTensor storage must be a CUDA float64 tensor")
        n = int(np.prod(shape)) if len(shape) else 1
        if storage.numel() < n:
            raise ValueError("storage smaller than shape")
        self.storage = storage.reshape(-1)[:n] if storage.numel() != n else storage.reshape(-1)
        self.shape = [int(s) for s in shape]

    # -- views and properties ------------------------------------------------
    @property
    def size(self) -> int:
        return int(np.prod(self.shape)) if self.shape else 1

    @property
    def stride(self) -> List[int]:
        return compute_row_major_strides(self.shape)

    def rank(self) -> int:
        return len(self.shape)

    def reshape(self, shape: Sequence[int]) -> "DenseTensor":
        """Zero-copy view (dense_tensor.mojo:614-635)."""
        if int(np.prod(shape)) != self.size:
            raise ValueError("reshape: total size must be preserved")
        return DenseTensor(self.storage, shape)

    def flatten_dims(self, start: int, end: int) -> "DenseTensor":
        """Merge axes [start, end) into one (dense_tensor.mojo:547-612)."""
        s = self.shape
        merged = int(np.prod(s[start:end]))
        return self.reshape(s[:start] + [merged] + s[end:])

    def transpose(self, perm: Sequence[int], ctx: DeviceContext | None = None) -> "DenseTensor":
        """Physical permute into a new buffer (dense_tensor.mojo:460-545)."""
        ctx = ctx or get_context()
        perm = [int(p) for p in perm]
        if sorted(perm) != list(range(len(self.shape))):
            raise ValueError("transpose: invalid permutation")
        out = torch.empty(self.size, dtype=torch.float64, device=self.storage.device)
        shp = _lib.i64_array(self.shape)
        prm = (C.c_int32 * len(perm))(*perm)
        ctx.call("ct_permute", _ptr(self.storage), _ptr(out), len(perm), shp, prm)
        return DenseTensor(out, [self.shape[p] for p in perm])

    # -- reductions / BLAS-1 (dense_tensor.mojo:637-754) -----------------------
    def norm_sq(self, ctx: DeviceContext | None = None) -> float:
        ctx = ctx or get_context()
        r = C.c_double()
        ctx.call("ct_vec_norm_sq", C.c_int64(self.size), _ptr(self.storage), C.byref(r))
        return r.value

    def norm(self, ctx: DeviceContext | None = None) -> float:
        return math.sqrt(self.norm_sq(ctx))

    def dot_product(self, other: "DenseTensor", ctx: DeviceContext | None = None) -> float:
        if other.size != self.size:
            raise ValueError("dot_product: size mismatch")
        ctx = ctx or get_context()
        r = C.c_double()
        ctx.call("ct_vec_dot", C.c_int64(self.size), _ptr(self.storage), _ptr(other.storage), C.byref(r))
        return r.value

    def axpy_in_place(self, alpha: float, x: "DenseTensor", ctx: DeviceContext | None = None) -> None:
        if x.size != self.size:
            raise ValueError("axpy_in_place: size mismatch")
        ctx = ctx or get_context()
        ctx.call("ct_vec_axpy", C.c_int64(self.size), C.c_double(alpha), _ptr(x.storage), _ptr(self.storage))

    def scale_in_place(self, s: float, ctx: DeviceContext | None = None) -> None:
        ctx = ctx or get_context()
        ctx.call("ct_vec_scale", C.c_int64(self.size), C.c_double(s), _ptr(self.storage))

    def copy(self) -> "DenseTensor":
        return DenseTensor(self.storage.clone(), self.shape)

    def to_numpy(self) -> np.ndarray:
        return self.storage.detach().cpu().numpy().reshape(self.shape)

    def __repr__(self) -> str:
        return f"DenseTensor(shape={self.shape})"


# -- creators (dense_tensor.mojo:815-961) ------------------------------------------
def _device(ctx: DeviceContext | None):
    return (ctx or get_context()).torch_device


def create_dense_tensor(ctx, shape: Sequence[int], init_value: float = 0.0) -> DenseTensor:
    n = int(np.prod(shape)) if len(shape) else 1
    return DenseTensor(torch.full((n,), float(init_value), dtype=torch.float64, device=_device(ctx)), shape)


def create_dense_tensor_uninitialized(ctx, shape: Sequence[int]) -> DenseTensor:
    n = int(np.prod(shape)) if len(shape) else 1
    return DenseTensor(torch.empty(n, dtype=torch.float64, device=_device(ctx)), shape)


def create_dense_tensor_from_data(ctx, data, shape: Sequence[int]) -> DenseTensor:
    a = np.ascontiguousarray(np.asarray(data, dtype=np.float64).reshape(-1))
    if a.size != int(np.prod(shape)):
        raise ValueError("data size does not match shape")
    return DenseTensor(torch.from_numpy(a).to(_device(ctx)), shape)


def create_dense_tensor_random(ctx, shape: Sequence[int], seed: int = 0) -> DenseTensor:
    """Seeded N(0,1) entries (the reference's DenseTensor.random is unseeded uniform)."""
    g = torch.Generator(device="cpu").manual_seed(int(seed))
    n = int(np.prod(shape))
    return DenseTensor(torch.randn(n, generator=g, dtype=torch.float64).to(_device(ctx)), shape)


# -- tensordot (dense_tensor.mojo:963-1328) ------------------------------------------
def dense_tensor_dot(C_out: DenseTensor, A: DenseTensor, B: DenseTensor, ctx: DeviceContext | None = None,
                     ndim_mult: int = 1, axrange_A: bool = False, axrange_B: bool = False,
                     prec: str = "fp64") -> None:
    """Generalised tensordot into a pre-allocated C.

    Contracts ``ndim_mult`` axes of A (leading if ``axrange_A`` else trailing)
    with ``ndim_mult`` axes of B (leading if ``axrange_B`` else trailing), in
    aligned order.  When both flags are False, B's side is inferred (leading
    preferred) exactly as dense_tensor.mojo:1141-1159 does.  The transposes
    the reference materialises are folded into the GEMM's operand strides.
    """
    ctx = ctx or get_context()
    rA, rB = len(A.shape), len(B.shape)
    if ndim_mult < 1 or rA < ndim_mult or rB < ndim_mult:
        raise ValueError("Invalid ndim_mult")
    eff_B = axrange_B
    if not axrange_A and not axrange_B:
        lead = all(A.shape[rA - ndim_mult + i] == B.shape[i] for i in range(ndim_mult))
        trail = all(A.shape[rA - ndim_mult + i] == B.shape[rB - ndim_mult + i] for i in range(ndim_mult))
        eff_B = True if lead else (False if trail else True)
    for i in range(ndim_mult):
        ax_a = (0 if axrange_A else rA - ndim_mult) + i
        ax_b = (0 if eff_B else rB - ndim_mult) + i
        if A.shape[ax_a] != B.shape[ax_b]:
            raise ValueError("Dim mismatch")
    if axrange_A:
        k_dims, a_free = A.shape[:ndim_mult], A.shape[ndim_mult:]
    else:
        k_dims, a_free = A.shape[rA - ndim_mult:], A.shape[:rA - ndim_mult]
    b_free = B.shape[ndim_mult:] if eff_B else B.shape[:rB - ndim_mult]
    m = int(np.prod(a_free)) if a_free else 1
    n = int(np.prod(b_free)) if b_free else 1
    k = int(np.prod(k_dims))
    expected = list(a_free) + list(b_free)
    if not expected:
        if C_out.shape not in ([], [1]):
            raise ValueError("Output tensor C for scalar result must be [] or [1]")
    elif list(C_out.shape) != expected:
        raise ValueError(f"Output tensor C has wrong shape: expected {expected} got {C_out.shape}")
    # A_flat is [m, k] (trailing) or [k, m] (leading -> op = transpose)
    trans_a = 1 if axrange_A else 0
    lda = m if axrange_A else k
    # B_flat is [k, n] (leading) or [n, k] (trailing -> op = transpose)
    trans_b = 0 if eff_B else 1
    ldb = n if eff_B else k
    ctx.call("ct_gemm", _lib.PRECISIONS[prec], trans_a, trans_b, C.c_int64(m), C.c_int64(n), C.c_int64(k),
             C.c_double(1.0), _ptr(A.storage), C.c_int64(lda), _ptr(B.storage), C.c_int64(ldb), C.c_double(0.0),
             _ptr(C_out.storage), C.c_int64(n))


def dense_tensor_qr(tensor: DenseTensor, ctx: DeviceContext | None = None):
    """Thin QR on the device (dense_tensor.mojo:1333-1433) -> (Q [m,k], R [k,n]), k = min(m,n).

    FP64.  diag(R) >= 0; LAPACK's Householder factors equal these up to the signs of Q's
    columns and R's rows.  A rank-2 tensor is required, as in the reference."""
    ctx = ctx or get_context()
    if len(tensor.shape) != 2:
        raise ValueError(f"QR decomposition requires a 2D matrix, got rank {len(tensor.shape)}")
    m, n = tensor.shape
    k = min(m, n)
    dev = tensor.storage.device
    Q = torch.empty(max(m * k, 1), dtype=torch.float64, device=dev)
    R = torch.empty(max(k * n, 1), dtype=torch.float64, device=dev)
    done = C.c_int()
    ctx.call("ct_qr", _ptr(tensor.storage), C.c_int64(m), C.c_int64(n), _ptr(Q), _ptr(R), C.byref(done))
    return DenseTensor(Q[:m * k], [m, k]), DenseTensor(R[:k * n], [k, n])


def dense_tensor_svd_trunc(tensor: DenseTensor, ctx: DeviceContext | None = None, chi_max: int = 1 << 30,
                           eps_trunc: float = 1e-12):
    """Truncated thin SVD of a 2-D tensor on the device -> (U, S, Vt, chi_kept)."""
    ctx = ctx or get_context()
    if len(tensor.shape) != 2:
        raise ValueError("dense_tensor_svd_trunc expects a matrix")
    m, n = tensor.shape
    k = min(m, n)
    dev = tensor.storage.device
    U = torch.empty(max(m * k, 1), dtype=torch.float64, device=dev)
    S = torch.empty(max(k, 1), dtype=torch.float64, device=dev)
    Vt = torch.empty(max(k * n, 1), dtype=torch.float64, device=dev)
    chi = C.c_int64()
    ctx.call("ct_svd_trunc", _ptr(tensor.storage), C.c_int64(m), C.c_int64(n), C.c_int64(chi_max),
             C.c_double(eps_trunc), _ptr(U), _ptr(S), _ptr(Vt), C.byref(chi))
    c = chi.value
    return (DenseTensor(U[:m * c], [m, c]), DenseTensor(S[:c], [c]), DenseTensor(Vt[:c * n], [c, n]), c)
