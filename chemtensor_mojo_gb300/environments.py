"""Environment contractions (src/state/environments.mojo) through the C ABI.

* ``update_left_environment``     environments.mojo:99-201
* ``update_right_environment``    environments.mojo:309-417
* ``build_right_environments``    environments.mojo:420-472
* ``expectation_value[_normalized]`` environments.mojo:475-532
"""
from __future__ import annotations

import ctypes as C
from typing import List

import torch

from . import _lib
from .dense_tensor import DenseTensor, DeviceContext, get_context, _ptr
from .mps_state import MatrixProductOperator, MatrixProductState, MPOSite, MPSSite


def _prec(prec: str) -> int:
    return _lib.PRECISIONS[prec]


def create_identity_environment(ctx, w: int, D: int) -> DenseTensor:
    ctx = ctx or get_context()
    out = torch.empty(w * D * D, dtype=torch.float64, device=ctx.torch_device)
    ctx.call("ct_env_identity", _ptr(out), C.c_int64(w), C.c_int64(D))
    return DenseTensor(out, [w, D, D])


def update_left_environment(L_prev: DenseTensor, A_site: MPSSite, W_site: MPOSite,
                            ctx: DeviceContext | None = None, prec: str = "fp64") -> DenseTensor:
    """L_next[wR,Dr,Dr'] = sum L[wL,Dl,Dl'] A[Dl,s,Dr] W[wL,s,s',wR] A[Dl',s',Dr']."""
    ctx = ctx or get_context()
    wL, Dl, Dl2 = L_prev.shape
    Dla, d, Dr = A_site.tensor.shape
    Wl, s_in, s_out, wR = W_site.tensor.shape
    if Dl != Dla or Dl2 != Dla or Wl != wL or s_in != d or s_out != d:
        raise ValueError("update_left_environment: shape mismatch")
    out = torch.empty(wR * Dr * Dr, dtype=torch.float64, device=ctx.torch_device)
    ctx.call("ct_env_left", _prec(prec), _ptr(L_prev.storage), _ptr(A_site.tensor.storage),
             _ptr(W_site.tensor.storage), _ptr(out), C.c_int64(Dl), C.c_int64(d), C.c_int64(Dr), C.c_int64(wL),
             C.c_int64(wR))
    return DenseTensor(out, [wR, Dr, Dr])


def update_right_environment(R_next: DenseTensor, A_site: MPSSite, W_site: MPOSite,
                             ctx: DeviceContext | None = None, prec: str = "fp64") -> DenseTensor:
    """R_prev[wL,Dl,Dl'] = sum R[wR,Dr,Dr'] A[Dl,s,Dr] W[wL,s,s',wR] A[Dl',s',Dr']."""
    ctx = ctx or get_context()
    wR, Dr, Dr2 = R_next.shape
    Dl, d, Dra = A_site.tensor.shape
    wL, s_in, s_out, Wr = W_site.tensor.shape
    if Dr != Dra or Dr2 != Dra or Wr != wR or s_in != d or s_out != d:
        raise ValueError("update_right_environment: shape mismatch")
    out = torch.empty(wL * Dl * Dl, dtype=torch.float64, device=ctx.torch_device)
    ctx.call("ct_env_right", _prec(prec), _ptr(R_next.storage), _ptr(A_site.tensor.storage),
             _ptr(W_site.tensor.storage), _ptr(out), C.c_int64(Dl), C.c_int64(d), C.c_int64(Dr), C.c_int64(wL),
             C.c_int64(wR))
    return DenseTensor(out, [wL, Dl, Dl])


def build_right_environments(mps: MatrixProductState, mpo: MatrixProductOperator,
                             ctx: DeviceContext | None = None, prec: str = "fp64") -> List[DenseTensor]:
    ctx = ctx or get_context()
    N = mps.num_sites()
    envs: List[DenseTensor] = [None] * (N + 1)
    envs[N] = create_identity_environment(ctx, mpo.bond_dimension(N), mps.bond_dimension(N))
    for i in range(N - 1, -1, -1):
        envs[i] = update_right_environment(envs[i + 1], mps.sites[i], mpo.sites[i], ctx, prec)
    return envs


def _mps_mpo_pointers(mps: MatrixProductState, mpo: MatrixProductOperator):
    mpo_pp, k1 = _lib.ptr_array([s.tensor.storage.data_ptr() for s in mpo.sites])
    mps_pp, k2 = _lib.ptr_array([s.tensor.storage.data_ptr() for s in mps.sites])
    return mpo_pp, mps_pp, (k1, k2)


def expectation_value(mps: MatrixProductState, mpo: MatrixProductOperator, ctx: DeviceContext | None = None):
    """<psi|H|psi> (not normalised), environments.mojo:475-500."""
    ctx = ctx or get_context()
    e = C.c_double()
    mpo_pp, mps_pp, keep = _mps_mpo_pointers(mps, mpo)
    ctx.call("ct_mps_expectation", _lib.CT_PREC_FP64, mps.num_sites(), mps.physical_dim,
             _lib.i64_array(mpo.bond_dims), mpo_pp, _lib.i64_array(mps.bond_dims), mps_pp, C.byref(e), None)
    return e.value


def expectation_value_normalized(mps: MatrixProductState, mpo: MatrixProductOperator,
                                 ctx: DeviceContext | None = None) -> float:
    """<psi|H|psi> / <psi|psi>, environments.mojo:503-532."""
    ctx = ctx or get_context()
    e = C.c_double()
    n = C.c_double()
    mpo_pp, mps_pp, keep = _mps_mpo_pointers(mps, mpo)
    ctx.call("ct_mps_expectation", _lib.CT_PREC_FP64, mps.num_sites(), mps.physical_dim,
             _lib.i64_array(mpo.bond_dims), mpo_pp, _lib.i64_array(mps.bond_dims), mps_pp, C.byref(e), C.byref(n))
    return e.value / n.value
