"""Environment contractions (src/state/environments.mojo) through the C ABI.

* ``update_left_environment``     environments.mojo:99-201
* ``update_right_environment``    environments.mojo:309-417
* ``build_right_environments``    environments.mojo:420-472
* ``expectation_value[_normalized]`` environments.mojo:475-532
* ``update_left_environment_two_mps`` environments.mojo:535-590
* ``expectation_value_two_mps``       environments.mojo:698-730
* ``mps_vdot_direct`` / ``mps_overlap`` environments.mojo:971-1025
* ``variance``                        environments.mojo:1071-1083
* ``mpo_compose``                     environments.mojo:1086-1132
* ``apply_mpo``                       environments.mojo:1135-1189
"""
from __future__ import annotations

import ctypes as C
from typing import List

import numpy as np
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


def expectation_value(mps: MatrixProductState, mpo: MatrixProductOperator, ctx: DeviceContext | None = None,
                      prec: str = "fp64"):
    """<psi|H|psi> (not normalised), environments.mojo:475-500.  prec "fp64_tc": the
    environment GEMMs on the BF16 tensor cores with FP64-accurate slicing."""
    ctx = ctx or get_context()
    e = C.c_double()
    mpo_pp, mps_pp, keep = _mps_mpo_pointers(mps, mpo)
    ctx.call("ct_mps_expectation", _lib.PRECISIONS[prec], mps.num_sites(), mps.physical_dim,
             _lib.i64_array(mpo.bond_dims), mpo_pp, _lib.i64_array(mps.bond_dims), mps_pp, C.byref(e), None)
    return e.value


def expectation_value_normalized(mps: MatrixProductState, mpo: MatrixProductOperator,
                                 ctx: DeviceContext | None = None, prec: str = "fp64") -> float:
    """<psi|H|psi> / <psi|psi>, environments.mojo:503-532 (prec as in expectation_value)."""
    ctx = ctx or get_context()
    e = C.c_double()
    n = C.c_double()
    mpo_pp, mps_pp, keep = _mps_mpo_pointers(mps, mpo)
    ctx.call("ct_mps_expectation", _lib.PRECISIONS[prec], mps.num_sites(), mps.physical_dim,
             _lib.i64_array(mpo.bond_dims), mpo_pp, _lib.i64_array(mps.bond_dims), mps_pp, C.byref(e), C.byref(n))
    return e.value / n.value


def update_left_environment_two_mps(L_prev: DenseTensor, A_bra: MPSSite, A_ket: MPSSite, W_site: MPOSite,
                                    ctx: DeviceContext | None = None) -> DenseTensor:
    """L_next[wR,Dr,Dr'] = sum L[wL,Dl,Dl'] A_ket[Dl,s,Dr] W[wL,s,s',wR] A_bra[Dl',s',Dr'] (FP64)."""
    ctx = ctx or get_context()
    wL, Dlk, Dlb = L_prev.shape
    Dlk2, d, Drk = A_ket.tensor.shape
    Dlb2, d2, Drb = A_bra.tensor.shape
    Wl, s_in, s_out, wR = W_site.tensor.shape
    if Dlk != Dlk2 or Dlb != Dlb2 or Wl != wL or s_in != d or s_out != d or d2 != d:
        raise ValueError("update_left_environment_two_mps: shape mismatch")
    out = torch.empty(wR * Drk * Drb, dtype=torch.float64, device=ctx.torch_device)
    ctx.call("ct_env_left2", _lib.CT_PREC_FP64, _ptr(L_prev.storage), _ptr(A_ket.tensor.storage),
             _ptr(A_bra.tensor.storage), _ptr(W_site.tensor.storage), _ptr(out), C.c_int64(Dlk), C.c_int64(Dlb),
             C.c_int64(d), C.c_int64(Drk), C.c_int64(Drb), C.c_int64(wL), C.c_int64(wR))
    return DenseTensor(out, [wR, Drk, Drb])


def _states_pointers(bra: MatrixProductState, ket: MatrixProductState):
    bra_pp, k1 = _lib.ptr_array([s.tensor.storage.data_ptr() for s in bra.sites])
    ket_pp, k2 = _lib.ptr_array([s.tensor.storage.data_ptr() for s in ket.sites])
    return bra_pp, ket_pp, (k1, k2)


def expectation_value_two_mps(mps_bra: MatrixProductState, mpo: MatrixProductOperator, mps_ket: MatrixProductState,
                              ctx: DeviceContext | None = None) -> float:
    """<bra|mpo|ket> with different bra and ket (environments.mojo:698-730)."""
    ctx = ctx or get_context()
    N = mps_bra.num_sites()
    if mpo.num_sites() != N or mps_ket.num_sites() != N:
        raise ValueError("expectation_value_two_mps: length mismatch")
    v = C.c_double()
    bra_pp, ket_pp, keep = _states_pointers(mps_bra, mps_ket)
    mpo_pp, k3 = _lib.ptr_array([s.tensor.storage.data_ptr() for s in mpo.sites])
    ctx.call("ct_mps_expectation2", _lib.CT_PREC_FP64, N, mps_ket.physical_dim, _lib.i64_array(mpo.bond_dims),
             mpo_pp, _lib.i64_array(mps_bra.bond_dims), bra_pp, _lib.i64_array(mps_ket.bond_dims), ket_pp,
             C.byref(v))
    return v.value


def mps_vdot_direct(bra: MatrixProductState, ket: MatrixProductState, ctx: DeviceContext | None = None) -> float:
    """<bra|ket> by the two-GEMM transfer step, no MPO (environments.mojo:971-1016)."""
    ctx = ctx or get_context()
    N = bra.num_sites()
    if ket.num_sites() != N:
        raise ValueError("mps_vdot_direct: length mismatch")
    v = C.c_double()
    bra_pp, ket_pp, keep = _states_pointers(bra, ket)
    ctx.call("ct_mps_expectation2", _lib.CT_PREC_FP64, N, ket.physical_dim, None, None,
             _lib.i64_array(bra.bond_dims), bra_pp, _lib.i64_array(ket.bond_dims), ket_pp, C.byref(v))
    return v.value


def mps_overlap(mps_bra: MatrixProductState, mps_ket: MatrixProductState, ctx: DeviceContext | None = None) -> float:
    """environments.mojo:1018-1025."""
    return mps_vdot_direct(mps_bra, mps_ket, ctx)


def mpo_compose(mpo_a: MatrixProductOperator, mpo_b: MatrixProductOperator,
                ctx: DeviceContext | None = None) -> MatrixProductOperator:
    """W[(al,bl),i,o,(ar,br)] = sum_m Wa[al,i,m,ar] Wb[bl,m,o,br] per site (environments.mojo:1086-1132)."""
    ctx = ctx or get_context()
    N = mpo_a.num_sites()
    if mpo_b.num_sites() != N:
        raise ValueError("MPO compose: length mismatch")
    sites = []
    for i in range(N):
        wLa, d_in, d_mid, wRa = mpo_a.sites[i].tensor.shape
        wLb, d_mid2, d_out, wRb = mpo_b.sites[i].tensor.shape
        if d_mid2 != d_mid:
            raise ValueError(f"MPO compose: physical dim mismatch at site {i}")
        shape = [wLa * wLb, d_in, d_out, wRa * wRb]
        out = torch.empty(int(np.prod(shape)), dtype=torch.float64, device=ctx.torch_device)
        ctx.call("ct_mpo_compose_site", _ptr(mpo_a.sites[i].tensor.storage), _ptr(mpo_b.sites[i].tensor.storage),
                 _ptr(out), C.c_int64(wLa), C.c_int64(d_in), C.c_int64(d_mid), C.c_int64(wRa), C.c_int64(wLb),
                 C.c_int64(d_out), C.c_int64(wRb))
        sites.append(MPOSite(DenseTensor(out, shape)))
    return MatrixProductOperator(sites)


def variance(mps: MatrixProductState, mpo: MatrixProductOperator, ctx: DeviceContext | None = None) -> float:
    """<H^2> - <H>^2 with H^2 = mpo_compose(H, H) (environments.mojo:1071-1083)."""
    ctx = ctx or get_context()
    E = expectation_value_normalized(mps, mpo, ctx)
    E2 = expectation_value_normalized(mps, mpo_compose(mpo, mpo, ctx), ctx)
    return E2 - E * E


def apply_mpo(mpo: MatrixProductOperator, mps: MatrixProductState,
              ctx: DeviceContext | None = None) -> MatrixProductState:
    """|out> = O|mps>, site shapes [wL*Dl, d_out, wR*Dr] (environments.mojo:1135-1189)."""
    ctx = ctx or get_context()
    N = mps.num_sites()
    if mpo.num_sites() != N:
        raise ValueError("apply_mpo: MPS and MPO must have same number of sites")
    sites = []
    for i in range(N):
        Dl, d, Dr = mps.sites[i].tensor.shape
        wL, d_in, d_out, wR = mpo.sites[i].tensor.shape
        if d_in != d:
            raise ValueError(f"apply_mpo: physical dim mismatch at site {i}")
        shape = [wL * Dl, d_out, wR * Dr]
        out = torch.empty(int(np.prod(shape)), dtype=torch.float64, device=ctx.torch_device)
        ctx.call("ct_apply_mpo_site", _ptr(mps.sites[i].tensor.storage), _ptr(mpo.sites[i].tensor.storage),
                 _ptr(out), C.c_int64(Dl), C.c_int64(d), C.c_int64(Dr), C.c_int64(wL), C.c_int64(d_out),
                 C.c_int64(wR))
        sites.append(MPSSite(DenseTensor(out, shape)))
    return MatrixProductState(sites)
