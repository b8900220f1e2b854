"""Two-site DMRG (src/algorithms/dmrg.mojo) over the C ABI.

Same names and argument meaning as the reference:

* ``DMRGParams``                  dmrg.mojo:22-36 (+ ``prec``, ``max_rotations``,
                                  ``reorth``: the precision form, the Jacobi
                                  rotation cap of the tridiagonal eigensolve,
                                  FP64 reorthogonalisation)
* ``build_two_site_theta``        dmrg.mojo:93-140
* ``split_two_site_theta_svd``    dmrg.mojo:143-252
* ``apply_two_site_heff``         dmrg.mojo:254-374
* ``dmrg_two_site``               dmrg.mojo:377-483 (runs the native sweep driver)
* ``lanczos_two_site_optimize``   dmrg.mojo:486-756
* ``dmrg_local_update_two_site``  dmrg.mojo:759-844
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import List, Optional, Tuple

import torch

from . import _lib
from .dense_tensor import DenseTensor, DeviceContext, get_context, _ptr
from .environments import (build_right_environments, create_identity_environment, update_left_environment,
                           update_right_environment)
from .mps_state import MatrixProductOperator, MatrixProductState, MPOSite, MPSSite

REFERENCE_JACOBI_ROTATIONS = 200   # dmrg.mojo:510


@dataclass
class DMRGParams:
    num_sweeps: int
    chi_max: int
    eps_trunc: float
    max_krylov_iter: int
    krylov_tol: float
    energy_tol: float
    two_site: bool = True
    verbose: int = 0            # 1: per-sweep energies; 2: also every split
    prec: str = "fp64"
    max_rotations: int = REFERENCE_JACOBI_ROTATIONS
    reorth: bool = False
    final_rayleigh: bool = False
    keep_bases: bool = False
    split_power_steps: int = 0   # -1: always the Jacobi SVD split
    cold_power_steps: int = -1   # >= 0: randomized subspace split on first visits

    def to_c(self) -> _lib.ct_dmrg_params:
        return _lib.ct_dmrg_params(int(self.num_sweeps), int(self.chi_max), float(self.eps_trunc),
                                   int(self.max_krylov_iter), float(self.krylov_tol), float(self.energy_tol),
                                   int(bool(self.two_site)), int(self.verbose), _lib.PRECISIONS[self.prec],
                                   int(self.max_rotations), int(bool(self.reorth)), int(bool(self.final_rayleigh)),
                                   int(bool(self.keep_bases)), int(self.split_power_steps),
                                   int(self.cold_power_steps))


@dataclass
class DMRGStats:
    seconds_total: float = 0.0
    seconds_lanczos: float = 0.0
    seconds_svd: float = 0.0
    seconds_env: float = 0.0
    heff_flops: float = 0.0
    env_flops: float = 0.0
    heff_applies: int = 0
    local_updates: int = 0
    max_discarded: float = 0.0
    energy_rayleigh: float = float("nan")
    subspace_splits: int = 0
    exact_splits: int = 0
    seconds_subspace: float = 0.0
    cold_splits: int = 0
    completed_rows: int = 0
    seconds_rayleigh: float = 0.0
    stale_retries: int = 0
    fp64_handovers: int = 0
    sweep_energies: List[float] = field(default_factory=list)
    discarded: List[float] = field(default_factory=list)


def _p(prec: str) -> int:
    return _lib.PRECISIONS[prec]


def build_two_site_theta(A_i: MPSSite, A_ip1: MPSSite, ctx: DeviceContext | None = None) -> DenseTensor:
    ctx = ctx or get_context()
    Dl, d, Dm = A_i.tensor.shape
    Dm2, d2, Dr = A_ip1.tensor.shape
    if Dm2 != Dm:
        raise ValueError("Bond dimension mismatch in build_two_site_theta")
    if d != d2:
        raise ValueError("Physical dimensions must match")
    out = torch.empty(Dl * d * d * Dr, dtype=torch.float64, device=ctx.torch_device)
    ctx.call("ct_theta2", _lib.CT_PREC_FP64, _ptr(A_i.tensor.storage), _ptr(A_ip1.tensor.storage), _ptr(out),
             C.c_int64(Dl), C.c_int64(d), C.c_int64(Dm), C.c_int64(Dr))
    return DenseTensor(out, [Dl, d, d, Dr])


def _heff_dims(theta: DenseTensor, L: DenseTensor, R: DenseTensor, W_i: MPOSite, W_ip1: MPOSite):
    Dl, d, d2, Dr = theta.shape
    wL, Dl1, Dl2 = L.shape
    wR, Dr1, Dr2 = R.shape
    if d != d2 or Dl1 != Dl or Dl2 != Dl or Dr1 != Dr or Dr2 != Dr:
        raise ValueError("apply_two_site_heff: shape mismatch")
    if W_i.tensor.shape[0] != wL or W_ip1.tensor.shape[3] != wR or W_i.tensor.shape[3] != W_ip1.tensor.shape[0]:
        raise ValueError("apply_two_site_heff: MPO bond mismatch")
    return Dl, d, Dr, wL, W_i.tensor.shape[3], wR


def apply_two_site_heff(theta: DenseTensor, L_env: DenseTensor, R_env: DenseTensor, W_i: MPOSite, W_ip1: MPOSite,
                        ctx: DeviceContext | None = None, prec: str = "fp64") -> DenseTensor:
    ctx = ctx or get_context()
    Dl, d, Dr, wL, wM, wR = _heff_dims(theta, L_env, R_env, W_i, W_ip1)
    out = torch.empty(Dl * d * d * Dr, dtype=torch.float64, device=ctx.torch_device)
    ctx.call("ct_heff2_apply", _p(prec), _ptr(theta.storage), _ptr(L_env.storage), _ptr(R_env.storage),
             _ptr(W_i.tensor.storage), _ptr(W_ip1.tensor.storage), _ptr(out), C.c_int64(Dl), C.c_int64(d),
             C.c_int64(Dr), C.c_int64(wL), C.c_int64(wM), C.c_int64(wR))
    return DenseTensor(out, [Dl, d, d, Dr])


@dataclass
class LanczosInfo:
    numiter: int
    alpha: List[float]
    beta: List[float]


def lanczos_two_site_optimize(initial_theta: DenseTensor, L_env: DenseTensor, R_env: DenseTensor, W_i: MPOSite,
                              W_ip1: MPOSite, ctx: DeviceContext | None = None, max_iter: int = 20,
                              tol: float = 1e-10, prec: str = "fp64",
                              max_rotations: int = REFERENCE_JACOBI_ROTATIONS, reorth: bool = False,
                              info: Optional[LanczosInfo] = None) -> Tuple[float, DenseTensor]:
    ctx = ctx or get_context()
    Dl, d, Dr, wL, wM, wR = _heff_dims(initial_theta, L_env, R_env, W_i, W_ip1)
    out = torch.empty(Dl * d * d * Dr, dtype=torch.float64, device=ctx.torch_device)
    E = C.c_double()
    nk = C.c_int()
    alpha = (C.c_double * max_iter)()
    beta = (C.c_double * max(max_iter - 1, 1))()
    ctx.call("ct_lanczos2", _p(prec), _ptr(initial_theta.storage), _ptr(out), _ptr(L_env.storage),
             _ptr(R_env.storage), _ptr(W_i.tensor.storage), _ptr(W_ip1.tensor.storage), C.c_int64(Dl),
             C.c_int64(d), C.c_int64(Dr), C.c_int64(wL), C.c_int64(wM), C.c_int64(wR), int(max_iter),
             C.c_double(tol), int(max_rotations), int(bool(reorth)), C.byref(E), C.byref(nk), alpha, beta)
    if info is not None:
        info.numiter = nk.value
        info.alpha = list(alpha)[:nk.value]
        info.beta = list(beta)[:max(nk.value - 1, 0)]
    return E.value, DenseTensor(out, [Dl, d, d, Dr])


def split_two_site_theta_svd(theta: DenseTensor, chi_max: int, eps_trunc: float, ctx: DeviceContext | None = None,
                             left_to_right: bool = True, return_spectrum: bool = False, prec: str = "fp64"):
    """-> (A_i, A_ip1, discarded_weight[, S])."""
    ctx = ctx or get_context()
    Dl, d, _, Dr = theta.shape
    k = min(Dl * d, d * Dr)
    dev = ctx.torch_device
    A = torch.empty(Dl * d * k, dtype=torch.float64, device=dev)
    B = torch.empty(k * d * Dr, dtype=torch.float64, device=dev)
    S = torch.empty(k, dtype=torch.float64, device=dev)
    chi = C.c_int64()
    disc = C.c_double()
    ctx.call("ct_svd_split", _p(prec), _ptr(theta.storage), C.c_int64(Dl), C.c_int64(d), C.c_int64(Dr), C.c_int64(chi_max),
             C.c_double(eps_trunc), int(bool(left_to_right)), _ptr(A), _ptr(B), _ptr(S), C.byref(chi),
             C.byref(disc))
    c = chi.value
    Ai = MPSSite(DenseTensor(A[:Dl * d * c], [Dl, d, c]))
    Bi = MPSSite(DenseTensor(B[:c * d * Dr], [c, d, Dr]))
    if return_spectrum:
        return Ai, Bi, disc.value, S[:c].cpu().numpy()
    return Ai, Bi, disc.value


class DMRGWorkspace:
    """Left/right environments of a sweep (dmrg.mojo:39-90)."""

    def __init__(self, mps: MatrixProductState, mpo: MatrixProductOperator, ctx: DeviceContext | None = None,
                 prec: str = "fp64"):
        ctx = ctx or get_context()
        self.num_sites = mps.num_sites()
        if mpo.num_sites() != self.num_sites:
            raise ValueError("MPS and MPO must have the same number of sites")
        self.R_env = build_right_environments(mps, mpo, ctx, prec)
        L0 = create_identity_environment(ctx, mpo.bond_dimension(0), mps.bond_dimension(0))
        self.L_env = [L0] * (self.num_sites + 1)


def dmrg_local_update_two_site(site_index: int, mps: MatrixProductState, mpo: MatrixProductOperator,
                               workspace: DMRGWorkspace, params: DMRGParams, ctx: DeviceContext | None = None,
                               left_to_right: bool = True) -> float:
    """One local update composed from the C-ABI pieces (dmrg.mojo:759-844)."""
    ctx = ctx or get_context()
    i = site_index
    theta = build_two_site_theta(mps.sites[i], mps.sites[i + 1], ctx)
    E, th = lanczos_two_site_optimize(theta, workspace.L_env[i], workspace.R_env[i + 2], mpo.sites[i],
                                      mpo.sites[i + 1], ctx, params.max_krylov_iter, params.krylov_tol,
                                      params.prec, params.max_rotations, params.reorth)
    A, B, _ = split_two_site_theta_svd(th, params.chi_max, params.eps_trunc, ctx, left_to_right, prec=params.prec)
    mps.sites[i] = A
    mps.sites[i + 1] = B
    mps.bond_dims[i + 1] = A.right_bond_dim()
    if left_to_right:
        workspace.L_env[i + 1] = update_left_environment(workspace.L_env[i], A, mpo.sites[i], ctx, params.prec)
    else:
        workspace.R_env[i + 1] = update_right_environment(workspace.R_env[i + 2], B, mpo.sites[i + 1], ctx,
                                                          params.prec)
    return E


def bond_capacities(bond_dims: List[int], d: int, chi_max: int) -> List[int]:
    """Largest bond dimension every bond can reach under two-site updates."""
    N = len(bond_dims) - 1
    big = 1 << 40
    lc = [0] * (N + 1)
    rc = [0] * (N + 1)
    lc[0] = bond_dims[0]
    for k in range(1, N + 1):
        lc[k] = min(lc[k - 1] * d, big)
    rc[N] = bond_dims[N]
    for k in range(N - 1, -1, -1):
        rc[k] = min(rc[k + 1] * d, big)
    cap = []
    for k in range(N + 1):
        c = bond_dims[k] if k in (0, N) else min(chi_max, lc[k], rc[k])
        cap.append(max(c, bond_dims[k]))
    return cap


def dmrg_two_site(ctx: DeviceContext | None, mpo: MatrixProductOperator, mps: MatrixProductState,
                  params: DMRGParams, stats: Optional[DMRGStats] = None) -> Tuple[float, MatrixProductState]:
    """Full sweeps on the device through ct_dmrg_two_site -> (energy, mps)."""
    ctx = ctx or get_context()
    if not params.two_site:
        raise ValueError("Only two-site DMRG is currently implemented")
    N = mps.num_sites()
    if N < 2:
        raise ValueError("DMRG requires at least 2 sites")
    if mpo.num_sites() != N:
        raise ValueError("MPS and MPO must have the same number of sites")
    d = mps.physical_dim
    cap = bond_capacities(list(mps.bond_dims), d, params.chi_max)
    dev = ctx.torch_device
    bufs = []
    for i in range(N):
        nb = torch.empty(cap[i] * d * cap[i + 1], dtype=torch.float64, device=dev)
        src = mps.sites[i].tensor.storage
        nb[:src.numel()].copy_(src)
        bufs.append(nb)
    bd = _lib.i64_array(mps.bond_dims)
    mpo_pp, k1 = _lib.ptr_array([s.tensor.storage.data_ptr() for s in mpo.sites])
    mps_pp, k2 = _lib.ptr_array([b.data_ptr() for b in bufs])
    capacity = _lib.i64_array([b.numel() for b in bufs])
    E = C.c_double()
    sweeps = (C.c_double * max(params.num_sweeps, 1))()
    done = C.c_int()
    disc = (C.c_double * max(params.num_sweeps * 2 * (N - 1), 1))()
    st = _lib.ct_dmrg_stats()
    cp = params.to_c()
    ctx.call("ct_dmrg_two_site", C.byref(cp), N, d, _lib.i64_array(mpo.bond_dims), mpo_pp, bd, mps_pp, capacity,
             C.byref(E), sweeps, C.byref(done), disc, C.byref(st))
    dims = [int(x) for x in bd]
    sites = [MPSSite(DenseTensor(bufs[i][:dims[i] * d * dims[i + 1]], [dims[i], d, dims[i + 1]]))
             for i in range(N)]
    if stats is not None:
        for f in ("seconds_total", "seconds_lanczos", "seconds_svd", "seconds_env", "heff_flops", "env_flops",
                  "heff_applies", "local_updates", "max_discarded", "energy_rayleigh", "subspace_splits",
                  "exact_splits", "seconds_subspace", "cold_splits", "completed_rows",
                  "seconds_rayleigh", "stale_retries", "fp64_handovers"):
            setattr(stats, f, getattr(st, f))
        stats.sweep_energies = list(sweeps)[:done.value]
        stats.discarded = list(disc)[:done.value * 2 * (N - 1)]
    return E.value, MatrixProductState(sites)
