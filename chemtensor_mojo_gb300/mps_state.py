"""MPS and MPO containers: the host side of src/state/mps_state.mojo and
src/state/mpo_state.mojo, plus the seeded initial states.

* ``MPSSite`` / ``MatrixProductState``          mps_state.mojo:13-167
* ``create_product_mps``                        mps_state.mojo:258-304
* ``create_uniform_mps``                        mps_state.mojo:220-255 (seeded here)
* ``create_random_mps_c_compatible``            rng_c_compat.mojo:174-231, run natively
* ``mps_right_normalize``                       device SVD sweep (no working
                                                reference counterpart)
* ``mps_to_statevector`` / ``mps_norm``         mps_state.mojo:454-508
* ``MPOSite`` / ``MatrixProductOperator``       mpo_state.mojo:10-193
* ``create_identity_mpo``                       mpo_state.mojo:196-241
* ``create_single_site_op_mpo``                 mpo_state.mojo:243-272
* ``create_two_site_op_mpo``                    mpo_state.mojo:275-310
* ``mps_local_orthonormalize_qr``               mps_state.mojo:307-379
* ``mps_orthogonalize_qr``                      mps_state.mojo:382-451
* ``MatrixProductState.left_canonicalize`` / ``right_canonicalize``
                                                QR sweeps on the device (mps_state.mojo:170-217
                                                is the reference's unfinished version)
"""
from __future__ import annotations

import ctypes as C
from typing import List, Sequence

import numpy as np
import torch

from . import _lib
from .dense_tensor import (DenseTensor, DeviceContext, create_dense_tensor_from_data, dense_tensor_dot,
                           dense_tensor_qr, create_dense_tensor, get_context, _ptr)


class MPSSite:
    """Rank-3 site tensor [left_bond, physical, right_bond]."""

    def __init__(self, tensor: DenseTensor):
        self.tensor = tensor

    def _assert_rank3(self):
        if len(self.tensor.shape) != 3:
            raise ValueError(f"MPSSite expects rank-3 tensors [bond_left, physical, bond_right], got rank "
                             f"{len(self.tensor.shape)}")

    def rank(self) -> int:
        return len(self.tensor.shape)

    def shape(self) -> List[int]:
        return list(self.tensor.shape)

    def physical_dim(self) -> int:
        self._assert_rank3()
        return self.tensor.shape[1]

    def left_bond_dim(self) -> int:
        self._assert_rank3()
        return self.tensor.shape[0]

    def right_bond_dim(self) -> int:
        self._assert_rank3()
        return self.tensor.shape[2]


class MatrixProductState:
    def __init__(self, sites: Sequence[MPSSite]):
        if len(sites) == 0:
            raise ValueError("MatrixProductState requires at least one site tensor")
        phys = sites[0].physical_dim()
        bonds = [sites[0].left_bond_dim()]
        for idx, site in enumerate(sites):
            if site.physical_dim() != phys:
                raise ValueError("All MPS sites must have the same physical dimension")
            if idx > 0 and site.left_bond_dim() != sites[idx - 1].right_bond_dim():
                raise ValueError(f"Bond mismatch between sites {idx - 1} and {idx}")
            bonds.append(site.right_bond_dim())
        self.sites = list(sites)
        self.physical_dim = phys
        self.length = len(self.sites)
        self.bond_dims = bonds

    def num_sites(self) -> int:
        return self.length

    def bond_dimension(self, index: int) -> int:
        return self.bond_dims[index]

    def site_shape(self, index: int) -> List[int]:
        return self.sites[index].shape()

    def describe(self) -> None:
        print(f"MatrixProductState(length={self.length}, physical_dim={self.physical_dim})")
        print("  bond_dims:", self.bond_dims)

    def to_numpy(self) -> List[np.ndarray]:
        return [s.tensor.to_numpy() for s in self.sites]

    def left_canonicalize(self, ctx: DeviceContext | None = None) -> None:
        """QR sweep left to right: every site but the last becomes left-orthonormal, R moves
        into the next site, and the last site is normalised (in place)."""
        ctx = ctx or get_context()
        for i in range(self.length - 1):
            A = self.sites[i].tensor
            Dl, d, Dr = A.shape
            Q, R = dense_tensor_qr(A.reshape([Dl * d, Dr]), ctx)
            k = Q.shape[1]
            self.sites[i] = MPSSite(Q.reshape([Dl, d, k]))
            nxt = self.sites[i + 1].tensor
            _, d2, Dr2 = nxt.shape
            out = create_dense_tensor(ctx, [k, d2 * Dr2])
            dense_tensor_dot(out, R, nxt.reshape([Dr, d2 * Dr2]), ctx)
            self.sites[i + 1] = MPSSite(out.reshape([k, d2, Dr2]))
            self.bond_dims[i + 1] = k
        last = self.sites[self.length - 1].tensor
        nrm = last.norm(ctx)
        if nrm > 0:
            last.scale_in_place(1.0 / nrm, ctx)

    def right_canonicalize(self, ctx: DeviceContext | None = None) -> None:
        """QR sweep right to left on the transposed sites (an LQ): every site but the first
        becomes right-orthonormal and the first site is normalised (in place)."""
        ctx = ctx or get_context()
        for i in range(self.length - 1, 0, -1):
            A = self.sites[i].tensor
            Dl, d, Dr = A.shape
            At = A.reshape([Dl, d * Dr]).transpose([1, 0], ctx)        # [d*Dr, Dl]
            Q, R = dense_tensor_qr(At, ctx)                              # A^T = Q R -> A = R^T Q^T
            k = Q.shape[1]
            self.sites[i] = MPSSite(Q.transpose([1, 0], ctx).reshape([k, d, Dr]))
            prev = self.sites[i - 1].tensor
            Dl0, d0, _ = prev.shape
            Rt = R.transpose([1, 0], ctx)                                # [Dl, k]
            out = create_dense_tensor(ctx, [Dl0 * d0, k])
            dense_tensor_dot(out, prev.reshape([Dl0 * d0, Dl]), Rt, ctx)
            self.sites[i - 1] = MPSSite(out.reshape([Dl0, d0, k]))
            self.bond_dims[i] = k
        first = self.sites[0].tensor
        nrm = first.norm(ctx)
        if nrm > 0:
            first.scale_in_place(1.0 / nrm, ctx)


class MPOSite:
    """Rank-4 site tensor [Wl, d_in, d_out, Wr]."""

    def __init__(self, tensor: DenseTensor):
        if len(tensor.shape) != 4:
            raise ValueError("MPOSite expects rank-4 tensors [Wl, d_in, d_out, Wr]")
        self.tensor = tensor

    def left_bond_dim(self) -> int:
        return self.tensor.shape[0]

    def right_bond_dim(self) -> int:
        return self.tensor.shape[3]

    def physical_in_dim(self) -> int:
        return self.tensor.shape[1]

    def physical_out_dim(self) -> int:
        return self.tensor.shape[2]


class MatrixProductOperator:
    def __init__(self, sites: Sequence[MPOSite]):
        if len(sites) == 0:
            raise ValueError("MatrixProductOperator requires at least one site")
        for i in range(1, len(sites)):
            if sites[i].left_bond_dim() != sites[i - 1].right_bond_dim():
                raise ValueError(f"MPO bond mismatch between sites {i - 1} and {i}")
        self.sites = list(sites)
        self.length = len(self.sites)
        self.bond_dims = [sites[0].left_bond_dim()] + [s.right_bond_dim() for s in sites]

    def num_sites(self) -> int:
        return self.length

    def bond_dimension(self, index: int) -> int:
        return self.bond_dims[index]

    def to_numpy(self) -> List[np.ndarray]:
        return [s.tensor.to_numpy() for s in self.sites]


def mpo_from_arrays(ctx, arrays: Sequence[np.ndarray]) -> MatrixProductOperator:
    return MatrixProductOperator([MPOSite(create_dense_tensor_from_data(ctx, a, a.shape)) for a in arrays])


def mps_from_arrays(ctx, arrays: Sequence[np.ndarray]) -> MatrixProductState:
    return MatrixProductState([MPSSite(create_dense_tensor_from_data(ctx, a, a.shape)) for a in arrays])


# -- creators ---------------------------------------------------------------------
def create_product_mps(ctx, physical_dim: int, basis: Sequence[int]) -> MatrixProductState:
    if len(basis) < 1:
        raise ValueError("basis must contain at least one element")
    if physical_dim < 1:
        raise ValueError("physical_dim must be >= 1")
    sites = []
    for i, choice in enumerate(basis):
        if choice < 0 or choice >= physical_dim:
            raise ValueError(f"Invalid basis index {choice} at site {i} (must be in [0, physical_dim))")
        data = np.zeros(physical_dim)
        data[choice] = 1.0
        sites.append(MPSSite(create_dense_tensor_from_data(ctx, data, [1, physical_dim, 1])))
    return MatrixProductState(sites)


def create_uniform_mps(ctx, num_sites: int, physical_dim: int, bond_dims: Sequence[int],
                       init_value: float | None = None, seed: int = 0) -> MatrixProductState:
    if num_sites < 1:
        raise ValueError("num_sites must be >= 1")
    if physical_dim < 1:
        raise ValueError("physical_dim must be >= 1")
    if len(bond_dims) != num_sites + 1:
        raise ValueError("bond_dims must have length num_sites + 1")
    g = np.random.default_rng(seed)
    sites = []
    for i in range(num_sites):
        dl, dr = bond_dims[i], bond_dims[i + 1]
        if dl < 1 or dr < 1:
            raise ValueError("Bond dimensions must be >= 1")
        shape = [dl, physical_dim, dr]
        if init_value is None:
            a = g.random(shape) / np.sqrt(dl * physical_dim * dr)
        else:
            a = np.full(shape, float(init_value))
        sites.append(MPSSite(create_dense_tensor_from_data(ctx, a, shape)))
    return MatrixProductState(sites)


def random_mps_c_compatible_arrays(nsites: int, d: int, chi_max: int, seed: int):
    """Host arrays of create_random_mps_c_compatible (native PCG32 + Box-Muller)."""
    lib = _lib.load()
    dims = (C.c_int64 * (nsites + 1))()
    _lib.check(lib.ct_random_mps_host(nsites, d, chi_max, C.c_uint64(seed), dims, None), "ct_random_mps_host")
    dims_l = [int(x) for x in dims]
    arrays = [np.empty((dims_l[i], d, dims_l[i + 1]), dtype=np.float64) for i in range(nsites)]
    pp, keep = _lib.ptr_array([a.ctypes.data for a in arrays])
    _lib.check(lib.ct_random_mps_host(nsites, d, chi_max, C.c_uint64(seed), dims, pp), "ct_random_mps_host")
    return arrays, dims_l


def create_random_mps_c_compatible(ctx, nsites: int, d: int, chi_max: int, seed: int) -> MatrixProductState:
    arrays, _ = random_mps_c_compatible_arrays(nsites, d, chi_max, seed)
    return mps_from_arrays(ctx, arrays)


def mps_right_normalize(ctx, mps: MatrixProductState) -> MatrixProductState:
    """Right-canonical form on the device (SVD sweep from the right, no truncation)."""
    ctx = ctx or get_context()
    n = mps.num_sites()
    bd = _lib.i64_array(mps.bond_dims)
    tensors = [s.tensor.storage.clone() for s in mps.sites]
    pp, keep = _lib.ptr_array([t.data_ptr() for t in tensors])
    ctx.call("ct_mps_right_normalize", n, mps.physical_dim, bd, pp)
    dims = [int(x) for x in bd]
    sites = [MPSSite(DenseTensor(tensors[i], [dims[i], mps.physical_dim, dims[i + 1]])) for i in range(n)]
    return MatrixProductState(sites)


def mps_to_statevector(psi: MatrixProductState, ctx: DeviceContext | None = None) -> DenseTensor:
    """Row-major contraction to the full vector (small L only), mps_state.mojo:454-492."""
    ctx = ctx or get_context()
    res = psi.sites[0].tensor
    left = res.shape[0] * res.shape[1]
    right = res.shape[2]
    res = res.reshape([left, right])
    for i in range(1, psi.num_sites()):
        site = psi.sites[i].tensor
        Di, di, Dn = site.shape
        if right != Di:
            raise ValueError("Bond dimension mismatch in mps_to_statevector")
        out = create_dense_tensor(ctx, [left, di * Dn])
        dense_tensor_dot(out, res, site.reshape([Di, di * Dn]), ctx)
        left, right = left * di, Dn
        res = out.reshape([left, right])
    if right != 1:
        raise ValueError("Expected trailing bond dimension 1 in mps_to_statevector")
    return res.reshape([left])


def mps_norm(psi: MatrixProductState, ctx: DeviceContext | None = None) -> float:
    return mps_to_statevector(psi, ctx).norm(ctx)


# -- operator MPOs (host-built, bond dimension 1) ----------------------------------
def create_identity_mpo(ctx, num_sites: int, physical_dim: int) -> MatrixProductOperator:
    """Identity on every site, shape [1, d, d, 1] (mpo_state.mojo:196-241)."""
    if num_sites < 1:
        raise ValueError("num_sites must be >= 1")
    if physical_dim < 1:
        raise ValueError("physical_dim must be >= 1")
    eye = np.eye(physical_dim).reshape(1, physical_dim, physical_dim, 1)
    return mpo_from_arrays(ctx, [eye] * num_sites)


def create_single_site_op_mpo(ctx, num_sites: int, site_idx: int, op_data: Sequence[float]) -> MatrixProductOperator:
    """2x2 row-major operator on one site, identity elsewhere (mpo_state.mojo:243-272)."""
    if num_sites < 1 or site_idx < 0 or site_idx >= num_sites:
        raise ValueError("create_single_site_op_mpo: invalid site_idx")
    if len(op_data) != 4:
        raise ValueError("create_single_site_op_mpo: op_data must be 4 elements (2x2)")
    arrays = [np.eye(2).reshape(1, 2, 2, 1)] * num_sites
    arrays = list(arrays)
    arrays[site_idx] = np.asarray(op_data, dtype=np.float64).reshape(1, 2, 2, 1)
    return mpo_from_arrays(ctx, arrays)


def create_two_site_op_mpo(ctx, num_sites: int, site_i: int, site_j: int, op_i_data: Sequence[float],
                           op_j_data: Sequence[float]) -> MatrixProductOperator:
    """O_i O_j with site_i < site_j, identity elsewhere (mpo_state.mojo:275-310)."""
    if num_sites < 2 or site_i < 0 or site_j >= num_sites or site_i >= site_j:
        raise ValueError("create_two_site_op_mpo: invalid sites")
    if len(op_i_data) != 4 or len(op_j_data) != 4:
        raise ValueError("create_two_site_op_mpo: op data must be 4 elements each")
    arrays = [np.eye(2).reshape(1, 2, 2, 1)] * num_sites
    arrays = list(arrays)
    arrays[site_i] = np.asarray(op_i_data, dtype=np.float64).reshape(1, 2, 2, 1)
    arrays[site_j] = np.asarray(op_j_data, dtype=np.float64).reshape(1, 2, 2, 1)
    return mpo_from_arrays(ctx, arrays)


# -- QR construction from a dense state (mps_state.mojo:307-451) -------------------
def mps_local_orthonormalize_qr(ctx, block: DenseTensor):
    """Left-orthonormalise one site of a block [left, phys, rest...] -> (MPSSite [left, phys, k],
    remainder [k, rest...]) with k = min(left*phys, prod(rest)) (mps_state.mojo:307-379)."""
    ctx = ctx or get_context()
    shape = list(block.shape)
    if len(shape) < 3:
        raise ValueError("mps_local_orthonormalize_qr requires rank >= 3 (left, physical, remainder)")
    left, phys, tail = shape[0], shape[1], shape[2:]
    right = int(np.prod(tail))
    if right < 1:
        raise ValueError("Right block dimension must be >= 1 in mps_local_orthonormalize_qr")
    Q, R = dense_tensor_qr(block.reshape([left * phys, right]), ctx)
    k = Q.shape[1]
    return MPSSite(Q.reshape([left, phys, k])), R.reshape([k] + tail)


def mps_orthogonalize_qr(ctx, full_state: DenseTensor) -> MatrixProductState:
    """Dense state [d, d, ..., d] -> left-canonical MPS by successive QR; the last site is
    normalised (mps_state.mojo:382-451)."""
    ctx = ctx or get_context()
    dims = list(full_state.shape)
    if len(dims) == 0:
        raise ValueError("full_state must have rank >= 1 to build an MPS")
    d = dims[0]
    for idx, x in enumerate(dims):
        if x != d:
            raise ValueError(f"All physical dimensions must match the first axis ({d}), but axis {idx} has size {x}")
    remainder = full_state.reshape([1] + dims)
    sites = []
    for _ in range(len(dims) - 1):
        site, remainder = mps_local_orthonormalize_qr(ctx, remainder)
        sites.append(site)
    if len(remainder.shape) != 2:
        raise ValueError(f"Unexpected remainder rank {len(remainder.shape)} while constructing final MPS site")
    final = remainder.reshape([remainder.shape[0], remainder.shape[1], 1])
    nrm = final.norm(ctx)
    if nrm > 0:
        final.scale_in_place(1.0 / nrm, ctx)
    sites.append(MPSSite(final))
    return MatrixProductState(sites)
