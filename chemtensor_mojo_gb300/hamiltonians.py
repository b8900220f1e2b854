"""Hamiltonian MPO builders (src/state/hamiltonians.mojo), uploaded to the device.

Each MPO is lower-triangular in the reference's channel convention: the
first site is the "start" row of the bulk tensor, the last site its
"completed" column.  Operators ``op`` (row-major d x d) are stored at
``W[wl, i, j, wr] = op[i, j]`` (hamiltonians.mojo:108-118).

``create_fermi_hubbard_mpo`` has no reference counterpart: it is the
Jordan-Wigner spinful Hubbard chain (bond dimension 6) that the Fermi-Hubbard
workload needs.
"""
from __future__ import annotations

from typing import Dict, List, Tuple

import numpy as np

from .mps_state import MatrixProductOperator, mpo_from_arrays

_I2 = np.eye(2)
_X = np.array([[0.0, 1.0], [1.0, 0.0]])
_Z = np.diag([1.0, -1.0])
_SP = np.array([[0.0, 1.0], [0.0, 0.0]])
_SM = np.array([[0.0, 0.0], [1.0, 0.0]])


def _assemble(nsites: int, D: int, d: int, entries: Dict[Tuple[int, int], np.ndarray], start: int,
              finish: int) -> List[np.ndarray]:
    """Site tensors from the bulk table ``entries[(wl, wr)] = op``.

    The first site is bulk row ``start``; the last site is bulk column ``finish``.
    """
    bulk = np.zeros((D, d, d, D))
    for (wl, wr), op in entries.items():
        bulk[wl, :, :, wr] = op
    first = bulk[start:start + 1].copy()
    last = bulk[:, :, :, finish:finish + 1].copy()
    return [first] + [bulk.copy() for _ in range(nsites - 2)] + [last]


def ising_1d_arrays(nsites: int, J: float = 1.0, h_longitudinal: float = 0.0, g_transverse: float = 1.0):
    if nsites < 2:
        raise ValueError("Ising model requires at least 2 sites")
    onsite = -h_longitudinal * _Z - g_transverse * _X
    e = {(0, 0): _I2, (1, 0): -J * _Z, (2, 0): onsite, (2, 1): _Z, (2, 2): _I2}
    return _assemble(nsites, 3, 2, e, start=2, finish=0)


def heisenberg_xxx_arrays(nsites: int, J: float = 1.0):
    if nsites < 2:
        raise ValueError("Heisenberg model requires at least 2 sites")
    e = {(0, 0): _I2, (0, 1): _SP, (0, 2): _SM, (0, 3): _Z,
         (1, 4): 2 * J * _SM, (2, 4): 2 * J * _SP, (3, 4): J * _Z, (4, 4): _I2}
    return _assemble(nsites, 5, 2, e, start=0, finish=4)


def heisenberg_xxz_arrays(nsites: int, J: float = 1.0, D: float = 1.0, h: float = 0.0):
    if nsites < 2:
        raise ValueError("Heisenberg model requires at least 2 sites")
    e = {(0, 0): _I2, (1, 0): -2 * J * _SM, (2, 0): -2 * J * _SP, (3, 0): -J * _Z,
         (4, 0): -h * _Z, (4, 1): _SP, (4, 2): _SM, (4, 3): D * _Z, (4, 4): _I2}
    return _assemble(nsites, 5, 2, e, start=4, finish=0)


def bose_hubbard_arrays(nsites: int, physical_dim: int, t: float = 1.0, u: float = 1.0, mu: float = 0.0):
    if nsites < 2:
        raise ValueError("Bose-Hubbard model requires at least 2 sites")
    d = physical_dim
    if d < 2:
        raise ValueError("Physical dimension must be >= 2")
    idx = np.arange(d)
    bdag = np.zeros((d, d))
    b = np.zeros((d, d))
    bdag[idx[:-1], idx[1:]] = np.sqrt(idx[1:].astype(float))   # b_dag[j-1, j] = sqrt(j)
    b[idx[1:], idx[:-1]] = np.sqrt(idx[1:].astype(float))      # b[i, i-1] = sqrt(i)
    n = np.diag(idx.astype(float))
    onsite = (u / 2.0) * np.diag((idx * (idx - 1)).astype(float)) - mu * n
    I = np.eye(d)
    e = {(0, 0): I, (1, 0): -t * b, (2, 0): -t * bdag, (3, 0): onsite, (3, 1): bdag, (3, 2): b, (3, 3): I}
    return _assemble(nsites, 4, d, e, start=3, finish=0)


def fermi_hubbard_arrays(nsites: int, t: float = 1.0, U: float = 8.0, mu: float = 0.0):
    """Spinful Hubbard chain, local basis |0>, |up>, |dn>, |up dn> = c+_up c+_dn |0>.

    Jordan-Wigner: c_{i,s} = (prod_{j<i} P_j) c~_{i,s} with P = (-1)^n, so a
    bond term c+_{i,s} c_{i+1,s} becomes (c~+_s P)_i (c~_s)_{i+1} and its
    conjugate (P c~_s)_i (c~+_s)_{i+1}.  Channels: 0 = completed, 1..4 = open
    hops, 5 = identity to the left.
    """
    if nsites < 2:
        raise ValueError("Fermi-Hubbard model requires at least 2 sites")
    cu = np.zeros((4, 4))
    cd = np.zeros((4, 4))
    cu[1, 0] = cu[3, 2] = 1.0
    cd[2, 0] = 1.0
    cd[3, 1] = -1.0
    P = np.diag([1.0, -1.0, -1.0, 1.0])
    nu = np.diag([0.0, 1.0, 0.0, 1.0])
    nd = np.diag([0.0, 0.0, 1.0, 1.0])
    I = np.eye(4)
    e = {(0, 0): I, (5, 0): U * nu @ nd - mu * (nu + nd), (5, 5): I}
    for k, (lop, rop) in enumerate([(cu @ P, cu.T), (cd @ P, cd.T), (P @ cu.T, cu), (P @ cd.T, cd)]):
        e[(5, k + 1)] = lop
        e[(k + 1, 0)] = -t * rop
    return _assemble(nsites, 6, 4, e, start=5, finish=0)


def create_ising_1d_mpo(ctx, num_sites: int, J: float = 1.0, h_longitudinal: float = 0.0,
                        g_transverse: float = 1.0) -> MatrixProductOperator:
    """H = -J sum Z Z - g sum X - h sum Z  (hamiltonians.mojo:55-174)."""
    return mpo_from_arrays(ctx, ising_1d_arrays(num_sites, J, h_longitudinal, g_transverse))


def create_transverse_ising_mpo(ctx, num_sites: int, J: float = 1.0, h: float = 0.5) -> MatrixProductOperator:
    """H = -J sum Z Z - h sum X  (hamiltonians.mojo:7-52)."""
    return create_ising_1d_mpo(ctx, num_sites, J=J, h_longitudinal=0.0, g_transverse=h)


def create_heisenberg_mpo(ctx, num_sites: int, J: float = 1.0) -> MatrixProductOperator:
    """H = J sum (XX + YY + ZZ)  (hamiltonians.mojo:177-341)."""
    return mpo_from_arrays(ctx, heisenberg_xxx_arrays(num_sites, J))


def create_heisenberg_xxz_mpo(ctx, num_sites: int, J: float = 1.0, D: float = 1.0,
                              h: float = 0.0) -> MatrixProductOperator:
    """H = -J sum (XX + YY + D ZZ) - h sum Z  (hamiltonians.mojo:344-521)."""
    return mpo_from_arrays(ctx, heisenberg_xxz_arrays(num_sites, J, D, h))


def create_spin_half_xxz_mpo(ctx, num_sites: int, Delta: float = 1.0) -> MatrixProductOperator:
    """H = sum (Sx Sx + Sy Sy + Delta Sz Sz) with S = sigma/2: the XXZ builder at J = -1/4."""
    return create_heisenberg_xxz_mpo(ctx, num_sites, J=-0.25, D=Delta, h=0.0)


def create_bose_hubbard_mpo(ctx, num_sites: int, physical_dim: int, t: float = 1.0, u: float = 1.0,
                            mu: float = 0.0) -> MatrixProductOperator:
    """H = -t sum (b+ b + h.c.) + u/2 sum n(n-1) - mu sum n  (hamiltonians.mojo:524-685)."""
    return mpo_from_arrays(ctx, bose_hubbard_arrays(num_sites, physical_dim, t, u, mu))


def create_fermi_hubbard_mpo(ctx, num_sites: int, t: float = 1.0, U: float = 8.0,
                             mu: float = 0.0) -> MatrixProductOperator:
    """Jordan-Wigner spinful Fermi-Hubbard chain (no reference counterpart)."""
    return mpo_from_arrays(ctx, fermi_hubbard_arrays(num_sites, t, U, mu))
