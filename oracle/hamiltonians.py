"""MPO builders, restating src/state/hamiltonians.mojo (test infrastructure only).

Every site tensor is a float64 array of shape [Wl, d_in, d_out, Wr].  An
operator ``op`` given as a row-major d x d matrix is stored at
``W[wl, i, j, wr] = op[i, j]``, exactly as the reference appends
``op_data[d_in * d + d_out]`` (e.g. hamiltonians.mojo:108-118).

* ``ising_1d``        hamiltonians.mojo:55-174 (H = -J ZZ - g X - h Z, D=3)
* ``heisenberg_xxx``  hamiltonians.mojo:177-341 (D=5)
* ``heisenberg_xxz``  hamiltonians.mojo:344-521 (H = -J(XX+YY+D ZZ) - h Z, D=5)
* ``bose_hubbard``    hamiltonians.mojo:524-685 (D=4)
* ``fermi_hubbard``   NEW: spinful Hubbard chain through Jordan-Wigner, D=6.
                      The reference has no builder for it.
"""
from __future__ import annotations

import numpy as np

I2 = np.eye(2)
X = np.array([[0.0, 1.0], [1.0, 0.0]])
Z = np.array([[1.0, 0.0], [0.0, -1.0]])
SP = np.array([[0.0, 1.0], [0.0, 0.0]])
SM = np.array([[0.0, 0.0], [1.0, 0.0]])


def _chain(first_row, bulk, last_col, nsites):
    """Assemble [1,d,d,D], [D,d,d,D]..., [D,d,d,1] from operator tables.

    ``bulk[wl][wr]`` is a d x d matrix or None (zero); ``first_row[wr]`` and
    ``last_col[wl]`` likewise.
    """
    D = len(bulk)
    d = None
    for row in bulk:
        for op in row:
            if op is not None:
                d = op.shape[0]
    sites = []
    W0 = np.zeros((1, d, d, D))
    for wr, op in enumerate(first_row):
        if op is not None:
            W0[0, :, :, wr] = op
    sites.append(W0)
    for _ in range(1, nsites - 1):
        W = np.zeros((D, d, d, D))
        for wl in range(D):
            for wr in range(D):
                if bulk[wl][wr] is not None:
                    W[wl, :, :, wr] = bulk[wl][wr]
        sites.append(W)
    WN = np.zeros((D, d, d, 1))
    for wl, op in enumerate(last_col):
        if op is not None:
            WN[wl, :, :, 0] = op
    sites.append(WN)
    return sites


def ising_1d(nsites: int, J: float = 1.0, h_longitudinal: float = 0.0,
             g_transverse: float = 1.0):
    """create_ising_1d_mpo (hamiltonians.mojo:55-174)."""
    if nsites < 2:
        raise ValueError("Ising model requires at least 2 sites")
    onsite = -h_longitudinal * Z - g_transverse * X
    bulk = [[I2, None, None],
            [-J * Z, None, None],
            [onsite, Z, I2]]
    return _chain([onsite, Z, I2], bulk, [I2, -J * Z, onsite], nsites)


def transverse_ising(nsites: int, J: float = 1.0, h: float = 0.5):
    """create_transverse_ising_mpo (hamiltonians.mojo:7-52)."""
    return ising_1d(nsites, J=J, h_longitudinal=0.0, g_transverse=h)


def heisenberg_xxx(nsites: int, J: float = 1.0):
    """create_heisenberg_mpo (hamiltonians.mojo:177-341): H = J(XX+YY+ZZ)."""
    if nsites < 2:
        raise ValueError("Heisenberg model requires at least 2 sites")
    zero = np.zeros((2, 2))
    bulk = [[I2, SP, SM, Z, None],
            [None, None, None, None, 2 * J * SM],
            [None, None, None, None, 2 * J * SP],
            [None, None, None, None, J * Z],
            [None, None, None, None, I2]]
    return _chain([I2, SP, SM, Z, zero], bulk,
                  [zero, 2 * J * SM, 2 * J * SP, J * Z, I2], nsites)


def heisenberg_xxz(nsites: int, J: float = 1.0, D: float = 1.0, h: float = 0.0):
    """create_heisenberg_xxz_mpo (hamiltonians.mojo:344-521).

    H = -J sum (X X + Y Y + D Z Z) - h sum Z with Pauli matrices.  The spin-1/2
    chain sum (Sx Sx + Sy Sy + Delta Sz Sz) is this builder with J=-1/4, D=Delta.
    """
    if nsites < 2:
        raise ValueError("Heisenberg model requires at least 2 sites")
    bulk = [[I2, None, None, None, None],
            [-2 * J * SM, None, None, None, None],
            [-2 * J * SP, None, None, None, None],
            [-J * Z, None, None, None, None],
            [-h * Z, SP, SM, D * Z, I2]]
    return _chain([-h * Z, SP, SM, D * Z, I2], bulk,
                  [I2, -2 * J * SM, -2 * J * SP, -J * Z, -h * Z], nsites)


def spin_half_xxz(nsites: int, Delta: float = 1.0):
    """H = sum (Sx Sx + Sy Sy + Delta Sz Sz), open chain (spin-1/2 operators)."""
    return heisenberg_xxz(nsites, J=-0.25, D=Delta, h=0.0)


def boson_ops(d: int):
    """b_dag, b, n, n(n-1) exactly as hamiltonians.mojo:589-622 fills them."""
    bdag = np.zeros((d, d))
    b = np.zeros((d, d))
    for i in range(d):
        for j in range(d):
            if j > 0 and i == j - 1:
                bdag[i, j] = np.sqrt(float(j))
            if i > 0 and j == i - 1:
                b[i, j] = np.sqrt(float(i))
    n = np.diag(np.arange(d, dtype=np.float64))
    nn1 = np.diag(np.array([i * (i - 1) for i in range(d)], dtype=np.float64))
    return bdag, b, n, nn1


def bose_hubbard(nsites: int, d: int, t: float = 1.0, u: float = 1.0, mu: float = 0.0):
    """create_bose_hubbard_mpo (hamiltonians.mojo:524-685), D=4."""
    if nsites < 2:
        raise ValueError("Bose-Hubbard model requires at least 2 sites")
    if d < 2:
        raise ValueError("Physical dimension must be >= 2")
    bdag, b, n, nn1 = boson_ops(d)
    I = np.eye(d)
    onsite = (u / 2.0) * nn1 - mu * n
    bulk = [[I, None, None, None],
            [-t * b, None, None, None],
            [-t * bdag, None, None, None],
            [onsite, bdag, b, I]]
    return _chain([onsite, bdag, b, I], bulk, [I, -t * b, -t * bdag, onsite], nsites)


def fermion_ops():
    """Spinful fermion operators on |0>, |up>, |dn>, |updn> = c+_up c+_dn |0>.

    Matrices are <row|op|col>.  Returns c+_up, c+_dn, P=(-1)^n, n_up, n_dn.
    """
    cu = np.zeros((4, 4))
    cd = np.zeros((4, 4))
    cu[1, 0] = 1.0     # c+_up |0>  = |up>
    cu[3, 2] = 1.0     # c+_up |dn> = |updn>
    cd[2, 0] = 1.0     # c+_dn |0>  = |dn>
    cd[3, 1] = -1.0    # c+_dn |up> = -|updn>
    P = np.diag([1.0, -1.0, -1.0, 1.0])
    nu = np.diag([0.0, 1.0, 0.0, 1.0])
    nd = np.diag([0.0, 0.0, 1.0, 1.0])
    return cu, cd, P, nu, nd


def fermi_hubbard(nsites: int, t: float = 1.0, U: float = 8.0, mu: float = 0.0):
    """Spinful Fermi-Hubbard chain through Jordan-Wigner, MPO bond dimension 6.

    H = -t sum_{i,s} (c+_{i,s} c_{i+1,s} + h.c.) + U sum n_up n_dn - mu sum n.
    With c_{i,s} = (prod_{j<i} P_j) c~_{i,s}, the bond terms become
    (c~+_s P)_i (c~_s)_{i+1} + (P c~_s)_i (c~+_s)_{i+1}.  Channels use the
    reference's lower-triangular order: 0 = completed, 5 = identity to the left.
    """
    if nsites < 2:
        raise ValueError("Fermi-Hubbard model requires at least 2 sites")
    cu, cd, P, nu, nd = fermion_ops()
    I = np.eye(4)
    onsite = U * (nu @ nd) - mu * (nu + nd)
    left_ops = [cu @ P, cd @ P, P @ cu.T, P @ cd.T]
    right_ops = [-t * cu.T, -t * cd.T, -t * cu, -t * cd]
    bulk = [[None] * 6 for _ in range(6)]
    bulk[0][0] = I
    for k in range(4):
        bulk[k + 1][0] = right_ops[k]
        bulk[5][k + 1] = left_ops[k]
    bulk[5][0] = onsite
    bulk[5][5] = I
    first = [onsite] + left_ops + [I]
    last = [I] + right_ops + [onsite]
    return _chain(first, bulk, last, nsites)
