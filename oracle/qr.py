"""FP64 restatement of the reference's QR path (test infrastructure only).

* ``dense_tensor_qr``           src/m_tensor/dense_tensor.mojo:1333-1433: economical QR
                                through Householder reflectors (MAX qr_factorization +
                                form_q, the LAPACK dgeqrf/dorgqr algorithm): Q [m,k],
                                R [k,n], k = min(m,n); here LAPACK's own through NumPy
* ``mps_local_orthonormalize_qr`` src/state/mps_state.mojo:307-379
* ``mps_orthogonalize_qr``      src/state/mps_state.mojo:382-451
"""
from __future__ import annotations

import numpy as np


def dense_tensor_qr(A):
    A = np.asarray(A, dtype=np.float64)
    if A.ndim != 2:
        raise ValueError(f"QR decomposition requires a 2D matrix, got rank {A.ndim}")
    Q, R = np.linalg.qr(A, mode="reduced")
    return Q, R


def mps_local_orthonormalize_qr(block):
    shape = block.shape
    if len(shape) < 3:
        raise ValueError("mps_local_orthonormalize_qr requires rank >= 3 (left, physical, remainder)")
    left, phys, tail = shape[0], shape[1], shape[2:]
    right = int(np.prod(tail))
    Q, R = dense_tensor_qr(block.reshape(left * phys, right))
    k = Q.shape[1]
    return Q.reshape(left, phys, k), R.reshape((k,) + tuple(tail))


def mps_orthogonalize_qr(full_state):
    full_state = np.asarray(full_state, dtype=np.float64)
    dims = full_state.shape
    if len(dims) == 0:
        raise ValueError("full_state must have rank >= 1 to build an MPS")
    if any(x != dims[0] for x in dims):
        raise ValueError("All physical dimensions must match")
    rem = full_state.reshape((1,) + dims)
    sites = []
    for _ in range(len(dims) - 1):
        site, rem = mps_local_orthonormalize_qr(rem)
        sites.append(site)
    final = rem.reshape(rem.shape[0], rem.shape[1], 1)
    nrm = np.linalg.norm(final)
    if nrm > 0:
        final = final / nrm
    sites.append(final)
    return sites
