"""Exact diagonalisation through the MPO (test infrastructure only).

Restates src/tests/state/mpo/mpo_test_helpers.mojo:23-176: contract the MPO to
a dense (d^L x d^L) matrix, then take its lowest eigenvalue.  For L up to ~12
with d=2 (or 6 with d=4) a sparse Lanczos (ARPACK) is used on the assembled
sparse matrix.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def mpo_to_sparse(mpo):
    """Matrix M[(s_in), (s_out)] = sum_w prod_i W_i[w_i, s_in_i, s_out_i, w_{i+1}],
    first site most significant (the row-major order of mps_to_statevector)."""
    # blocks[w] is the sparse operator accumulated so far, ending in channel w
    W0 = mpo[0]
    blocks = [sp.csr_matrix(W0[0, :, :, w]) for w in range(W0.shape[3])]
    for W in mpo[1:]:
        Dl, d, _, Dr = W.shape
        new = []
        for wr in range(Dr):
            acc = None
            for wl in range(Dl):
                op = W[wl, :, :, wr]
                if not np.any(op):
                    continue
                term = sp.kron(blocks[wl], sp.csr_matrix(op), format="csr")
                acc = term if acc is None else acc + term
            if acc is None:
                acc = sp.csr_matrix((blocks[0].shape[0] * d, blocks[0].shape[1] * d))
            new.append(acc)
        blocks = new
    assert len(blocks) == 1
    return blocks[0].tocsr()


def ground_energy(mpo):
    M = mpo_to_sparse(mpo)
    n = M.shape[0]
    Ms = 0.5 * (M + M.T)
    if n <= 64:
        return float(np.linalg.eigvalsh(Ms.toarray())[0])
    vals = spla.eigsh(Ms, k=1, which="SA", tol=1e-13, maxiter=100000)[0]
    return float(vals[0])
