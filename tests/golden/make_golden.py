"""Generates tests/golden/*.npz from the CPU oracle (run from the repo root).

    python tests/golden/make_golden.py

Fixtures (small, FP64):
  rng_seed0.npz        first 256 randnf() values of seed 0 and the L=12/d=2/chi=32
                       random-MPS bond dimensions (rng_c_compat.mojo recipe)
  heff_small.npz       one H_eff apply and both environment updates on seeded
                       random tensors
  tfim12_converged.npz per-sweep energies, kept bond dimensions and discarded
                       weights of TFIM L=12 (J=h=1, chi 32, 6 sweeps, 20 Lanczos
                       steps, eps 1e-10) with the converged eigensolve, plus
                       the exact ground energy
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import dmrg as od  # noqa: E402
from oracle import ed  # noqa: E402
from oracle import hamiltonians as oh  # noqa: E402
from oracle import rng as orng  # noqa: E402


def main():
    st = orng.seed_rng_state(0)
    vals = np.array([st.randnf() for _ in range(256)], dtype=np.float32)
    _, dims = orng.create_random_mps_c_compatible(12, 2, 32, 0)
    np.savez(os.path.join(HERE, "rng_seed0.npz"), randnf=vals, dims=np.array(dims))

    g = np.random.default_rng(1234)
    Dl, d, Dr, wL, wM, wR = 6, 2, 5, 3, 4, 3
    th = g.standard_normal((Dl, d, d, Dr))
    L = g.standard_normal((wL, Dl, Dl))
    R = g.standard_normal((wR, Dr, Dr))
    W1 = g.standard_normal((wL, d, d, wM))
    W2 = g.standard_normal((wM, d, d, wR))
    A = g.standard_normal((Dl, d, Dr))
    W = g.standard_normal((wL, d, d, wR))
    np.savez(os.path.join(HERE, "heff_small.npz"), th=th, L=L, R=R, W1=W1, W2=W2, A=A, W=W,
             heff=od.apply_two_site_heff(th, L, R, W1, W2), left=od.update_left_environment(L, A, W),
             right=od.update_right_environment(R, A, W))

    Lc = 12
    mpo = oh.ising_1d(Lc, J=1.0, h_longitudinal=0.0, g_transverse=1.0)
    sites, _ = orng.create_random_mps_c_compatible(Lc, 2, 32, 0)
    mps = od.right_normalize(sites)
    log = od.SweepLog()
    p = od.DMRGParams(6, 32, 1e-10, 20, 1e-10, 0.0)
    E, out = od.dmrg_two_site(mpo, mps, p, eig="exact", log=log)
    np.savez(os.path.join(HERE, "tfim12_converged.npz"), energies=np.array(log.energies),
             chis=np.array(log.chis), discarded=np.array(log.discarded), E_ed=ed.ground_energy(mpo))


if __name__ == "__main__":
    main()
