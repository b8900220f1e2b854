"""CPU FP64 oracle for the two-site DMRG hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports this
package; only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` use it, and only as the checker (or as the timed CPU
baseline), never as the thing that is measured or shipped.

It is a restatement, in NumPy/SciPy FP64, of the reference algorithm of
``BatuhanGQskt/chemtensor_mojo``:

* ``oracle.rng``          -- PCG32 + Box-Muller seeded random MPS
                             (src/tests/benchmarks/rng_c_compat.mojo:14-231)
* ``oracle.hamiltonians`` -- MPO builders (src/state/hamiltonians.mojo:7-685)
                             plus a Jordan-Wigner Fermi-Hubbard builder that
                             the reference does not have
* ``oracle.dmrg``         -- theta build, H_eff apply, environment updates,
                             Lanczos + capped Jacobi, truncated SVD split,
                             sweep driver (src/algorithms/dmrg.mojo:22-844,
                             src/state/environments.mojo:99-472,
                             src/m_tensor/dense_tensor.mojo:1483-1623)
* ``oracle.ed``           -- exact diagonalisation through the MPO
                             (src/tests/state/mpo/mpo_test_helpers.mojo:23-176)

Pinning: the reference's own golden files (C-generated JSON dumps) are not in
the reference tree (its .gitignore:59-60 excludes them).  The oracle is pinned
against every known answer that the reference's tests hold (E0=-3 for the
4-site XXX chain, E0=-1 for the 2-site Ising chain, the [3, 2] SVD fixture, the
LCG test data) and against exact diagonalisation; see tests/test_oracle.py.
"""
