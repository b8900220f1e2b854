"""Sweep-level parity of the FP64 device DMRG against the oracle and exact diagonalisation.

* TFIM L=12 (J=h=1, chi<=32, 6 sweeps, 20 Lanczos steps, eps 1e-10) from the
  seed-0 right-normalised random MPS, converged tridiagonal eigensolve: the
  per-sweep energies equal the oracle's to 1e-10 relative, the bond
  dimensions and discarded weights are identical, and the energy matches ED
  to 1e-8.
* The same chain in the reference's capped-Jacobi semantics: every local
  Lanczos update equals the oracle's on the same inputs to 1e-6 (whole
  trajectories in that mode are chaotic, so they are not compared).
* 4-site XXX (test_dmrg_exact_small.mojo:17-65): E0 = -3.
* Small Bose-Hubbard and Jordan-Wigner Fermi-Hubbard chains against ED.
"""
import numpy as np
import pytest

from oracle import dmrg as od
from oracle import ed
from oracle import hamiltonians as oh
from oracle import rng as orng

pytestmark = pytest.mark.gpu


def ct_mod():
    import chemtensor_mojo_gb300 as ct
    return ct


def run_device(ctx, mpo_arrays, mps_arrays, params):
    ct = ct_mod()
    mps = ct.mps_from_arrays(ctx, mps_arrays)
    mpo = ct.mpo_from_arrays(ctx, mpo_arrays)
    stats = ct.DMRGStats()
    E, out = ct.dmrg_two_site(ctx, mpo, mps, params, stats)
    return E, out, stats


@pytest.fixture(scope="module")
def tfim12():
    L = 12
    mpo = oh.ising_1d(L, J=1.0, h_longitudinal=0.0, g_transverse=1.0)
    sites, dims = orng.create_random_mps_c_compatible(L, 2, 32, 0)
    mps = od.right_normalize(sites)
    return mpo, mps


def test_tfim12_trajectory_matches_oracle(ctx, tfim12):
    """Converged eigensolve: whole 6-sweep trajectory equals the oracle's."""
    ct = ct_mod()
    mpo, mps = tfim12
    p = ct.DMRGParams(num_sweeps=6, chi_max=32, eps_trunc=1e-10, max_krylov_iter=20, krylov_tol=1e-10,
                      energy_tol=0.0, max_rotations=0)
    E, out, stats = run_device(ctx, mpo, mps, p)
    pref = od.DMRGParams(6, 32, 1e-10, 20, 1e-10, 0.0)
    log = od.SweepLog()
    E_ref, mps_ref = od.dmrg_two_site(mpo, mps, pref, eig="exact", log=log)
    assert out.bond_dims == [1] + [a.shape[2] for a in mps_ref]
    np.testing.assert_allclose(stats.sweep_energies, log.energies, rtol=1e-10, atol=0)
    assert abs(E - E_ref) <= 1e-10 * abs(E_ref)
    np.testing.assert_allclose(stats.discarded, log.discarded, atol=1e-12)
    assert abs(E - ed.ground_energy(mpo)) < 1e-8


def test_tfim12_reorthogonalised_lanczos(ctx, tfim12):
    """FP64 form with the reorthogonalised Lanczos (the mixed form's Krylov step) over six
    sweeps.  The chain's end bonds have theta spaces of 16 and 64 states under 20 Krylov
    steps, and after the first sweep each start vector is nearly the ground state, so the
    Krylov space nearly closes -- the case where a Gram-Schmidt scheme that orthogonalises
    the large alpha / beta components only once loses orthogonality and its Ritz values
    fall below the spectrum.  Every sweep energy must stay within 1e-8 of the plain form's,
    never below the ground state, and end within 1e-8 of exact diagonalisation."""
    ct = ct_mod()
    mpo, mps = tfim12
    runs = {}
    for reorth in (False, True):
        p = ct.DMRGParams(num_sweeps=6, chi_max=32, eps_trunc=1e-10, max_krylov_iter=20, krylov_tol=1e-10,
                          energy_tol=0.0, max_rotations=0, reorth=reorth)
        runs[reorth] = run_device(ctx, mpo, mps, p)
    E_plain, _, st_plain = runs[False]
    E_re, _, st_re = runs[True]
    e0 = ed.ground_energy(mpo)
    for a, b in zip(st_re.sweep_energies, st_plain.sweep_energies):
        assert a >= e0 - 1e-10 * abs(e0)          # variational: never below the ground state
        assert abs(a - b) <= 1e-8 * abs(b)
    assert abs(E_re - e0) < 1e-8


def test_tfim12_reference_jacobi_local_parity(ctx, tfim12):
    """Reference semantics (Jacobi capped at 200 rotations, dmrg.mojo:507-598).

    The capped eigensolve is ill-conditioned: a 1e-15 relative perturbation of
    H_eff moves single local energies by up to ~4e-7 and whole trajectories by
    ~1e-3 (tests/test_oracle.py::test_capped_jacobi_is_chaotic).  Parity is
    therefore checked per local update along the device's own trajectory:
    every device Lanczos result equals the oracle's on the same inputs to
    1e-6, and both runs end in the same energy band.
    """
    ct = ct_mod()
    mpo_a, mps_a = tfim12
    mps = ct.mps_from_arrays(ctx, mps_a)
    mpo = ct.mpo_from_arrays(ctx, mpo_a)
    p = ct.DMRGParams(num_sweeps=2, chi_max=32, eps_trunc=1e-10, max_krylov_iter=20, krylov_tol=1e-10,
                      energy_tol=0.0)
    ws = ct.DMRGWorkspace(mps, mpo, ctx)
    N = mps.num_sites()
    worst = 0.0
    for sweep in range(2):
        for l2r, order in ((True, range(N - 1)), (False, range(N - 2, -1, -1))):
            for i in order:
                th = od.build_two_site_theta(mps.sites[i].tensor.to_numpy(), mps.sites[i + 1].tensor.to_numpy())
                E_ref, _ = od.lanczos_two_site_optimize(th, ws.L_env[i].to_numpy(), ws.R_env[i + 2].to_numpy(),
                                                        mpo_a[i], mpo_a[i + 1], 20, 1e-10)
                E = ct.dmrg_local_update_two_site(i, mps, mpo, ws, p, ctx, l2r)
                worst = max(worst, abs(E - E_ref))
    assert worst < 1e-6
    E_full, _, _ = run_device(ctx, mpo_a, mps_a, ct.DMRGParams(num_sweeps=6, chi_max=32, eps_trunc=1e-10,
                                                               max_krylov_iter=20, krylov_tol=1e-10,
                                                               energy_tol=0.0))
    assert abs(E_full - ed.ground_energy(mpo_a)) < 2e-2


def test_xxx_4site_exact(ctx):
    """test_dmrg_exact_small.mojo:17-65 (Neel start, chi=8, 6 sweeps): E0 = -3."""
    ct = ct_mod()
    mpo = oh.heisenberg_xxz(4, J=1.0, D=1.0, h=0.0)
    neel = []
    for i in range(4):
        a = np.zeros((1, 2, 1))
        a[0, i % 2, 0] = 1.0
        neel.append(a)
    p = ct.DMRGParams(num_sweeps=6, chi_max=8, eps_trunc=1e-10, max_krylov_iter=20, krylov_tol=1e-8,
                      energy_tol=1e-8)
    E, out, _ = run_device(ctx, mpo, neel, p)
    assert abs(E - (-3.0)) < 1e-10


@pytest.mark.parametrize("model", ["bose_hubbard", "fermi_hubbard", "xxz"])
def test_small_models_vs_ed(ctx, model):
    ct = ct_mod()
    if model == "bose_hubbard":
        L, d = 6, 3
        mpo = oh.bose_hubbard(L, d, t=1.0, u=4.0, mu=0.0)
    elif model == "fermi_hubbard":
        L, d = 6, 4
        mpo = oh.fermi_hubbard(L, t=1.0, U=8.0)
    else:
        L, d = 10, 2
        mpo = oh.spin_half_xxz(L, 1.0)
    sites, _ = orng.create_random_mps_c_compatible(L, d, 64, 1)
    mps = od.right_normalize(sites)
    p = ct.DMRGParams(num_sweeps=6, chi_max=64, eps_trunc=1e-12, max_krylov_iter=24, krylov_tol=1e-12,
                      energy_tol=0.0, max_rotations=0)
    E, out, _ = run_device(ctx, mpo, mps, p)
    assert abs(E - ed.ground_energy(mpo)) < 1e-8 * max(1.0, abs(E))


def test_expectation_matches_energy(ctx, tfim12):
    """Tier A of test_dmrg_gauge_safe.mojo:52-88: E_dmrg equals <psi|H|psi>/<psi|psi>."""
    ct = ct_mod()
    mpo, mps = tfim12
    p = ct.DMRGParams(num_sweeps=4, chi_max=32, eps_trunc=1e-10, max_krylov_iter=20, krylov_tol=1e-10,
                      energy_tol=0.0, max_rotations=0)
    E, out, _ = run_device(ctx, mpo, mps, p)
    E2 = ct.expectation_value_normalized(out, ct.mpo_from_arrays(ctx, mpo), ctx)
    assert abs(E - E2) < 1e-8
    ref = od.expectation(out.to_numpy(), mpo) / od.norm_sq(out.to_numpy())
    assert abs(E2 - ref) < 1e-12


def test_right_normalize_on_device(ctx):
    ct = ct_mod()
    arrays, dims = ct.random_mps_c_compatible_arrays(10, 2, 16, 3)
    mps = ct.mps_right_normalize(ctx, ct.mps_from_arrays(ctx, arrays))
    for a in mps.to_numpy()[1:]:
        m = a.reshape(a.shape[0], -1)
        assert np.allclose(m @ m.T, np.eye(a.shape[0]), atol=1e-12)
    psi = ct.mps_to_statevector(mps, ctx).to_numpy()
    psi0 = od.mps_to_statevector(arrays)
    assert abs(abs(psi @ psi0) / np.linalg.norm(psi0) - 1.0) < 1e-12
