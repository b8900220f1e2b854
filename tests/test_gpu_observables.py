"""Device observables against the oracle (environments.mojo:475-1189, dmrg_utils.mojo:18-91).

* <bra|mpo|ket> and <bra|ket> with different bond dimensions, through the C ABI
  (ct_mps_expectation2, ct_env_left2) against oracle.observables, 1e-12
  relative (FP64 everywhere; only the summation order differs);
* one two-MPS environment step against the oracle entrywise;
* apply_mpo and mpo_compose site tensors against the oracle entrywise (exact
  products of two or d terms);
* variance, energy, fidelity and the spin observables against the oracle;
* the reference's own checks (test_mps_observables.mojo): <psi|psi> =
  ||psi||^2 and O(1) ranges for its random-MPS setup; and the three tiers of
  test_dmrg_gauge_safe.mojo (TFIM from a product state: energy() equals the
  sweep energy, small variance, spin observables in range);
* error paths: length mismatches and a final environment that is not a scalar.
"""
import numpy as np
import pytest

from oracle import dmrg as od
from oracle import hamiltonians as oh
from oracle import observables as ob

pytestmark = pytest.mark.gpu

REL = 1e-12


def ct_mod():
    import chemtensor_mojo_gb300 as ct
    return ct


def random_mps(L, d, chi, seed, scale=True):
    rng = np.random.default_rng(seed)
    dims = [1] + [min(chi, d ** min(k, L - k)) for k in range(1, L)] + [1]
    return [rng.standard_normal((dims[i], d, dims[i + 1])) / (np.sqrt(dims[i] * d) if scale else 1.0)
            for i in range(L)]


def random_mpo(L, d, D, seed):
    rng = np.random.default_rng(seed)
    dims = [1] + [D] * (L - 1) + [1]
    return [rng.standard_normal((dims[i], d, d, dims[i + 1])) for i in range(L)]


@pytest.mark.parametrize("L,d,chi_bra,chi_ket,D", [(6, 2, 8, 5, 3), (5, 3, 4, 9, 2), (10, 2, 64, 48, 5),
                                                   (8, 4, 32, 20, 6)])
def test_two_mps_expectation_and_overlap(ctx, L, d, chi_bra, chi_ket, D):
    ct = ct_mod()
    bra, ket = random_mps(L, d, chi_bra, 1), random_mps(L, d, chi_ket, 2)
    mpo = random_mpo(L, d, D, 3)
    tb, tk, tm = ct.mps_from_arrays(ctx, bra), ct.mps_from_arrays(ctx, ket), ct.mpo_from_arrays(ctx, mpo)
    ref = ob.expectation_value_two_mps(bra, mpo, ket)
    assert ct.expectation_value_two_mps(tb, tm, tk, ctx) == pytest.approx(ref, rel=REL, abs=1e-14)
    assert ct.mps_overlap(tb, tk, ctx) == pytest.approx(ob.mps_overlap(bra, ket), rel=REL, abs=1e-14)
    assert ct.mps_vdot_direct(tk, tk, ctx) == pytest.approx(ob.mps_vdot_direct(ket, ket), rel=REL)


def test_two_mps_environment_step(ctx):
    import torch
    ct = ct_mod()
    rng = np.random.default_rng(5)
    wL, wR, d, Dlk, Dlb, Drk, Drb = 3, 4, 2, 17, 9, 12, 31
    L = rng.standard_normal((wL, Dlk, Dlb))
    Ak, Ab = rng.standard_normal((Dlk, d, Drk)), rng.standard_normal((Dlb, d, Drb))
    W = rng.standard_normal((wL, d, d, wR))
    out = ct.update_left_environment_two_mps(ct.create_dense_tensor_from_data(ctx, L, L.shape),
                                             ct.MPSSite(ct.create_dense_tensor_from_data(ctx, Ab, Ab.shape)),
                                             ct.MPSSite(ct.create_dense_tensor_from_data(ctx, Ak, Ak.shape)),
                                             ct.MPOSite(ct.create_dense_tensor_from_data(ctx, W, W.shape)), ctx)
    torch.cuda.synchronize()
    ref = ob.update_left_environment_two_mps(L, Ab, Ak, W)
    np.testing.assert_allclose(out.to_numpy().reshape(ref.shape), ref, rtol=1e-12, atol=1e-12)


def test_apply_mpo_and_compose(ctx):
    ct = ct_mod()
    L, d = 6, 3
    psi = random_mps(L, d, 7, 7)
    a, b = random_mpo(L, d, 3, 8), random_mpo(L, d, 2, 9)
    tpsi, ta, tb = ct.mps_from_arrays(ctx, psi), ct.mpo_from_arrays(ctx, a), ct.mpo_from_arrays(ctx, b)
    out = ct.apply_mpo(ta, tpsi, ctx)
    for got, ref in zip(out.to_numpy(), ob.apply_mpo(a, psi)):
        np.testing.assert_allclose(got.reshape(ref.shape), ref, rtol=1e-13, atol=1e-14)
    comp = ct.mpo_compose(ta, tb, ctx)
    for site, ref in zip(comp.sites, ob.mpo_compose(a, b)):
        np.testing.assert_allclose(site.tensor.to_numpy().reshape(ref.shape), ref, rtol=1e-13, atol=1e-14)


def test_apply_mpo_large_site(ctx):
    """one chi = 512, D = 5 site (the kernel's row loop and column stride)"""
    ct = ct_mod()
    rng = np.random.default_rng(12)
    A = rng.standard_normal((512, 2, 700))
    W = rng.standard_normal((5, 2, 2, 4))
    out = ct.apply_mpo(ct.mpo_from_arrays(ctx, [W]), ct.mps_from_arrays(ctx, [A]), ctx)
    ref = ob.apply_mpo([W], [A])[0]
    np.testing.assert_allclose(out.sites[0].tensor.to_numpy().reshape(ref.shape), ref, rtol=1e-13, atol=1e-13)


def test_variance_energy_and_spin_observables(ctx):
    ct = ct_mod()
    L = 8
    mpo = oh.heisenberg_xxz(L, J=1.0, D=0.7, h=0.1)
    psi = random_mps(L, 2, 12, 11)
    tm, tp = ct.mpo_from_arrays(ctx, mpo), ct.mps_from_arrays(ctx, psi)
    u = ct.dmrg_utils
    assert u.energy(tp, tm, ctx) == pytest.approx(ob.energy(psi, mpo), rel=REL)
    assert u.variance_op(tp, tm, ctx) == pytest.approx(ob.variance_op(psi, mpo), rel=1e-10)
    assert u.fidelity(tp, tp, ctx) == pytest.approx(ob.fidelity(psi, psi), rel=REL)
    assert u.observe_sz(tp, 3, ctx) == pytest.approx(ob.observe_sz(psi, 3), rel=REL, abs=1e-14)
    assert u.observe_sz_sz(tp, 1, 6, ctx) == pytest.approx(ob.observe_sz_sz(psi, 1, 6), rel=REL, abs=1e-14)
    assert u.observe_sx_sx(tp, 0, 7, ctx) == pytest.approx(ob.observe_sx_sx(psi, 0, 7), rel=REL, abs=1e-14)


def test_reference_observable_checks(ctx):
    """test_mps_observables.mojo: 6 sites, d = 2, chi 16, uniform random MPS scaled by
    1/sqrt(nelem), Ising MPO (J = 1, h = g = 0)."""
    ct = ct_mod()
    dims = [1] + [16] * 5 + [1]
    psi = ct.create_uniform_mps(ctx, 6, 2, dims, seed=1)
    chi = ct.create_uniform_mps(ctx, 6, 2, dims, seed=2)
    mpo = ct.create_ising_1d_mpo(ctx, 6, J=1.0, h_longitudinal=0.0, g_transverse=0.0)
    n = ct.mps_norm(psi, ctx)
    assert 1e-6 < n < 100.0
    assert abs(ct.mps_overlap(chi, psi, ctx)) < 50.0
    assert abs(ct.expectation_value_two_mps(chi, mpo, psi, ctx)) < 50.0
    napp = ct.mps_norm(ct.apply_mpo(mpo, psi, ctx), ctx)
    assert 1e-6 < napp < 100.0
    assert ct.mps_overlap(psi, psi, ctx) == pytest.approx(n * n, rel=1e-12)


def _tfim_dmrg(ctx, L, chi, sweeps, kiter, ktol, etol):
    ct = ct_mod()
    H = ct.create_transverse_ising_mpo(ctx, L, J=1.0, h=0.5)
    psi0 = ct.create_product_mps(ctx, 2, [0] * L)
    params = ct.DMRGParams(num_sweeps=sweeps, chi_max=chi, eps_trunc=1e-10, max_krylov_iter=kiter, krylov_tol=ktol,
                           energy_tol=etol)
    E, psi = ct.dmrg_two_site(ctx, H, psi0, params)
    return H, E, psi


def test_gauge_safe_tier_a(ctx):
    """test_dmrg_gauge_safe.mojo:52-88: TFIM L=8 (J=1, h=0.5) from |0...0>, chi 32, 8 sweeps,
    30 Lanczos steps: E_dmrg = energy(mps, H) to 1e-6 and variance < 1e-3."""
    ct = ct_mod()
    H, E, psi = _tfim_dmrg(ctx, 8, 32, 8, 30, 1e-10, 1e-10)
    assert ct.dmrg_utils.energy(psi, H, ctx) == pytest.approx(E, abs=1e-6)
    assert ct.dmrg_utils.variance_op(psi, H, ctx) < 1e-3


def test_gauge_safe_tier_b(ctx):
    """test_dmrg_gauge_safe.mojo:95-131: L=10, chi 64, 6 sweeps; Sz, SzSz, SxSx in range,
    and each equal to the oracle's value for the same MPS."""
    ct = ct_mod()
    H, E, psi = _tfim_dmrg(ctx, 10, 64, 6, 30, 1e-10, 1e-10)
    u = ct.dmrg_utils
    E2 = u.energy(psi, H, ctx)
    sz0, szm = u.observe_sz(psi, 0, ctx), u.observe_sz(psi, 5, ctx)
    szsz, sxsx = u.observe_sz_sz(psi, 0, 1, ctx), u.observe_sx_sx(psi, 0, 1, ctx)
    assert -100 < E2 < 100
    assert -0.5 - 1e-5 <= sz0 <= 0.5 + 1e-5 and -0.5 - 1e-5 <= szm <= 0.5 + 1e-5
    assert -0.25 - 1e-5 <= szsz <= 0.25 + 1e-5
    host = psi.to_numpy()
    assert sz0 == pytest.approx(ob.observe_sz(host, 0), rel=1e-10, abs=1e-12)
    assert szsz == pytest.approx(ob.observe_sz_sz(host, 0, 1), rel=1e-10, abs=1e-12)
    assert sxsx == pytest.approx(ob.observe_sx_sx(host, 0, 1), rel=1e-10, abs=1e-12)


def test_gauge_safe_tier_c(ctx):
    """test_dmrg_gauge_safe.mojo:138-171: L=8, chi 24, 6 sweeps, 25 Lanczos steps, tol 1e-8:
    -10 < E < 0 and variance < 0.01."""
    ct = ct_mod()
    H, E, psi = _tfim_dmrg(ctx, 8, 24, 6, 25, 1e-8, 1e-8)
    assert -10 < E < 0
    assert ct.dmrg_utils.variance_op(psi, H, ctx) < 0.01


def test_observable_errors(ctx):
    ct = ct_mod()
    a = ct.mps_from_arrays(ctx, random_mps(4, 2, 4, 0))
    b = ct.mps_from_arrays(ctx, random_mps(5, 2, 4, 0))
    with pytest.raises(ValueError):
        ct.mps_overlap(a, b, ctx)
    with pytest.raises(ValueError):
        ct.apply_mpo(ct.mpo_from_arrays(ctx, random_mpo(4, 3, 2, 0)), a, ctx)
    # open right bond: the final environment is not a scalar
    sites = random_mps(3, 2, 4, 0)
    sites[-1] = np.ones((sites[-1].shape[0], 2, 2))
    c = ct.mps_from_arrays(ctx, sites)
    with pytest.raises(ct.CTDMRGError):
        ct.mps_overlap(c, c, ctx)


def test_bond_entropies(ctx):
    ct = ct_mod()
    L = 8
    psi = random_mps(L, 2, 8, 21)
    got = ct.mps_bond_entropies(ct.mps_from_arrays(ctx, psi), ctx)
    ref = ob.bond_entropies_statevector(od.mps_to_statevector(psi), L, 2)
    assert got == pytest.approx(ref, rel=1e-10, abs=1e-12)
    # GHZ: ln 2 across every bond
    ghz = [np.zeros((1, 2, 2))] + [np.zeros((2, 2, 2)) for _ in range(L - 2)] + [np.zeros((2, 2, 1))]
    ghz[0][0, 0, 0] = ghz[0][0, 1, 1] = 1.0
    for A in ghz[1:-1]:
        A[0, 0, 0] = A[1, 1, 1] = 1.0
    ghz[-1][0, 0, 0] = ghz[-1][1, 1, 0] = 1.0
    assert ct.mps_bond_entropies(ct.mps_from_arrays(ctx, ghz), ctx) == pytest.approx([np.log(2.0)] * (L - 1),
                                                                                    rel=1e-12)


def test_dmrg_results_json_end_to_end(ctx, tmp_path):
    ct = ct_mod()
    L, chi = 10, 16
    mpo = ct.create_heisenberg_xxz_mpo(ctx, L, J=1.0, D=0.5, h=0.0)
    arrays, _ = ct.random_mps_c_compatible_arrays(L, 2, 8, seed=5)
    mps = ct.mps_right_normalize(ctx, ct.mps_from_arrays(ctx, arrays))
    params = ct.DMRGParams(num_sweeps=4, chi_max=chi, eps_trunc=1e-10, max_krylov_iter=20, krylov_tol=1e-12,
                           energy_tol=0.0)
    stats = ct.DMRGStats()
    E, out = ct.dmrg_two_site(ctx, mpo, mps, params, stats)
    ent = ct.mps_bond_entropies(out, ctx)
    psi = out.to_numpy()
    ref_ent = ob.bond_entropies_statevector(od.mps_to_statevector(psi), L, 2)
    assert ent == pytest.approx(ref_ent, rel=1e-9, abs=1e-12)
    jp = ct.DMRGJsonParams(nsites=L, d=2, J=1.0, D=0.5, h=0.0, num_sweeps=4, maxiter_lanczos=20, chi_max=chi,
                           tol_split=1e-10)
    path = str(tmp_path / "dmrg_results_gb300.json")
    norm = float(np.sqrt(ct.mps_overlap(out, out, ctx)))
    ct.save_dmrg_results_to_json(path, "gb300", "heisenberg_xxz", jp, E, stats.sweep_energies, ent, out.bond_dims,
                                 norm)
    ref = ct.load_dmrg_reference(path)
    assert ref.energy_final == E and ref.en_sweeps == stats.sweep_energies and ref.bond_dims == out.bond_dims
    assert ref.entropy == ent and ref.norm == pytest.approx(1.0, abs=1e-10)
    assert len(ref.en_sweeps) == 4 and ref.tol_split == 1e-10
