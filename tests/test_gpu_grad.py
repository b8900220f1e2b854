"""Adjoint energy gradient (ct_energy_grad / torch.autograd) against
central finite differences and against 2 (H_eff theta - E theta) / <psi|psi>.

Tolerance: the adjoint is exact up to FP64 rounding, finite differences with
step 1e-6 carry O(h^2) truncation and O(eps/h) rounding, so the comparison is
held to 1e-6 relative.
"""
import numpy as np
import pytest
import torch

from oracle import dmrg as od
from oracle import hamiltonians as oh
from oracle import rng as orng

pytestmark = pytest.mark.gpu


def energy_cpu(mps, mpo):
    return od.expectation(mps, mpo) / od.norm_sq(mps)


def dev_sites(mps):
    return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in mps]


@pytest.mark.parametrize("ckpt", [0, 2, 3])
def test_gradient_vs_finite_differences(ctx, ckpt):
    import chemtensor_mojo_gb300 as ct
    from chemtensor_mojo_gb300.autograd import energy_and_gradient
    L = 6
    mpo_a = oh.heisenberg_xxz(L, J=1.0, D=0.7, h=0.1)
    mps, _ = orng.create_random_mps_c_compatible(L, 2, 4, 11)
    mpo = ct.mpo_from_arrays(ctx, mpo_a)
    E, grads = energy_and_gradient(mpo, dev_sites(mps), checkpoint_every=ckpt, ctx=ctx)
    assert abs(E - energy_cpu(mps, mpo_a)) < 1e-12 * max(1.0, abs(E))
    h = 1e-6
    for i in range(L):
        g = grads[i].cpu().numpy()
        fd = np.zeros_like(mps[i])
        for idx in np.ndindex(mps[i].shape):
            plus = [a.copy() for a in mps]
            minus = [a.copy() for a in mps]
            plus[i][idx] += h
            minus[i][idx] -= h
            fd[idx] = (energy_cpu(plus, mpo_a) - energy_cpu(minus, mpo_a)) / (2 * h)
        assert np.linalg.norm(g - fd) <= 1e-6 * max(np.linalg.norm(fd), 1e-8)


def test_gradient_matches_two_site_heff_residual(ctx):
    """Mixed-canonical MPS with centre on (i, i+1): dE/dA_i = sum 2 (H_eff th - E th) A_{i+1} / <psi|psi>."""
    import chemtensor_mojo_gb300 as ct
    from chemtensor_mojo_gb300.autograd import energy_and_gradient
    L, i = 8, 3
    mpo_a = oh.ising_1d(L, J=1.0, h_longitudinal=0.2, g_transverse=0.9)
    mps, _ = orng.create_random_mps_c_compatible(L, 2, 8, 5)
    mps = od.right_normalize(mps)
    # left-canonicalise sites < i by QR, pushing R into site i
    for j in range(i):
        Dl, d, Dr = mps[j].shape
        Q, R = np.linalg.qr(mps[j].reshape(Dl * d, Dr))
        mps[j] = Q.reshape(Dl, d, Q.shape[1])
        mps[j + 1] = np.tensordot(R, mps[j + 1], axes=([1], [0]))
    mpo = ct.mpo_from_arrays(ctx, mpo_a)
    E, grads = energy_and_gradient(mpo, dev_sites(mps), ctx=ctx)
    Lenv = od.identity_env(1, 1)
    for j in range(i):
        Lenv = od.update_left_environment(Lenv, mps[j], mpo_a[j])
    Renv = od.build_right_environments(mps, mpo_a)[i + 2]
    th = od.build_two_site_theta(mps[i], mps[i + 1])
    nrm = float(np.sum(th * th))
    Gth = 2.0 * (od.apply_two_site_heff(th, Lenv, Renv, mpo_a[i], mpo_a[i + 1]) - E * th) / nrm
    gi = np.tensordot(Gth, mps[i + 1], axes=([2, 3], [1, 2]))
    assert np.linalg.norm(grads[i].cpu().numpy() - gi) <= 1e-9 * max(np.linalg.norm(gi), 1e-12)


def test_autograd_function_bose_hubbard(ctx):
    """Bose-Hubbard L=32, n_max=3, t=1, U=4, chi=128, checkpoints every 6 sites (FD on sampled entries)."""
    import chemtensor_mojo_gb300 as ct
    from chemtensor_mojo_gb300.autograd import mps_energy
    L, d, chi = 32, 4, 128
    mpo_a = oh.bose_hubbard(L, d, t=1.0, u=4.0, mu=0.0)
    mps = [a for a in orng.gaussian_mps(L, d, chi, 3)[0]]
    mpo = ct.mpo_from_arrays(ctx, mpo_a)
    sites = [t.requires_grad_(True) for t in dev_sites(mps)]
    E = mps_energy(mpo, sites, checkpoint_every=6)
    E.backward()
    assert abs(E.item() - energy_cpu(mps, mpo_a)) < 1e-10 * abs(E.item())
    rng = np.random.default_rng(0)
    h = 1e-6
    gmax = max(float(t.grad.abs().max()) for t in sites)
    for _ in range(6):
        i = int(rng.integers(L))
        idx = tuple(int(rng.integers(s)) for s in mps[i].shape)
        plus = [a.copy() for a in mps]
        minus = [a.copy() for a in mps]
        plus[i][idx] += h
        minus[i][idx] -= h
        fd = (energy_cpu(plus, mpo_a) - energy_cpu(minus, mpo_a)) / (2 * h)
        g = sites[i].grad[idx].item()
        assert abs(g - fd) <= 1e-6 * gmax


@pytest.mark.parametrize("case", ["bose_hubbard", "xxz_ragged"])
def test_tf32x3_gradient_matches_fp64(ctx, case):
    """The mixed form of the adjoint (environments and one-site effective Hamiltonians on the
    tensor cores, TF32x3) against the FP64 adjoint.  Each environment step carries FP32-level
    rounding (~sqrt(K) 6e-8 relative for K-term sums, K up to 512 here), which random-walks
    along the chain: over 32 unnormalised random sites that is a few 1e-6 on the energy
    (2.4e-6 measured).  Bounds: energy 3e-5, gradient 3e-4 relative (normwise).  The FP64
    adjoint is the one held to the 1e-6 finite-difference bound above."""
    import chemtensor_mojo_gb300 as ct
    from chemtensor_mojo_gb300.autograd import energy_and_gradient
    if case == "bose_hubbard":
        L, d, chi = 32, 4, 128
        mpo_a = oh.bose_hubbard(L, d, t=1.0, u=4.0, mu=0.0)
        mps = [a for a in orng.gaussian_mps(L, d, chi, 3)[0]]
    else:
        L = 12
        mpo_a = oh.heisenberg_xxz(L, J=1.0, D=0.7, h=0.1)
        rng = np.random.default_rng(4)
        dims = [1, 2, 4, 8, 16, 33, 45, 37, 16, 8, 4, 2, 1]
        mps = [rng.standard_normal((dims[i], 2, dims[i + 1])) / np.sqrt(2 * dims[i]) for i in range(L)]
    mpo = ct.mpo_from_arrays(ctx, mpo_a)
    E64, g64 = energy_and_gradient(mpo, dev_sites(mps), checkpoint_every=5, ctx=ctx, prec="fp64")
    Etc, gtc = energy_and_gradient(mpo, dev_sites(mps), checkpoint_every=5, ctx=ctx, prec="tf32x3")
    num = float(torch.sqrt(sum(((a - b) ** 2).sum() for a, b in zip(gtc, g64))))
    den = float(torch.sqrt(sum((b ** 2).sum() for b in g64)))
    print(f"{case}: energy rel diff {abs(Etc - E64) / abs(E64):.3e}, gradient rel diff {num / den:.3e}")
    assert abs(Etc - E64) <= 3e-5 * abs(E64)
    assert num <= 3e-4 * den
