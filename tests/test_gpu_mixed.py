"""Mixed form (TF32x3 on tcgen05 tensor cores) against FP64 references.

Tolerances: a 3xTF32 product with FP32 accumulation carries ~1e-6 relative
error, so single contractions are held to 2e-5 normwise relative error and
energies to the |dE/E| bounds stated in each test.
"""
import numpy as np
import pytest

from oracle import dmrg as od
from oracle import ed
from oracle import hamiltonians as oh
from oracle import rng as orng

pytestmark = pytest.mark.gpu

TOL = 2e-5


def ct_mod():
    import chemtensor_mojo_gb300 as ct
    return ct


def dt(ctx, a):
    return ct_mod().create_dense_tensor_from_data(ctx, a, a.shape)


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300)


@pytest.mark.parametrize("m,n,k,ta,tb", [(128, 128, 32, 0, 0), (128, 128, 64, 0, 1), (200, 130, 70, 1, 0),
                                        (1, 5, 3, 0, 0), (257, 384, 1000, 1, 1), (512, 512, 512, 0, 0)])
def test_tc_gemm_matches_fp64(ctx, m, n, k, ta, tb):
    import ctypes as C
    import torch
    ct = ct_mod()
    rng = np.random.default_rng(m + n + k)
    A = rng.standard_normal((k, m) if ta else (m, k))
    B = rng.standard_normal((n, k) if tb else (k, n))
    Cin = rng.standard_normal((m, n))
    ref = 0.5 * ((A.T if ta else A) @ (B.T if tb else B)) - 2.0 * Cin
    tA, tB = dt(ctx, A), dt(ctx, B)
    tC = dt(ctx, Cin)
    lda = A.shape[1]
    ldb = B.shape[1]
    ctx.call("ct_gemm", 1, ta, tb, C.c_int64(m), C.c_int64(n), C.c_int64(k), C.c_double(0.5),
             C.c_void_p(tA.storage.data_ptr()), C.c_int64(lda), C.c_void_p(tB.storage.data_ptr()), C.c_int64(ldb),
             C.c_double(-2.0), C.c_void_p(tC.storage.data_ptr()), C.c_int64(n))
    torch.cuda.synchronize()
    assert rel(tC.to_numpy(), ref) < TOL


def test_dense_tensor_dot_tf32x3(ctx):
    ct = ct_mod()
    rng = np.random.default_rng(11)
    A = rng.standard_normal((6, 40, 33))
    B = rng.standard_normal((33, 7, 9))
    out = ct.create_dense_tensor(ctx, [6, 40, 7, 9])
    ct.dense_tensor_dot(out, dt(ctx, A), dt(ctx, B), ctx, prec="tf32x3")
    assert rel(out.to_numpy(), np.tensordot(A, B, axes=1)) < TOL


HEFF_SHAPES = [(1, 2, 1, 1, 3, 3), (16, 2, 16, 5, 5, 5), (33, 2, 17, 5, 5, 1), (20, 4, 12, 4, 4, 4),
               (64, 2, 64, 5, 5, 5), (130, 2, 96, 5, 5, 5)]


@pytest.mark.parametrize("shape", HEFF_SHAPES)
def test_heff_tf32x3(ctx, shape):
    ct = ct_mod()
    Dl, d, Dr, wL, wM, wR = shape
    rng = np.random.default_rng(sum(shape) + 1)
    th = rng.standard_normal((Dl, d, d, Dr))
    L = rng.standard_normal((wL, Dl, Dl))
    R = rng.standard_normal((wR, Dr, Dr))
    W1 = rng.standard_normal((wL, d, d, wM))
    W2 = rng.standard_normal((wM, d, d, wR))
    ref = od.apply_two_site_heff(th, L, R, W1, W2)
    out = ct.apply_two_site_heff(dt(ctx, th), dt(ctx, L), dt(ctx, R), ct.MPOSite(dt(ctx, W1)),
                                 ct.MPOSite(dt(ctx, W2)), ctx, prec="tf32x3")
    assert rel(out.to_numpy(), ref) < TOL


ENV_SHAPES = [(1, 2, 2, 1, 3), (16, 2, 7, 5, 5), (9, 4, 11, 4, 4), (64, 2, 64, 5, 5), (100, 2, 70, 3, 4)]


@pytest.mark.parametrize("shape", ENV_SHAPES)
def test_envs_tf32x3(ctx, shape):
    ct = ct_mod()
    Dl, d, Dr, wL, wR = shape
    rng = np.random.default_rng(sum(shape) + 2)
    A = rng.standard_normal((Dl, d, Dr))
    W = rng.standard_normal((wL, d, d, wR))
    L = rng.standard_normal((wL, Dl, Dl))
    R = rng.standard_normal((wR, Dr, Dr))
    outL = ct.update_left_environment(dt(ctx, L), ct.MPSSite(dt(ctx, A)), ct.MPOSite(dt(ctx, W)), ctx,
                                      prec="tf32x3")
    assert rel(outL.to_numpy(), od.update_left_environment(L, A, W)) < TOL
    outR = ct.update_right_environment(dt(ctx, R), ct.MPSSite(dt(ctx, A)), ct.MPOSite(dt(ctx, W)), ctx,
                                       prec="tf32x3")
    assert rel(outR.to_numpy(), od.update_right_environment(R, A, W)) < TOL


def test_dmrg_tf32x3_vs_fp64(ctx):
    """TFIM L=12 (converged eigensolve): mixed and FP64 forms agree to |dE/E| <= 1e-9."""
    ct = ct_mod()
    L = 12
    mpo_a = oh.ising_1d(L, J=1.0, h_longitudinal=0.0, g_transverse=1.0)
    sites, _ = orng.create_random_mps_c_compatible(L, 2, 32, 0)
    mps_a = od.right_normalize(sites)
    res = {}
    for prec in ("fp64", "tf32x3"):
        p = ct.DMRGParams(num_sweeps=6, chi_max=32, eps_trunc=1e-10, max_krylov_iter=20, krylov_tol=1e-10,
                          energy_tol=0.0, max_rotations=0, prec=prec)
        E, out = ct.dmrg_two_site(ctx, ct.mpo_from_arrays(ctx, mpo_a), ct.mps_from_arrays(ctx, mps_a), p)
        res[prec] = E
    E_ed = ed.ground_energy(mpo_a)
    assert abs(res["tf32x3"] - res["fp64"]) <= 1e-9 * abs(res["fp64"])
    assert abs(res["fp64"] - E_ed) < 1e-8
