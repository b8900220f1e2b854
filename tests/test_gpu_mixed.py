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


@pytest.mark.parametrize("bn", ["128", "256"])
@pytest.mark.parametrize("m,n,k", [(128, 256, 32), (300, 520, 96), (130, 1000, 333), (1024, 768, 256)])
def test_tc_gemm_tile_widths(ctx, monkeypatch, bn, m, n, k):
    """Both tile shapes of the TF32x3 GEMM (128x128 / 3 stages, 128x256 / 2 stages), forced
    through CTDMRG_TC_BN, on ragged M, N and K."""
    import ctypes as C
    import torch
    monkeypatch.setenv("CTDMRG_TC_BN", bn)
    rng = np.random.default_rng(m * 7 + n + k)
    A = rng.standard_normal((m, k))
    B = rng.standard_normal((k, n))
    Cin = rng.standard_normal((m, n))
    ref = 1.5 * (A @ B) + 0.25 * Cin
    tA, tB, tC = dt(ctx, A), dt(ctx, B), dt(ctx, Cin)
    ctx.call("ct_gemm", 1, 0, 0, C.c_int64(m), C.c_int64(n), C.c_int64(k), C.c_double(1.5),
             C.c_void_p(tA.storage.data_ptr()), C.c_int64(k), C.c_void_p(tB.storage.data_ptr()), C.c_int64(n),
             C.c_double(0.25), C.c_void_p(tC.storage.data_ptr()), C.c_int64(n))
    torch.cuda.synchronize()
    assert rel(tC.to_numpy(), ref) < TOL


def _tc_gemm(ctx, A, B):
    import ctypes as C
    import torch
    m, k = A.shape
    n = B.shape[1]
    tA, tB, tC = dt(ctx, A), dt(ctx, B), dt(ctx, np.zeros((m, n)))
    ctx.call("ct_gemm", 1, 0, 0, C.c_int64(m), C.c_int64(n), C.c_int64(k), C.c_double(1.0),
             C.c_void_p(tA.storage.data_ptr()), C.c_int64(k), C.c_void_p(tB.storage.data_ptr()), C.c_int64(n),
             C.c_double(0.0), C.c_void_p(tC.storage.data_ptr()), C.c_int64(n))
    torch.cuda.synchronize()
    return tC.to_numpy()


@pytest.mark.parametrize("bn", ["128", "192", "224", "256"])
@pytest.mark.parametrize("kc", ["1", "2", "3", "64"])
@pytest.mark.parametrize("m,n,k", [(128, 256, 32), (300, 520, 200), (257, 1000, 1000)])
def test_tc_gemm_chunked(ctx, monkeypatch, bn, kc, m, n, k):
    """The chunked-accumulation kernel (CTDMRG_TC_KCHUNK k-blocks per TMEM
    accumulator) on ragged shapes, chunk counts that do and do not divide K, and
    every tile width (192 and 224 exist only in this kernel)."""
    monkeypatch.setenv("CTDMRG_TC_BN", bn)
    monkeypatch.setenv("CTDMRG_TC_KCHUNK", kc)
    rng = np.random.default_rng(m + 3 * n + k)
    A = rng.standard_normal((m, k))
    B = rng.standard_normal((k, n))
    assert rel(_tc_gemm(ctx, A, B), A @ B) < TOL


@pytest.mark.parametrize("bn,m,n,k", [("128", 2560, 1024, 2048), ("128", 2500, 1000, 2000), ("128", 2560, 1024, 9000),
                                      ("192", 2560, 1600, 2048), ("192", 2500, 1700, 1500),
                                      ("224", 2560, 1800, 2048), ("224", 2500, 1700, 999),
                                      ("256", 2560, 2100, 2048), ("256", 2400, 2300, 1200)])
def test_tc_gemm_hybrid_schedule(ctx, monkeypatch, bn, m, n, k):
    """The chunked kernel's hybrid schedule: whole waves of tiles, then the last partial wave's
    k-blocks shared out over all SMs, each split tile summed by the piece that arrives last
    (shapes of 160-180 tiles on 152 SMs; K = 9000 cuts a tile into up to 19 pieces).
    Against FP64 and against the whole-tile schedule (CTDMRG_TC_HYBRID=0), whose summation
    order differs; two runs of the same product are bit-identical (the pieces' partials are
    added in piece order whichever arrives last)."""
    monkeypatch.setenv("CTDMRG_TC_BN", bn)
    rng = np.random.default_rng(m + 5 * n + k)
    A = rng.standard_normal((m, k))
    B = rng.standard_normal((k, n))
    ref = A @ B
    first = _tc_gemm(ctx, A, B)
    second = _tc_gemm(ctx, A, B)
    monkeypatch.setenv("CTDMRG_TC_HYBRID", "0")
    whole = _tc_gemm(ctx, A, B)
    assert rel(first, ref) < TOL
    assert rel(whole, ref) < TOL
    assert np.array_equal(first, second)
    assert rel(first, whole) < 2e-6
    assert not np.array_equal(first, whole)


@pytest.mark.parametrize("bn", ["128", "192", "224", "256"])
@pytest.mark.parametrize("m,n,k", [(300, 520, 200), (1024, 4096, 640), (4100, 1000, 700)])
def test_tc_gemm_transposed_product(ctx, monkeypatch, bn, m, n, k):
    """The launcher's transposed form (CTDMRG_TC_TRANS=1 forces it): the kernel computes
    C^T = B A^T with B's rows as tile rows and stores its rows as C's columns, with alpha and
    beta; ragged shapes, every tile width, and (1024 x 4096 at 224) the stream-K last wave."""
    import ctypes as C
    import torch
    monkeypatch.setenv("CTDMRG_TC_TRANS", "1")
    monkeypatch.setenv("CTDMRG_TC_BN", bn)
    rng = np.random.default_rng(m + 7 * n + k)
    A = rng.standard_normal((m, k))
    B = rng.standard_normal((k, n))
    Cin = rng.standard_normal((m, n))
    ref = -0.75 * (A @ B) + 0.5 * Cin
    tA, tB, tC = dt(ctx, A), dt(ctx, B), dt(ctx, Cin)
    ctx.call("ct_gemm", 1, 0, 0, C.c_int64(m), C.c_int64(n), C.c_int64(k), C.c_double(-0.75),
             C.c_void_p(tA.storage.data_ptr()), C.c_int64(k), C.c_void_p(tB.storage.data_ptr()), C.c_int64(n),
             C.c_double(0.5), C.c_void_p(tC.storage.data_ptr()), C.c_int64(n))
    torch.cuda.synchronize()
    assert rel(tC.to_numpy(), ref) < TOL


def test_tc_gemm_accumulation_bias(ctx, monkeypatch):
    """All-positive operands, K = 5120: every partial sum has the same sign, so the
    truncating FP32 accumulation of the tensor cores shrinks the product coherently.
    In one accumulator that is ~3e-5 of the result; with a fresh accumulator every
    64 of K (the default) and the chunks added in FP32 with round-to-nearest it
    stays below 1e-6."""
    rng = np.random.default_rng(17)
    A = rng.random((256, 5120))
    B = rng.random((5120, 256))
    ref = A @ B
    monkeypatch.setenv("CTDMRG_TC_KCHUNK", "0")
    bias_single = float(np.mean(_tc_gemm(ctx, A, B) / ref - 1.0))
    monkeypatch.delenv("CTDMRG_TC_KCHUNK")
    out = _tc_gemm(ctx, A, B)
    bias_chunked = float(np.mean(out / ref - 1.0))
    assert bias_single < -5e-6, bias_single
    assert abs(bias_chunked) < 1e-6, bias_chunked
    assert np.max(np.abs(out / ref - 1.0)) < 2e-6


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
    """TFIM L=12 (converged eigensolve), mixed vs FP64 form.

    The tensor cores accumulate in FP32 with round-toward-zero, which shrinks
    every H_eff product by ~1e-7 per MMA step: the mixed form's Lanczos
    eigenvalues sit ~1e-6 above the FP64 ones (checked below at 1e-5).  A
    near-uniform shrinkage leaves the ground state's direction alone, so the
    FP64 Rayleigh quotient of the mixed-form MPS agrees with the FP64 form to
    |dE/E| <= 1e-9.
    """
    ct = ct_mod()
    L = 12
    mpo_a = oh.ising_1d(L, J=1.0, h_longitudinal=0.0, g_transverse=1.0)
    sites, _ = orng.create_random_mps_c_compatible(L, 2, 32, 0)
    mps_a = od.right_normalize(sites)
    res = {}
    for prec in ("fp64", "tf32x3"):
        p = ct.DMRGParams(num_sweeps=6, chi_max=32, eps_trunc=1e-10, max_krylov_iter=20, krylov_tol=1e-10,
                          energy_tol=0.0, max_rotations=0, prec=prec, final_rayleigh=True)
        st = ct.DMRGStats()
        E, out = ct.dmrg_two_site(ctx, ct.mpo_from_arrays(ctx, mpo_a), ct.mps_from_arrays(ctx, mps_a), p, st)
        res[prec] = (E, st.energy_rayleigh)
    E64, rq64 = res["fp64"]
    Emx, rqmx = res["tf32x3"]
    assert abs(rq64 - E64) < 1e-9 * abs(E64)
    assert abs(Emx - E64) < 1e-5 * abs(E64)
    assert abs(rqmx - E64) <= 1e-9 * abs(E64)
    assert abs(E64 - ed.ground_energy(mpo_a)) < 1e-8


@pytest.mark.parametrize("l2r", [True, False])
@pytest.mark.parametrize("dims,chi_max,eps", [((96, 2, 96), 150, 1e-10), ((96, 2, 80), 64, 0.0),
                                              ((50, 4, 60), 300, 1e-12)])
def test_svd_split_mixed(ctx, dims, chi_max, eps, l2r):
    """Mixed form with the spectrum returned, or with eps_trunc deciding chi: the split is the
    FP64 Jacobi's, so chi equals the oracle's, the discarded weight and the squared singular
    values agree to 1e-12, and the canonical factor is orthonormal to FP64 accuracy."""
    ct = ct_mod()
    Dl, d, Dr = dims
    rng = np.random.default_rng(Dl + 3 * Dr)
    m, n = Dl * d, d * Dr
    k = min(m, n)
    U0, _ = np.linalg.qr(rng.standard_normal((m, k)))
    V0, _ = np.linalg.qr(rng.standard_normal((n, k)))
    s0 = np.exp(-0.08 * np.arange(k))
    th = ((U0 * s0) @ V0.T).reshape(Dl, d, d, Dr)
    A_ref, B_ref, info = od.split_two_site_theta_svd(th, chi_max, eps, l2r)
    A, B, disc, S = ct.split_two_site_theta_svd(dt(ctx, th), chi_max, eps, ctx, l2r, return_spectrum=True,
                                                prec="tf32x3")
    chi = A.right_bond_dim()
    a, b = A.tensor.to_numpy(), B.tensor.to_numpy()
    assert chi == info.chi
    recon = np.tensordot(a, b, axes=([2], [0]))
    committed = np.sum((recon - th) ** 2) / np.sum(th * th)
    assert abs(committed - info.discarded_weight) <= 1e-12
    assert np.allclose(S[:chi] ** 2, info.S[:chi] ** 2, rtol=0, atol=1e-12 * info.S[0] ** 2)
    am, bm = a.reshape(-1, chi), b.reshape(chi, -1)
    if l2r:
        assert np.abs(am.T @ am - np.eye(chi)).max() < 1e-12
    else:
        assert np.abs(bm @ bm.T - np.eye(chi)).max() < 1e-12
    if chi == info.chi:
        prod = np.tensordot(a, b, axes=([2], [0]))
        prod_ref = np.tensordot(A_ref, B_ref, axes=([2], [0]))
        assert rel(prod, prod_ref) < 1e-5


@pytest.mark.parametrize("l2r", [True, False])
def test_svd_split_mixed_chi_max_binds(ctx, l2r):
    """eps_trunc > 0 far from the cut (the tail at chi_max = 64 is ~1e-5 of |theta|^2, eps 1e-10):
    the mixed split keeps its own result.  chi = chi_max as in the oracle; the reported discarded
    weight is that of the factors returned (FP64 projection) and, the excess over the optimal
    one being second order in the FP32 Jacobi's angles, within 1e-12 of the oracle's
    (measured: 6e-14)."""
    ct = ct_mod()
    Dl, d, Dr = 96, 2, 96
    rng = np.random.default_rng(17)
    m, n = Dl * d, d * Dr
    U0, _ = np.linalg.qr(rng.standard_normal((m, m)))
    V0, _ = np.linalg.qr(rng.standard_normal((n, m)))
    th = ((U0 * np.exp(-0.08 * np.arange(m))) @ V0.T).reshape(Dl, d, d, Dr)
    _, _, info = od.split_two_site_theta_svd(th, 64, 1e-10, l2r)
    A, B, disc = ct.split_two_site_theta_svd(dt(ctx, th), 64, 1e-10, ctx, l2r, prec="tf32x3")
    chi = A.right_bond_dim()
    assert chi == info.chi == 64
    a, b = A.tensor.to_numpy(), B.tensor.to_numpy()
    committed = np.sum((np.tensordot(a, b, axes=([2], [0])) - th) ** 2) / np.sum(th * th)
    assert abs(committed - disc) <= 1e-13
    assert abs(disc - info.discarded_weight) <= 1e-12
    am, bm = a.reshape(-1, chi), b.reshape(chi, -1)
    if l2r:
        assert np.abs(am.T @ am - np.eye(chi)).max() < 1e-12
    else:
        assert np.abs(bm @ bm.T - np.eye(chi)).max() < 1e-12


def test_dmrg_warm_subspace_split(ctx):
    """Heisenberg L=20, chi_max=128 (central bonds 256 x 256, chi_max binding), 4 sweeps in one
    call: after the first half-sweep the mixed form splits the large bonds by the warm-started
    subspace iteration; its FP64 Rayleigh energy matches the FP64 form (exact Jacobi splits) to
    1e-9 and the canonical factors are orthonormal to 1e-12."""
    ct = ct_mod()
    L = 20
    mpo_a = oh.spin_half_xxz(L, 1.0)
    sites, _ = orng.create_random_mps_c_compatible(L, 2, 128, 2)
    mps_a = od.right_normalize(sites)
    out = {}
    for prec in ("fp64", "tf32x3"):
        st = ct.DMRGStats()
        p = ct.DMRGParams(num_sweeps=4, chi_max=128, eps_trunc=0.0, max_krylov_iter=20, krylov_tol=1e-10,
                          energy_tol=0.0, max_rotations=0, prec=prec, final_rayleigh=True)
        E, mps = ct.dmrg_two_site(ctx, ct.mpo_from_arrays(ctx, mpo_a), ct.mps_from_arrays(ctx, mps_a), p, st)
        out[prec] = st
        if prec == "tf32x3":
            # the run ends right-to-left: sites 1.. are right-canonical to FP64 accuracy
            for a in mps.to_numpy()[1:]:
                mat = a.reshape(a.shape[0], -1)
                assert np.abs(mat @ mat.T - np.eye(a.shape[0])).max() < 1e-12
    assert out["tf32x3"].subspace_splits > 0
    e64 = out["fp64"].energy_rayleigh
    assert abs(out["tf32x3"].energy_rayleigh - e64) <= 1e-9 * abs(e64)


def test_dmrg_keep_bases_across_calls(ctx):
    """keep_bases: a call that continues the previous call's MPS on the same handle starts its
    first left-to-right half-sweep from the kept bases (more subspace splits than a cold call),
    and the energy keeps improving."""
    ct = ct_mod()
    L = 20
    mpo = ct.mpo_from_arrays(ctx, oh.spin_half_xxz(L, 1.0))
    sites, _ = orng.create_random_mps_c_compatible(L, 2, 128, 3)
    mps = ct.mps_from_arrays(ctx, od.right_normalize(sites))

    def params(keep):
        return ct.DMRGParams(num_sweeps=1, chi_max=128, eps_trunc=0.0, max_krylov_iter=20, krylov_tol=1e-10,
                             energy_tol=0.0, max_rotations=0, prec="tf32x3", final_rayleigh=True, keep_bases=keep)

    st1 = ct.DMRGStats()
    p1 = params(False)
    p1.num_sweeps = 2
    E1, mps = ct.dmrg_two_site(ctx, mpo, mps, p1, st1)
    st_keep = ct.DMRGStats()
    E2, mps = ct.dmrg_two_site(ctx, mpo, mps, params(True), st_keep)
    st_cold = ct.DMRGStats()
    E3, mps = ct.dmrg_two_site(ctx, mpo, mps, params(False), st_cold)
    assert st_cold.subspace_splits > 0
    assert st_keep.subspace_splits > st_cold.subspace_splits
    assert st_keep.subspace_splits + st_keep.exact_splits == st_cold.subspace_splits + st_cold.exact_splits
    # sweeps at fixed chi_max do not raise the energy beyond truncation noise
    assert st_keep.energy_rayleigh <= st1.energy_rayleigh + 1e-8 * abs(E1)
    assert st_cold.energy_rayleigh <= st_keep.energy_rayleigh + 1e-8 * abs(E1)


def test_dmrg_cold_subspace_split(ctx):
    """cold_power_steps: first visits of large bonds use the subspace split from random rows (two
    power steps) instead of the Jacobi SVD; after four sweeps the FP64 Rayleigh energy matches the
    FP64 form to 1e-9 and the sites stay right-canonical."""
    ct = ct_mod()
    L = 20
    mpo_a = oh.spin_half_xxz(L, 1.0)
    sites, _ = orng.create_random_mps_c_compatible(L, 2, 128, 2)
    mps_a = od.right_normalize(sites)
    out = {}
    for prec, cold in (("fp64", -1), ("tf32x3", 2)):
        st = ct.DMRGStats()
        p = ct.DMRGParams(num_sweeps=4, chi_max=128, eps_trunc=0.0, max_krylov_iter=20, krylov_tol=1e-10,
                          energy_tol=0.0, max_rotations=0, prec=prec, final_rayleigh=True, cold_power_steps=cold)
        E, mps = ct.dmrg_two_site(ctx, ct.mpo_from_arrays(ctx, mpo_a), ct.mps_from_arrays(ctx, mps_a), p, st)
        out[prec] = st
        if prec == "tf32x3":
            for a in mps.to_numpy()[1:]:
                mat = a.reshape(a.shape[0], -1)
                assert np.abs(mat @ mat.T - np.eye(a.shape[0])).max() < 1e-12
    assert out["tf32x3"].cold_splits > 0
    e64 = out["fp64"].energy_rayleigh
    assert abs(out["tf32x3"].energy_rayleigh - e64) <= 1e-9 * abs(e64)


@pytest.mark.parametrize("l2r", [True, False])
def test_svd_split_warm_entry(ctx, l2r):
    """ct_svd_split_warm (C ABI): from a slightly perturbed exact basis, the split is accepted,
    the canonical factor is orthonormal to 1e-12, A B reproduces the rank-chi truncation of theta
    to the optimal discarded weight (within the TF32x3 resolution of the residual), and the kept
    basis it writes spans the same subspace as the canonical factor."""
    import ctypes as C
    import torch
    ct = ct_mod()
    Dl, d, Dr, c = 256, 2, 256, 200
    m, n = Dl * d, d * Dr
    rng = np.random.default_rng(7)
    U, _ = np.linalg.qr(rng.standard_normal((m, m)))
    V, _ = np.linalg.qr(rng.standard_normal((n, n)))
    s = np.exp(-0.02 * np.arange(m))
    M = (U * s) @ V.T
    X0 = (V[:, :c] if l2r else U[:, :c]) + 1e-6 * rng.standard_normal(((n if l2r else m), c))
    X, _ = np.linalg.qr(X0)
    dev = ctx.torch_device
    th = torch.from_numpy(M.reshape(Dl, d, d, Dr).copy()).to(dev)
    Xd = torch.from_numpy(np.ascontiguousarray(X.T)).to(dev)
    bout = torch.zeros(c * (m if l2r else n), dtype=torch.float64, device=dev)
    A = torch.zeros(m * c, dtype=torch.float64, device=dev)
    B = torch.zeros(c * n, dtype=torch.float64, device=dev)
    acc, disc = C.c_int(), C.c_double()
    piv = (C.c_double * 3)()
    ctx.call("ct_svd_split_warm", C.c_void_p(th.data_ptr()), Dl, d, Dr, c, int(l2r), C.c_void_p(Xd.data_ptr()), 0,
             C.c_void_p(bout.data_ptr()), C.c_void_p(A.data_ptr()), C.c_void_p(B.data_ptr()), C.byref(acc),
             C.byref(disc), piv)
    torch.cuda.synchronize()
    assert acc.value == 1 and piv[2] == 0
    a = A.cpu().numpy().reshape(m, c)
    b = B.cpu().numpy().reshape(c, n)
    can = a.T @ a if l2r else b @ b.T
    assert np.abs(can - np.eye(c)).max() < 1e-12
    opt = np.sum(s[c:] ** 2) / np.sum(s ** 2)
    err = np.sum((a @ b - M) ** 2) / np.sum(s ** 2)
    assert err <= opt * (1 + 1e-3) + 1e-9
    assert abs(disc.value - err) <= 1e-9
    kept = bout.cpu().numpy().reshape(c, -1)
    canon = a.T if l2r else b
    # same row space: projecting the kept rows on the canonical rows loses nothing
    assert np.abs(kept @ canon.T @ canon - kept).max() < 1e-10


def test_dmrg_cold_split_rank_completion(ctx):
    """A chi ramp with d = 4 and a step smaller than d (Bose-Hubbard L=12, chi 32 -> 64): on the
    first left-to-right visit at chi = 64, theta is (4 Dl) x (4 Dr) with the right bond still at
    32, so its numerical rank is about 32 while 64 states are kept.  The cold subspace split
    completes the missing rows with random ones instead of falling back to the Jacobi SVD: rows
    are completed, the sites stay right-canonical, and after the ramp the FP64 Rayleigh energy
    matches the FP64 form (same ramp, Jacobi splits) to 1e-8."""
    ct = ct_mod()
    L, d = 12, 4
    mpo_a = oh.bose_hubbard(L, d, t=1.0, u=4.0, mu=0.0)
    sites, _ = orng.create_random_mps_c_compatible(L, d, 32, 7)
    mps_a = od.right_normalize(sites)
    res = {}
    for prec, cold in (("fp64", -1), ("tf32x3", 2)):
        mps = ct.mps_from_arrays(ctx, mps_a)
        stages = []
        for k, (chi, ns) in enumerate(((32, 2), (64, 3))):
            st = ct.DMRGStats()
            p = ct.DMRGParams(num_sweeps=ns, chi_max=chi, eps_trunc=0.0, max_krylov_iter=20, krylov_tol=1e-10,
                              energy_tol=0.0, max_rotations=0, prec=prec, final_rayleigh=True,
                              keep_bases=k > 0, cold_power_steps=cold)
            E, mps = ct.dmrg_two_site(ctx, ct.mpo_from_arrays(ctx, mpo_a), mps, p, st)
            stages.append(st)
        res[prec] = (stages, mps)
    st_b = res["tf32x3"][0][1]
    assert st_b.completed_rows > 0
    for a in res["tf32x3"][1].to_numpy()[1:]:
        mat = a.reshape(a.shape[0], -1)
        assert np.abs(mat @ mat.T - np.eye(a.shape[0])).max() < 1e-12
    e64 = res["fp64"][0][1].energy_rayleigh
    assert abs(st_b.energy_rayleigh - e64) <= 1e-8 * abs(e64)
