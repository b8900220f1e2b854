"""Parity of every device building block against the CPU FP64 oracle (FP64 form).

Tolerances: the FP64 form must agree with the oracle to rounding, so
contractions are compared at 1e-12 relative to the output norm, Lanczos
energies at 1e-10 relative, singular values at 1e-12 relative to s_max and
kept bond dimensions exactly.
"""
import numpy as np
import pytest
import torch

from oracle import dmrg as od
from oracle import hamiltonians as oh

pytestmark = pytest.mark.gpu

RTOL_CONTRACT = 1e-12


def ct_mod():
    import chemtensor_mojo_gb300 as ct
    return ct


def dt(ctx, a):
    return ct_mod().create_dense_tensor_from_data(ctx, a, a.shape)


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300)


def rand(rng, *shape):
    return rng.standard_normal(shape)


def sym_mpo(rng, wl, d, wr):
    W = rng.standard_normal((wl, d, d, wr))
    return 0.5 * (W + W.transpose(0, 2, 1, 3))


HEFF_SHAPES = [
    # Dl, d, Dr, wL, wM, wR
    (1, 2, 1, 1, 3, 3),
    (3, 2, 5, 3, 3, 3),
    (16, 2, 16, 5, 5, 5),
    (33, 2, 17, 5, 5, 1),
    (20, 4, 12, 4, 4, 4),
    (7, 4, 9, 6, 6, 6),
    (64, 2, 64, 5, 5, 5),
]


@pytest.mark.parametrize("shape", HEFF_SHAPES)
def test_heff_apply_matches_oracle(ctx, shape):
    ct = ct_mod()
    Dl, d, Dr, wL, wM, wR = shape
    rng = np.random.default_rng(sum(shape))
    th = rand(rng, Dl, d, d, Dr)
    L = rand(rng, wL, Dl, Dl)
    R = rand(rng, wR, Dr, Dr)
    W1 = sym_mpo(rng, wL, d, wM)
    W2 = sym_mpo(rng, wM, d, wR)
    ref = od.apply_two_site_heff(th, L, R, W1, W2)
    out = ct.apply_two_site_heff(dt(ctx, th), dt(ctx, L), dt(ctx, R), ct.MPOSite(dt(ctx, W1)),
                                 ct.MPOSite(dt(ctx, W2)), ctx)
    assert rel(out.to_numpy(), ref) < RTOL_CONTRACT


ENV_SHAPES = [(1, 2, 2, 1, 3), (4, 2, 8, 3, 3), (16, 2, 7, 5, 5), (9, 4, 11, 4, 4), (32, 2, 32, 5, 1), (5, 3, 4, 2, 6)]


@pytest.mark.parametrize("shape", ENV_SHAPES)
def test_left_environment_matches_oracle(ctx, shape):
    ct = ct_mod()
    Dl, d, Dr, wL, wR = shape
    rng = np.random.default_rng(100 + sum(shape))
    L = rand(rng, wL, Dl, Dl)
    A = rand(rng, Dl, d, Dr)
    W = rand(rng, wL, d, d, wR)
    ref = od.update_left_environment(L, A, W)
    out = ct.update_left_environment(dt(ctx, L), ct.MPSSite(dt(ctx, A)), ct.MPOSite(dt(ctx, W)), ctx)
    assert out.shape == [wR, Dr, Dr]
    assert rel(out.to_numpy(), ref) < RTOL_CONTRACT


@pytest.mark.parametrize("shape", ENV_SHAPES)
def test_right_environment_matches_oracle(ctx, shape):
    ct = ct_mod()
    Dl, d, Dr, wL, wR = shape
    rng = np.random.default_rng(200 + sum(shape))
    R = rand(rng, wR, Dr, Dr)
    A = rand(rng, Dl, d, Dr)
    W = rand(rng, wL, d, d, wR)
    ref = od.update_right_environment(R, A, W)
    out = ct.update_right_environment(dt(ctx, R), ct.MPSSite(dt(ctx, A)), ct.MPOSite(dt(ctx, W)), ctx)
    assert out.shape == [wL, Dl, Dl]
    assert rel(out.to_numpy(), ref) < RTOL_CONTRACT


def test_theta_matches_oracle(ctx):
    ct = ct_mod()
    rng = np.random.default_rng(5)
    A = rand(rng, 13, 2, 21)
    B = rand(rng, 21, 2, 6)
    ref = od.build_two_site_theta(A, B)
    out = ct.build_two_site_theta(ct.MPSSite(dt(ctx, A)), ct.MPSSite(dt(ctx, B)), ctx)
    assert out.shape == [13, 2, 2, 6]
    assert rel(out.to_numpy(), ref) < RTOL_CONTRACT


@pytest.mark.parametrize("case", [
    # shapes of A, B, ndim_mult, axrange_A, axrange_B (dense_tensor_dot semantics)
    ((3, 4), (4, 5), 1, False, False),
    ((3, 4), (5, 4), 1, False, False),          # inferred trailing B
    ((2, 3, 4), (4, 5, 6), 1, False, False),
    ((2, 3, 4, 5), (4, 5, 6, 7), 2, False, False),
    ((4, 2, 3), (5, 6, 4), 1, True, False),     # A leading, B trailing
    ((4, 2, 3), (4, 6), 1, True, True),         # both leading
    ((4, 4), (4, 4), 1, False, False),          # square: leading preferred
    ((7,), (7,), 1, False, False),              # scalar result
])
def test_dense_tensor_dot_semantics(ctx, case):
    ct = ct_mod()
    sa, sb, nm, ra, rb = case
    rng = np.random.default_rng(len(sa) * 10 + len(sb))
    A = rand(rng, *sa)
    B = rand(rng, *sb)
    rA, rB = len(sa), len(sb)
    eff_b = rb
    if not ra and not rb:
        lead = all(sa[rA - nm + i] == sb[i] for i in range(nm))
        trail = all(sa[rA - nm + i] == sb[rB - nm + i] for i in range(nm))
        eff_b = True if lead else (False if trail else True)
    ax_a = list(range(nm)) if ra else list(range(rA - nm, rA))
    ax_b = list(range(nm)) if eff_b else list(range(rB - nm, rB))
    ref = np.tensordot(A, B, axes=(ax_a, ax_b))
    out_shape = list(ref.shape) if ref.ndim else [1]
    Cout = ct.create_dense_tensor(ctx, out_shape)
    ct.dense_tensor_dot(Cout, dt(ctx, A), dt(ctx, B), ctx, ndim_mult=nm, axrange_A=ra, axrange_B=rb)
    assert rel(Cout.to_numpy().reshape(ref.shape), ref) < 1e-13


def test_dense_tensor_dot_shape_errors(ctx):
    ct = ct_mod()
    A = ct.create_dense_tensor(ctx, [3, 4])
    B = ct.create_dense_tensor(ctx, [5, 6])
    with pytest.raises(ValueError):
        ct.dense_tensor_dot(ct.create_dense_tensor(ctx, [3, 6]), A, B, ctx)
    with pytest.raises(ValueError):
        ct.dense_tensor_dot(ct.create_dense_tensor(ctx, [3, 3]), A, ct.create_dense_tensor(ctx, [4, 5]), ctx)


def test_vector_ops(ctx):
    ct = ct_mod()
    rng = np.random.default_rng(9)
    for n in (1, 2, 3, 1001, 1 << 20):
        x = rand(rng, n)
        y = rand(rng, n)
        X, Y = dt(ctx, x), dt(ctx, y)
        assert abs(X.dot_product(Y, ctx) - x @ y) <= 1e-12 * np.linalg.norm(x) * np.linalg.norm(y)
        assert abs(X.norm_sq(ctx) - x @ x) <= 1e-12 * (x @ x)
        Y.axpy_in_place(0.5, X, ctx)
        assert rel(Y.to_numpy(), y + 0.5 * x) < 1e-15
        X.scale_in_place(-2.0, ctx)
        assert rel(X.to_numpy(), -2.0 * x) < 1e-15


def test_transpose_matches_numpy(ctx):
    ct = ct_mod()
    rng = np.random.default_rng(3)
    a = rand(rng, 3, 4, 5, 2)
    for perm in ([1, 0, 2, 3], [3, 2, 1, 0], [1, 3, 0, 2]):
        t = dt(ctx, a).transpose(perm, ctx)
        assert np.array_equal(t.to_numpy(), a.transpose(perm))


def _lanczos_case(seed, Dl, d, Dr, wL, wM, wR):
    rng = np.random.default_rng(seed)
    th = rand(rng, Dl, d, d, Dr)
    L = rand(rng, wL, Dl, Dl)
    L = 0.5 * (L + L.transpose(0, 2, 1))
    R = rand(rng, wR, Dr, Dr)
    R = 0.5 * (R + R.transpose(0, 2, 1))
    W1 = sym_mpo(rng, wL, d, wM)
    W2 = sym_mpo(rng, wM, d, wR)
    return th, L, R, W1, W2


@pytest.mark.parametrize("max_rot", [200, 0])
@pytest.mark.parametrize("dims", [(4, 2, 4, 3, 3, 3), (12, 2, 9, 5, 5, 5), (6, 4, 5, 4, 4, 4)])
def test_lanczos_matches_oracle(ctx, dims, max_rot):
    ct = ct_mod()
    th, L, R, W1, W2 = _lanczos_case(sum(dims), *dims)
    tr = od.LanczosTrace()
    E_ref, v_ref = od.lanczos_two_site_optimize(th, L, R, W1, W2, 16, 1e-10,
                                                eig="jacobi" if max_rot else "exact", trace=tr)
    info = ct.dmrg.LanczosInfo(0, [], [])
    E, v = ct.lanczos_two_site_optimize(dt(ctx, th), dt(ctx, L), dt(ctx, R), ct.MPOSite(dt(ctx, W1)),
                                        ct.MPOSite(dt(ctx, W2)), ctx, max_iter=16, tol=1e-10,
                                        max_rotations=max_rot, info=info)
    assert info.numiter == tr.numiter
    assert np.allclose(info.alpha, tr.alpha, rtol=1e-9, atol=1e-9 * np.abs(tr.alpha).max())
    assert abs(E - E_ref) <= 1e-10 * max(1.0, abs(E_ref))
    # Ritz vectors agree up to sign
    vv = v.to_numpy().reshape(-1)
    vr = v_ref.reshape(-1)
    assert abs(abs(vv @ vr) - 1.0) < 1e-8


@pytest.mark.parametrize("prec", ["fp64", "tf32x3"])
@pytest.mark.parametrize("dims", [(12, 2, 9, 5, 5, 5), (6, 4, 5, 4, 4, 4), (40, 2, 33, 5, 5, 5)])
def test_lanczos_reorth_matches_oracle(ctx, dims, prec):
    """Reorthogonalised Lanczos (the reference recurrence, then one Gram-Schmidt pass of w
    against the whole Krylov basis, fused into two kernels with last-block reductions)
    against the oracle's recurrence followed by Gram-Schmidt.  FP64: alpha, beta and the
    energy to 1e-9 / 1e-10; TF32x3 (tensor-core H_eff): the energy to 1e-6."""
    ct = ct_mod()
    th, L, R, W1, W2 = _lanczos_case(sum(dims) + 7, *dims)
    tr = od.LanczosTrace()
    E_ref, v_ref = od.lanczos_two_site_optimize(th, L, R, W1, W2, 20, 1e-10, eig="exact", trace=tr, reorth=True)
    info = ct.dmrg.LanczosInfo(0, [], [])
    E, v = ct.lanczos_two_site_optimize(dt(ctx, th), dt(ctx, L), dt(ctx, R), ct.MPOSite(dt(ctx, W1)),
                                        ct.MPOSite(dt(ctx, W2)), ctx, max_iter=20, tol=1e-10, prec=prec,
                                        max_rotations=0, reorth=True, info=info)
    assert info.numiter == tr.numiter
    if prec == "fp64":
        scale = np.abs(tr.alpha).max()
        assert np.allclose(info.alpha, tr.alpha, rtol=1e-9, atol=1e-9 * scale)
        assert np.allclose(info.beta, tr.beta, rtol=1e-9, atol=1e-9 * scale)
        assert abs(E - E_ref) <= 1e-10 * max(1.0, abs(E_ref))
        vv = v.to_numpy().reshape(-1)
        assert abs(abs(vv @ v_ref.reshape(-1)) - 1.0) < 1e-8
    else:
        assert abs(E - E_ref) <= 1e-6 * max(1.0, abs(E_ref))


@pytest.mark.parametrize("dims", [(1, 2, 4, 1, 3, 3), (2, 2, 3, 3, 3, 3), (3, 2, 2, 3, 3, 1), (2, 4, 2, 3, 3, 3)])
def test_lanczos_mixed_exhausted_krylov(ctx, dims):
    """Mixed form, reorthogonalised, on bonds whose whole space (N = Dl d^2 Dr <= 32) is smaller
    than or equal to 24 Lanczos steps, as at the ends of a chain: the Krylov space closes, w after
    the recurrence lies almost entirely inside the basis, and the FP32 pass alone would leave a
    1e-7 residual along it that is not small against beta (ghost eigenvalues far below the
    spectrum were measured).  The gated FP64 pass must take over: the energy equals the lowest
    eigenvalue of the dense H_eff to 1e-6 and never lies below it by more."""
    ct = ct_mod()
    th, L, R, W1, W2 = _lanczos_case(101 + sum(dims), *dims)
    Dl, d, Dr = dims[0], dims[1], dims[2]
    n = Dl * d * d * Dr
    H = np.zeros((n, n))
    for i in range(n):
        e = np.zeros(n)
        e[i] = 1.0
        H[:, i] = od.apply_two_site_heff(e.reshape(Dl, d, d, Dr), L, R, W1, W2).reshape(-1)
    e0 = np.linalg.eigvalsh(0.5 * (H + H.T))[0]
    E, _ = ct.lanczos_two_site_optimize(dt(ctx, th), dt(ctx, L), dt(ctx, R), ct.MPOSite(dt(ctx, W1)),
                                        ct.MPOSite(dt(ctx, W2)), ctx, max_iter=24, tol=1e-10, prec="tf32x3",
                                        max_rotations=0, reorth=True)
    scale = max(1.0, np.abs(np.linalg.eigvalsh(0.5 * (H + H.T))).max())
    assert abs(E - e0) <= 1e-6 * scale


def test_lanczos_breakdown_matches_oracle(ctx):
    """Rank-deficient H_eff: the Krylov space closes early (beta below 100 n eps)."""
    ct = ct_mod()
    Dl, d, Dr = 1, 2, 1
    L = np.ones((1, 1, 1))
    R = np.ones((1, 1, 1))
    W1 = np.zeros((1, d, d, 1))
    W1[0, :, :, 0] = np.diag([1.0, -1.0])
    W2 = np.zeros((1, d, d, 1))
    W2[0, :, :, 0] = np.eye(2)
    th = np.array([1.0, 2.0, 3.0, 4.0]).reshape(1, 2, 2, 1)
    tr = od.LanczosTrace()
    E_ref, _ = od.lanczos_two_site_optimize(th, L, R, W1, W2, 10, 1e-12, trace=tr)
    info = ct.dmrg.LanczosInfo(0, [], [])
    E, _ = ct.lanczos_two_site_optimize(dt(ctx, th), dt(ctx, L), dt(ctx, R), ct.MPOSite(dt(ctx, W1)),
                                        ct.MPOSite(dt(ctx, W2)), ctx, max_iter=10, tol=1e-12, info=info)
    assert tr.numiter < 10
    assert info.numiter == tr.numiter
    assert abs(E - E_ref) < 1e-12


def test_lanczos_zero_norm_raises(ctx):
    ct = ct_mod()
    th = np.zeros((2, 2, 2, 2))
    L = np.ones((1, 2, 2))
    R = np.ones((1, 2, 2))
    W = np.ones((1, 2, 2, 1))
    with pytest.raises(ct.CTDMRGError) as e:
        ct.lanczos_two_site_optimize(dt(ctx, th), dt(ctx, L), dt(ctx, R), ct.MPOSite(dt(ctx, W)),
                                     ct.MPOSite(dt(ctx, W)), ctx, max_iter=4)
    assert e.value.status == -5


# ---- SVD -----------------------------------------------------------------------
def lcg_data(nelem, seed):
    """make_host_data_f32 of src/tests/test_utils.mojo:13-21 (values in [-0.5, 0.5))."""
    state = seed
    out = []
    for _ in range(nelem):
        state = (1664525 * state + 1013904223) % (1 << 32)
        out.append(np.float32(state / float(1 << 32) - 0.5))
    return np.array(out, dtype=np.float64)


@pytest.mark.parametrize("n,rate", [(32, 0.5), (512, 0.04), (512, 0.12)])
def test_svd_split_decaying_spectrum(ctx, n, rate):
    """FP64 split of theta whose singular values decay geometrically far below machine
    precision (exp(-rate k); 512 x 2 = 1024: the cooperative Jacobi, 32 x 2: one CTA), the
    shape of a converged DMRG bond.  The rotations among the tiny columns sit at the noise
    floor of the FP64 dot products; the split must converge (no CT_ERR_NOCONV), keep an
    orthonormal canonical factor and give the spectrum to 1e-13 of s_0."""
    import ctypes as C
    import torch
    ct = ct_mod()
    m = 2 * n
    rng = np.random.default_rng(n + int(rate * 100))
    U, _ = np.linalg.qr(rng.standard_normal((m, m)))
    V, _ = np.linalg.qr(rng.standard_normal((m, m)))
    s = np.exp(-rate * np.arange(m))
    th = ((U * s) @ V.T).reshape(n, 2, 2, n)
    A, B, disc, S = ct.split_two_site_theta_svd(dt(ctx, th), m, 0.0, ctx, True, return_spectrum=True)
    chi = A.right_bond_dim()
    am = A.tensor.to_numpy().reshape(-1, chi)
    assert np.abs(am.T @ am - np.eye(chi)).max() < 1e-12
    ref = np.linalg.svd(th.reshape(m, m), compute_uv=False)
    assert np.allclose(S[:chi], ref[:chi], rtol=0, atol=1e-13 * ref[0])
    sweeps = C.c_int()
    total = C.c_int64()
    ctx.call("ct_svd_sweeps", C.byref(sweeps), C.byref(total))
    assert 0 < sweeps.value < 48


@pytest.mark.parametrize("m,n", [(300, 200), (200, 300), (512, 512)])
def test_svd_trunc_qr_preconditioned_shapes(ctx, m, n):
    """ct_svd_trunc above the one-CTA size: the Householder-QR-preconditioned Jacobi on the
    shorter side.  Singular values to 1e-13 of s_0, both factors orthonormal to 1e-12 (no
    singular value below the noise floor here), reconstruction to 1e-13."""
    ct = ct_mod()
    rng = np.random.default_rng(m + 7 * n)
    M = rng.standard_normal((m, n)) * np.exp(-0.03 * np.arange(n))[None, :]
    U, S, Vt, c = ct.dense_tensor_svd_trunc(dt(ctx, M), ctx, chi_max=1 << 30, eps_trunc=0.0)
    u, s, vt = U.to_numpy(), S.to_numpy(), Vt.to_numpy()
    ref = np.linalg.svd(M, compute_uv=False)
    assert c == min(m, n)
    assert np.abs(s - ref).max() <= 1e-13 * ref[0]
    assert np.abs(u.T @ u - np.eye(c)).max() < 1e-12
    assert np.abs(vt @ vt.T - np.eye(c)).max() < 1e-12
    assert np.abs((u * s) @ vt - M).max() <= 1e-13 * np.abs(M).max()


def test_mps_schmidt_values_below_noise_floor(ctx):
    """Schmidt values of a 16-site state whose middle bond carries a spectrum down to 1e-30
    (below the Jacobi's eps |M|_F floor, so the normalised factor U = X / sigma is noise there):
    every bond's weights sum to 1 within 1e-12 and match the state vector's SVD to 1e-13."""
    ct = ct_mod()
    L = 16
    arrays, _ = ct.random_mps_c_compatible_arrays(L, 2, 256, 9)
    sites = od.right_normalize(arrays)
    mid = sites[7]
    lam = np.exp(-np.linspace(0.0, 69.0, mid.shape[2]))
    sites[7] = mid * lam[None, None, :]
    sites = od.right_normalize(sites)
    mps = ct.mps_from_arrays(ctx, sites)
    sv = ct.mps_schmidt_values(mps, ctx)
    psi = od.mps_to_statevector(sites)
    psi = psi / np.linalg.norm(psi)
    assert min(float(x.min()) for x in sv) < 1e-20
    for b, x in enumerate(sv):
        assert abs(np.sum(x * x) - 1.0) < 1e-12, b
        r = np.linalg.svd(psi.reshape(2 ** (b + 1), -1), compute_uv=False)
        k = min(len(x), len(r))
        assert np.abs(x[:k] - r[:k]).max() < 1e-13, b


def test_svd_known_singular_values(ctx):
    """test_svd_lapack.mojo:55-91: rank-2 4x3 matrix with singular values [3, 2]."""
    ct = ct_mod()
    a = np.array([[2.0, 0, 0], [0, 3.0, 0], [0, 0, 0], [0, 0, 0]])
    U, S, Vt, chi = ct.dense_tensor_svd_trunc(dt(ctx, a), ctx, chi_max=2, eps_trunc=1e-12)
    assert chi == 2 and U.shape == [4, 2] and S.shape == [2] and Vt.shape == [2, 3]
    assert np.allclose(S.to_numpy(), [3.0, 2.0], atol=1e-14)


@pytest.mark.parametrize("m,n,chi_max,seed", [(6, 4, 4, 200), (8, 5, 5, 301), (5, 7, 5, 302), (6, 4, 4, 400),
                                              (5, 3, 10, 501), (3, 3, 3, 600), (2, 5, 2, 700), (4, 3, 2, 800)])
def test_svd_lapack_fixtures(ctx, m, n, chi_max, seed):
    """The LCG fixtures of test_svd_lapack.mojo:94-263, checked at FP64 tolerance."""
    ct = ct_mod()
    a = lcg_data(m * n, seed).reshape(m, n)
    U, S, Vt, chi = ct.dense_tensor_svd_trunc(dt(ctx, a), ctx, chi_max=chi_max, eps_trunc=0.0)
    Ur, Sr, Vtr, chir = od.svd_trunc(a, chi_max, 0.0)
    assert chi == chir == min(m, n, chi_max)
    s = S.to_numpy()
    assert np.allclose(s, Sr, atol=1e-13 * Sr[0])
    assert np.all(np.diff(s) <= 0) and np.all(s >= 0)
    u, vt = U.to_numpy(), Vt.to_numpy()
    assert np.allclose(u.T @ u, np.eye(chi), atol=1e-12)
    assert np.allclose(vt @ vt.T, np.eye(chi), atol=1e-12)
    recon = (u * s) @ vt
    best = (Ur * Sr) @ Vtr
    assert np.linalg.norm(recon - best) < 1e-12 * np.linalg.norm(a)


def test_svd_eps_trunc_monotone(ctx):
    ct = ct_mod()
    a = lcg_data(16, 900).reshape(4, 4)
    _, _, _, chi_full = ct.dense_tensor_svd_trunc(dt(ctx, a), ctx, chi_max=4, eps_trunc=0.0)
    _, _, _, chi_tr = ct.dense_tensor_svd_trunc(dt(ctx, a), ctx, chi_max=4, eps_trunc=0.5)
    assert chi_full == 4 and chi_tr <= chi_full
    assert chi_tr == od.svd_trunc(a, 4, 0.5)[3]


@pytest.mark.parametrize("l2r", [True, False])
@pytest.mark.parametrize("dims,chi_max,eps", [((8, 2, 8), 16, 1e-10), ((8, 2, 8), 5, 1e-10),
                                              ((16, 2, 4), 32, 0.0), ((5, 4, 7), 9, 1e-3),
                                              ((40, 2, 40), 64, 1e-10), ((70, 2, 80), 100, 1e-12)])
def test_svd_split_matches_oracle(ctx, dims, chi_max, eps, l2r):
    ct = ct_mod()
    Dl, d, Dr = dims
    rng = np.random.default_rng(Dl * 7 + Dr)
    # graded spectrum so that eps truncation is exercised
    U0, _ = np.linalg.qr(rng.standard_normal((Dl * d, Dl * d)))
    V0, _ = np.linalg.qr(rng.standard_normal((d * Dr, d * Dr)))
    k = min(Dl * d, d * Dr)
    s0 = np.exp(-0.35 * np.arange(k))
    th = ((U0[:, :k] * s0) @ V0[:, :k].T).reshape(Dl, d, d, Dr)
    A_ref, B_ref, info = od.split_two_site_theta_svd(th, chi_max, eps, l2r)
    A, B, disc, S = ct.split_two_site_theta_svd(dt(ctx, th), chi_max, eps, ctx, l2r, return_spectrum=True)
    assert A.right_bond_dim() == info.chi
    assert np.allclose(S, info.S, atol=1e-13 * info.S[0])
    assert abs(disc - info.discarded_weight) < 1e-13
    a, b = A.tensor.to_numpy(), B.tensor.to_numpy()
    prod = np.tensordot(a, b, axes=([2], [0]))
    prod_ref = np.tensordot(A_ref, B_ref, axes=([2], [0]))
    assert rel(prod, prod_ref) < 1e-12
    am = a.reshape(-1, info.chi)
    bm = b.reshape(info.chi, -1)
    if l2r:
        assert np.allclose(am.T @ am, np.eye(info.chi), atol=1e-12)
    else:
        assert np.allclose(bm @ bm.T, np.eye(info.chi), atol=1e-12)


def test_svd_split_large_path(ctx):
    """A split whose Jacobi does not fit one CTA's shared memory (multi-launch path)."""
    ct = ct_mod()
    Dl, d, Dr = 96, 2, 96
    rng = np.random.default_rng(77)
    th = rng.standard_normal((Dl, d, d, Dr)) * np.exp(-0.02 * np.arange(Dr))
    for l2r in (True, False):
        A_ref, B_ref, info = od.split_two_site_theta_svd(th, 150, 1e-10, l2r)
        A, B, disc, S = ct.split_two_site_theta_svd(dt(ctx, th), 150, 1e-10, ctx, l2r, return_spectrum=True)
        assert A.right_bond_dim() == info.chi
        assert np.allclose(S, info.S, atol=1e-12 * info.S[0])
        prod = np.tensordot(A.tensor.to_numpy(), B.tensor.to_numpy(), axes=([2], [0]))
        assert rel(prod, np.tensordot(A_ref, B_ref, axes=([2], [0]))) < 1e-11


def test_workspace_limit_reports_oom(ctx):
    ct = ct_mod()
    h2 = ct.DeviceContext(0)
    h2.set_workspace_limit(1 << 10)
    rng = np.random.default_rng(1)
    th = rand(rng, 16, 2, 2, 16)
    L = rand(rng, 5, 16, 16)
    R = rand(rng, 5, 16, 16)
    W = rand(rng, 5, 2, 2, 5)
    with pytest.raises(ct.CTDMRGError) as e:
        ct.apply_two_site_heff(dt(h2, th), dt(h2, L), dt(h2, R), ct.MPOSite(dt(h2, W)), ct.MPOSite(dt(h2, W)), h2)
    assert e.value.status == -3
