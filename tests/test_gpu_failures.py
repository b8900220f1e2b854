"""Failure paths through the C ABI: non-finite inputs and iteration caps.

The reference raises where LAPACK's dgesdd reports a failure
(src/mylinalg/svd.mojo:74-76) and where the Lanczos start vector has zero
norm (src/algorithms/dmrg.mojo:605-611); a NaN or an infinity in its inputs
it carries on into NaN energies.  Here a NaN or an infinity planted into a
host array before upload makes the entry point return CT_ERR_NONFINITE, and a
Jacobi sweep cap of 1 (ct_set_svd_max_sweeps) makes an SVD that needs more
sweeps return CT_ERR_NOCONV.  Every wait on the device is bounded, so none of
these cases can hang; after each failure the same handle runs a clean call.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import dmrg as od
from oracle import hamiltonians as oh
from oracle import rng as orng

pytestmark = pytest.mark.gpu


def _lib():
    from chemtensor_mojo_gb300 import _lib as L
    return L


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def _p(t):
    return C.c_void_p(t.data_ptr())


@pytest.fixture()
def handle():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    L = _lib()
    lib = L.load()
    torch.cuda.set_device(0)
    h = C.c_void_p()
    L.check(lib.ct_create(0, None, C.byref(h)), "ct_create")
    yield lib, h
    lib.ct_destroy(h)


def _heff_inputs(seed, Dl=6, d=2, Dr=6, w=3):
    rng = np.random.default_rng(seed)
    L = rng.standard_normal((w, Dl, Dl))
    R = rng.standard_normal((w, Dr, Dr))
    W = rng.standard_normal((w, d, d, w))
    return (rng.standard_normal((Dl, d, d, Dr)), 0.5 * (L + L.transpose(0, 2, 1)),
            0.5 * (R + R.transpose(0, 2, 1)), 0.5 * (W + W.transpose(0, 2, 1, 3)))


def _lanczos(lib, h, th, L, R, W, prec=0):
    Dl, d, _, Dr = th.shape
    w = W.shape[0]
    t_in, t_out = _dev(th), _dev(np.zeros_like(th))
    dL, dR, dW = _dev(L), _dev(R), _dev(W)
    E = C.c_double()
    nk = C.c_int()
    st = lib.ct_lanczos2(h, prec, _p(t_in), _p(t_out), _p(dL), _p(dR), _p(dW), _p(dW), Dl, d, Dr, w, w, w, 12,
                         1e-10, 0, 0, C.byref(E), C.byref(nk), None, None)
    return st, E.value


@pytest.mark.parametrize("bad", [np.nan, np.inf, -np.inf])
def test_lanczos_nonfinite_start_vector(handle, bad):
    lib, h = handle
    L = _lib()
    th, Le, Re, W = _heff_inputs(1)
    th_bad = th.copy()
    th_bad[2, 1, 0, 3] = bad
    st, _ = _lanczos(lib, h, th_bad, Le, Re, W)
    assert st == L.CT_ERR_NONFINITE
    st, E = _lanczos(lib, h, th, Le, Re, W)   # the handle is still usable
    assert st == L.CT_OK and np.isfinite(E)


@pytest.mark.parametrize("which", ["L", "R", "W"])
def test_lanczos_nonfinite_operator(handle, which):
    """A NaN in an environment or an MPO tensor reaches alpha / beta, which the
    tridiagonal eigensolve refuses."""
    lib, h = handle
    L = _lib()
    th, Le, Re, W = _heff_inputs(2)
    arrs = {"L": Le.copy(), "R": Re.copy(), "W": W.copy()}
    arrs[which].flat[5] = np.nan
    st, _ = _lanczos(lib, h, th, arrs["L"], arrs["R"], arrs["W"])
    assert st == L.CT_ERR_NONFINITE
    st, E = _lanczos(lib, h, th, Le, Re, W)
    assert st == L.CT_OK and np.isfinite(E)


def _split(lib, h, th, chi_max, prec=0):
    Dl, d, _, Dr = th.shape
    k = min(Dl * d, d * Dr)
    dth = _dev(th)
    A = _dev(np.zeros(Dl * d * k))
    B = _dev(np.zeros(k * d * Dr))
    S = _dev(np.zeros(k))
    chi = C.c_int64()
    disc = C.c_double()
    st = lib.ct_svd_split(h, prec, _p(dth), Dl, d, Dr, chi_max, 0.0, 1, _p(A), _p(B), _p(S), C.byref(chi),
                          C.byref(disc))
    return st, S.cpu().numpy()[:chi.value]


@pytest.mark.parametrize("bad", [np.nan, np.inf])
def test_split_nonfinite(handle, bad):
    lib, h = handle
    L = _lib()
    th = np.random.default_rng(3).standard_normal((16, 2, 2, 16))
    th_bad = th.copy()
    th_bad[0, 0, 1, 7] = bad
    st, _ = _split(lib, h, th_bad, 32)
    assert st == L.CT_ERR_NONFINITE
    st, S = _split(lib, h, th, 32)
    assert st == L.CT_OK
    ref = np.linalg.svd(th.reshape(32, 32), compute_uv=False)
    assert np.allclose(S, ref, rtol=1e-12, atol=1e-12 * ref[0])


def test_svd_trunc_nonfinite(handle):
    lib, h = handle
    L = _lib()
    M = np.random.default_rng(4).standard_normal((20, 12))
    M[3, 4] = np.nan
    dM = _dev(M)
    U, S, Vt = _dev(np.zeros(20 * 12)), _dev(np.zeros(12)), _dev(np.zeros(12 * 12))
    chi = C.c_int64()
    st = lib.ct_svd_trunc(h, _p(dM), 20, 12, 12, 0.0, _p(U), _p(S), _p(Vt), C.byref(chi))
    assert st == L.CT_ERR_NONFINITE


@pytest.mark.parametrize("shape", [(16, 16), (150, 150)])
def test_svd_sweep_cap(handle, shape):
    """Sweep cap 1: the one-CTA Jacobi (32 x 32) and the cooperative one (300 x 300)
    stop after one sweep and report CT_ERR_NOCONV; cap 0 restores the default."""
    lib, h = handle
    L = _lib()
    Dl, Dr = shape
    th = np.random.default_rng(5).standard_normal((Dl, 2, 2, Dr))
    L.check(lib.ct_set_svd_max_sweeps(h, 1), "ct_set_svd_max_sweeps")
    try:
        st, _ = _split(lib, h, th, 2 * Dl)
        assert st == L.CT_ERR_NOCONV
    finally:
        L.check(lib.ct_set_svd_max_sweeps(h, 0), "ct_set_svd_max_sweeps")
    st, S = _split(lib, h, th, 2 * Dl)
    assert st == L.CT_OK
    ref = np.linalg.svd(th.reshape(2 * Dl, 2 * Dr), compute_uv=False)
    assert np.allclose(S, ref, rtol=1e-11, atol=1e-12 * ref[0])
    assert lib.ct_set_svd_max_sweeps(h, -1) == L.CT_ERR_INVALID


def test_dmrg_nonfinite_site(ctx):
    """NaN in one MPS site before upload: the sweep driver stops with CT_ERR_NONFINITE
    (the reference would run on and report a NaN energy); a clean run on the same
    handle then matches the oracle's first-sweep energy."""
    import chemtensor_mojo_gb300 as ct
    L = _lib()
    n = 6
    mpo_a = oh.ising_1d(n, J=1.0, h_longitudinal=0.0, g_transverse=1.0)
    sites, _ = orng.create_random_mps_c_compatible(n, 2, 8, 0)
    mps_a = od.right_normalize(sites)
    bad = [s.copy() for s in mps_a]
    bad[3].flat[2] = np.nan
    mpo = ct.mpo_from_arrays(ctx, mpo_a)
    p = ct.DMRGParams(num_sweeps=1, chi_max=8, eps_trunc=0.0, max_krylov_iter=10, krylov_tol=1e-10,
                      energy_tol=0.0, max_rotations=0)
    with pytest.raises(L.CTDMRGError) as err:
        ct.dmrg_two_site(ctx, mpo, ct.mps_from_arrays(ctx, bad), p)
    assert err.value.status == L.CT_ERR_NONFINITE
    E, _ = ct.dmrg_two_site(ctx, mpo, ct.mps_from_arrays(ctx, mps_a), p)
    E_ref, _ = od.dmrg_two_site(mpo_a, mps_a, od.DMRGParams(1, 8, 0.0, 10, 1e-10, 0.0), eig="exact")
    assert abs(E - E_ref) <= 1e-10 * abs(E_ref)
