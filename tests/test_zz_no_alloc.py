"""The allocation-free H_eff apply, ct_heff2_apply_noalloc, through the C ABI.

It serves callers that cannot let a library allocate device memory (for
example a Mojo/MAX host whose allocator owns every buffer): its scratch is a
static device array.  Two calls in a row, with different shapes, must agree
with the allocating entry point ct_heff2_apply on the same inputs to the
FP64 tolerance of the other contraction tests (1e-12 relative); oversized
problems are refused with CT_ERR_TOO_LARGE.  The first shape is one whose
last GEMM splits K over the SMs, the step that used to grow a handle-owned
buffer: fifty calls on it must leave the device's free memory where it was.
This file sorts last so that a failure here stops a -x run only after every
other test has run.
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _inputs(seed, Dl, d, Dr, wL, wM, wR):
    rng = np.random.default_rng(seed)
    return [_dev(x) for x in (rng.standard_normal((Dl, d, d, Dr)), rng.standard_normal((wL, Dl, Dl)),
                              rng.standard_normal((wR, Dr, Dr)), rng.standard_normal((wL, d, d, wM)),
                              rng.standard_normal((wM, d, d, wR)))]


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def test_noalloc_heff_matches_allocating_entry_point():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from chemtensor_mojo_gb300 import _lib
    lib = _lib.load()
    torch.cuda.set_device(0)
    h = C.c_void_p()
    _lib.check(lib.ct_create(0, None, C.byref(h)), "ct_create")
    try:
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        for seed, dims in ((1, (24, 2, 40, 5, 5, 5)), (2, (33, 4, 17, 4, 6, 3))):
            Dl, d, Dr, wL, wM, wR = dims
            th, L, R, W1, W2 = _inputs(seed, *dims)
            ref = torch.empty(Dl * d * d * Dr, dtype=torch.float64, device="cuda")
            out = torch.full_like(ref, float("nan"))
            dims_c = [C.c_int64(x) for x in dims]
            _lib.check(lib.ct_heff2_apply(h, 0, _ptr(th), _ptr(L), _ptr(R), _ptr(W1), _ptr(W2), _ptr(ref), *dims_c),
                       "ct_heff2_apply", h)
            lib.ct_synchronize(h)
            _lib.check(lib.ct_heff2_apply_noalloc(stream, _ptr(th), _ptr(L), _ptr(R), _ptr(W1), _ptr(W2), _ptr(out),
                                                  *dims_c), "ct_heff2_apply_noalloc")
            torch.cuda.synchronize()
            r, o = ref.cpu().numpy(), out.cpu().numpy()
            assert np.all(np.isfinite(o))
            assert np.linalg.norm(o - r) <= 1e-12 * np.linalg.norm(r)
        # no allocation: (24,2,40,5,5,5) makes the last GEMM M=96, N=40, K=200, six
        # 32x32 tiles, so K is split six ways; its partial sums must come from the
        # static array.  A cudaMalloc per call would lower the free memory.
        dims = (24, 2, 40, 5, 5, 5)
        th, L, R, W1, W2 = _inputs(1, *dims)
        out = torch.empty(24 * 4 * 40, dtype=torch.float64, device="cuda")
        args = [_ptr(t) for t in (th, L, R, W1, W2, out)] + [C.c_int64(x) for x in dims]
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        for _ in range(50):
            _lib.check(lib.ct_heff2_apply_noalloc(stream, *args), "ct_heff2_apply_noalloc")
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        assert free1 >= free0 - (1 << 20), f"device free memory fell by {free0 - free1} bytes over 50 calls"
        # a size past the limit: refused before any work
        big = (256, 2, 256, 5, 5, 5)
        th, L, R, W1, W2 = _inputs(3, *big)
        out = torch.empty(256 * 4 * 256, dtype=torch.float64, device="cuda")
        st = lib.ct_heff2_apply_noalloc(stream, _ptr(th), _ptr(L), _ptr(R), _ptr(W1), _ptr(W2), _ptr(out),
                                        *[C.c_int64(x) for x in big])
        assert st == _lib.CT_ERR_TOO_LARGE
    finally:
        lib.ct_destroy(h)
