"""ctypes binding of libctdmrg.so (include/ctdmrg.h).

The library is the product: there is no CPU fallback.  Loading fails loudly
when the shared object is missing, and every entry point raises
``CTDMRGError`` on a non-zero status.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libctdmrg.so"

CT_OK = 0
CT_ERR_INVALID = -1
CT_ERR_CUDA = -2
CT_ERR_OOM = -3
CT_ERR_NOCONV = -4
CT_ERR_ZERO_NORM = -5
CT_ERR_SHAPE = -6
CT_ERR_UNSUPPORTED = -7
CT_ERR_NONFINITE = -8
CT_ERR_EMPTY = -9
CT_ERR_TOO_LARGE = -10
NOALLOC_SCRATCH_DOUBLES = 1 << 21

CT_PREC_FP64 = 0
CT_PREC_TF32X3 = 1
CT_PREC_FP64_TC = 2
PRECISIONS = {"fp64": CT_PREC_FP64, "tf32x3": CT_PREC_TF32X3, "fp64_tc": CT_PREC_FP64_TC}


class CTDMRGError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        super().__init__(f"{where}: status {status} ({error_string(status)}){': ' + detail if detail else ''}")


class ct_dmrg_params(C.Structure):
    _fields_ = [("num_sweeps", C.c_int), ("chi_max", C.c_int), ("eps_trunc", C.c_double),
                ("max_krylov_iter", C.c_int), ("krylov_tol", C.c_double), ("energy_tol", C.c_double),
                ("two_site", C.c_int), ("verbose", C.c_int), ("prec", C.c_int), ("max_rotations", C.c_int),
                ("reorth", C.c_int), ("final_rayleigh", C.c_int), ("keep_bases", C.c_int),
                ("split_power_steps", C.c_int), ("cold_power_steps", C.c_int)]


class ct_dmrg_stats(C.Structure):
    _fields_ = [("seconds_total", C.c_double), ("seconds_lanczos", C.c_double), ("seconds_svd", C.c_double),
                ("seconds_env", C.c_double), ("heff_flops", C.c_double), ("env_flops", C.c_double),
                ("heff_applies", C.c_int64), ("local_updates", C.c_int64), ("max_discarded", C.c_double),
                ("energy_rayleigh", C.c_double), ("subspace_splits", C.c_int64), ("exact_splits", C.c_int64),
                ("seconds_subspace", C.c_double), ("cold_splits", C.c_int64),
                ("completed_rows", C.c_int64), ("seconds_rayleigh", C.c_double),
                ("stale_retries", C.c_int64), ("fp64_handovers", C.c_int64)]


P = C.c_void_p
I64 = C.c_int64
I32 = C.c_int
D = C.c_double
PP = C.POINTER(C.c_void_p)

# name -> (argtypes); every function returns int except the string ones
SIGNATURES = {
    "ct_create": [I32, P, C.POINTER(P)],
    "ct_destroy": [P],
    "ct_set_stream": [P, P],
    "ct_synchronize": [P],
    "ct_get_status": [P, C.POINTER(I32)],
    "ct_version": [],
    "ct_workspace_bytes": [P, C.POINTER(I64)],
    "ct_set_workspace_limit": [P, I64],
    "ct_set_svd_max_sweeps": [P, I32],
    "ct_svd_sweeps": [P, C.POINTER(I32), C.POINTER(I64)],
    "ct_gemm": [P, I32, I32, I32, I64, I64, I64, D, P, I64, P, I64, D, P, I64],
    "ct_permute": [P, P, P, I32, C.POINTER(I64), C.POINTER(C.c_int32)],
    "ct_vec_dot": [P, I64, P, P, C.POINTER(D)],
    "ct_vec_norm_sq": [P, I64, P, C.POINTER(D)],
    "ct_vec_axpy": [P, I64, D, P, P],
    "ct_vec_scale": [P, I64, D, P],
    "ct_env_identity": [P, P, I64, I64],
    "ct_theta2": [P, I32, P, P, P, I64, I64, I64, I64],
    "ct_heff2_apply": [P, I32, P, P, P, P, P, P, I64, I64, I64, I64, I64, I64],
    "ct_env_left": [P, I32, P, P, P, P, I64, I64, I64, I64, I64],
    "ct_env_right": [P, I32, P, P, P, P, I64, I64, I64, I64, I64],
    "ct_lanczos2": [P, I32, P, P, P, P, P, P, I64, I64, I64, I64, I64, I64, I32, D, I32, I32,
                    C.POINTER(D), C.POINTER(I32), C.POINTER(D), C.POINTER(D)],
    "ct_svd_trunc": [P, P, I64, I64, I64, D, P, P, P, C.POINTER(I64)],
    "ct_svd_split": [P, I32, P, I64, I64, I64, I64, D, I32, P, P, P, C.POINTER(I64), C.POINTER(D)],
    "ct_dmrg_two_site": [P, C.POINTER(ct_dmrg_params), I32, I32, C.POINTER(I64), PP, C.POINTER(I64), PP,
                         C.POINTER(I64), C.POINTER(D), C.POINTER(D), C.POINTER(I32), C.POINTER(D),
                         C.POINTER(ct_dmrg_stats)],
    "ct_mps_right_normalize": [P, I32, I32, C.POINTER(I64), PP],
    "ct_mps_expectation": [P, I32, I32, I32, C.POINTER(I64), PP, C.POINTER(I64), PP, C.POINTER(D), C.POINTER(D)],
    "ct_env_left2": [P, I32, P, P, P, P, P, I64, I64, I64, I64, I64, I64, I64],
    "ct_mps_expectation2": [P, I32, I32, I32, C.POINTER(I64), PP, C.POINTER(I64), PP, C.POINTER(I64), PP,
                            C.POINTER(D)],
    "ct_mpo_compose_site": [P, P, P, P, I64, I64, I64, I64, I64, I64, I64],
    "ct_apply_mpo_site": [P, P, P, P, I64, I64, I64, I64, I64, I64],
    "ct_qr": [P, P, I64, I64, P, P, C.POINTER(I32)],
    "ct_random_mps_host": [I32, I32, I32, C.c_uint64, C.POINTER(I64), PP],
    "ct_rng_randnf_host": [C.c_uint64, I64, C.POINTER(C.c_float)],
    "ct_tc_gemm_time": [P, I64, I64, I64, I32, C.POINTER(D)],
    "ct_tc_gemm_plan": [I64, I64, I64, I32, C.POINTER(I64)],
    "ct_svd_split_warm": [P, P, I64, I64, I64, I64, I32, P, I32, P, P, P, C.POINTER(I32), C.POINTER(D),
                          C.POINTER(D)],
    "ct_kernel_timing": [P, I32],
    "ct_kernel_timing_read": [P, C.POINTER(I64), C.POINTER(D), C.POINTER(D)],
    "ct_kernel_timing_read_class": [P, I32, C.POINTER(I64), C.POINTER(D), C.POINTER(D)],
    "ct_heff2_apply_noalloc": [P, P, P, P, P, P, P, I64, I64, I64, I64, I64, I64],
    "ct_energy_grad": [P, I32, I32, I32, C.POINTER(I64), PP, C.POINTER(I64), PP, PP, I32, C.POINTER(D)],
}
STRING_FUNCS = {"ct_error_string": [I32], "ct_last_error": [P]}
INT64_FUNCS = {"ct_launch_count": []}

_lib = None
_lock = threading.Lock()


def load() -> C.CDLL:
    """Load libctdmrg.so; raises if it has not been built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = Path(os.environ.get("CTDMRG_LIB", LIB_PATH))
        if not path.exists():
            raise RuntimeError(
                f"libctdmrg.so not found at {path}; build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)")
        lib = C.CDLL(str(path))
        for name, args in SIGNATURES.items():
            f = getattr(lib, name)
            f.argtypes = args
            f.restype = C.c_int
        for name, args in INT64_FUNCS.items():
            f = getattr(lib, name)
            f.argtypes = args
            f.restype = C.c_int64
        for name, args in STRING_FUNCS.items():
            f = getattr(lib, name)
            f.argtypes = args
            f.restype = C.c_char_p
        _lib = lib
        return lib


def launch_count() -> int:
    return int(load().ct_launch_count())


def error_string(status: int) -> str:
    try:
        return load().ct_error_string(status).decode()
    except Exception:  # pragma: no cover - library missing
        return "?"


def check(status: int, where: str, handle=None) -> None:
    if status != CT_OK:
        detail = ""
        if handle is not None:
            try:
                detail = load().ct_last_error(handle).decode()
            except Exception:  # pragma: no cover
                detail = ""
        raise CTDMRGError(status, where, detail)


def ptr_array(ptrs):
    arr = (C.c_void_p * len(ptrs))(*[C.c_void_p(int(p)) for p in ptrs])
    return C.cast(arr, PP), arr


def i64_array(vals):
    arr = (C.c_int64 * len(vals))(*[int(v) for v in vals])
    return arr
