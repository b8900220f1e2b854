"""CPU-only checks of the boundary and the host logic (no GPU compute calls)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from oracle import hamiltonians as oh
from oracle import rng as orng

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def lib():
    from chemtensor_mojo_gb300 import _lib
    if not _lib.LIB_PATH.exists():
        from chemtensor_mojo_gb300 import build
        build.build()
    return _lib.load()


def header_symbols():
    text = (ROOT / "include" / "ctdmrg.h").read_text()
    return re.findall(r"^CT_API\s+(?:const\s+char\s*\*|int64_t|int)\s+(ct_\w+)\s*\(", text, flags=re.M)


def test_library_exports_every_header_symbol(lib):
    syms = header_symbols()
    assert len(syms) >= 25
    for s in syms:
        assert hasattr(lib, s), s


def test_bindings_cover_header(lib):
    from chemtensor_mojo_gb300 import _lib
    bound = set(_lib.SIGNATURES) | set(_lib.STRING_FUNCS) | set(_lib.INT64_FUNCS)
    assert set(header_symbols()) == bound


def test_version_and_error_strings(lib):
    assert lib.ct_version() == 1
    assert lib.ct_error_string(0) == b"ok"
    assert lib.ct_error_string(-5) == b"initial vector has zero norm"
    assert lib.ct_error_string(-9) == b"truncation kept no singular values"


def test_null_handle_is_rejected(lib):
    assert lib.ct_destroy(None) == -1
    assert lib.ct_synchronize(None) == -1
    assert lib.ct_vec_scale(None, 4, C.c_double(1.0), None) == -1


def test_rng_matches_oracle(lib):
    n = 512
    out = (C.c_float * n)()
    assert lib.ct_rng_randnf_host(C.c_uint64(0), n, out) == 0
    st = orng.seed_rng_state(0)
    ref = np.array([st.randnf() for _ in range(n)], dtype=np.float32)
    got = np.frombuffer(out, dtype=np.float32)
    # float32 Box-Muller: libm logf/sinf vs NumPy's float32 loops may differ by an ulp
    np.testing.assert_allclose(got, ref, rtol=2e-6, atol=2e-7)


@pytest.mark.parametrize("L,d,chi,seed", [(12, 2, 32, 0), (9, 3, 4, 7), (6, 4, 8, 42)])
def test_random_mps_matches_oracle(lib, L, d, chi, seed):
    from chemtensor_mojo_gb300.mps_state import random_mps_c_compatible_arrays
    arrays, dims = random_mps_c_compatible_arrays(L, d, chi, seed)
    ref, ref_dims = orng.create_random_mps_c_compatible(L, d, chi, seed)
    assert dims == ref_dims
    for a, b in zip(arrays, ref):
        np.testing.assert_allclose(a, b, rtol=4e-6, atol=1e-7)


def test_mpo_builders_match_oracle():
    from chemtensor_mojo_gb300 import hamiltonians as H
    pairs = [
        (H.ising_1d_arrays(6, 1.0, 0.3, 0.7), oh.ising_1d(6, 1.0, 0.3, 0.7)),
        (H.heisenberg_xxx_arrays(5, 0.8), oh.heisenberg_xxx(5, 0.8)),
        (H.heisenberg_xxz_arrays(5, 1.0, 0.5, 0.2), oh.heisenberg_xxz(5, 1.0, 0.5, 0.2)),
        (H.bose_hubbard_arrays(4, 4, 1.0, 4.0, 0.3), oh.bose_hubbard(4, 4, 1.0, 4.0, 0.3)),
        (H.fermi_hubbard_arrays(5, 1.0, 8.0, 0.1), oh.fermi_hubbard(5, 1.0, 8.0, 0.1)),
        (H.ising_1d_arrays(2, 1.0, 0.0, 0.0), oh.ising_1d(2, 1.0, 0.0, 0.0)),
    ]
    for mine, ref in pairs:
        assert len(mine) == len(ref)
        for a, b in zip(mine, ref):
            assert a.shape == b.shape
            assert np.array_equal(a, b)


def test_bond_capacities():
    from chemtensor_mojo_gb300.dmrg import bond_capacities
    assert bond_capacities([1] * 9, 2, 1000) == [1, 2, 4, 8, 16, 8, 4, 2, 1]
    assert bond_capacities([1] * 9, 2, 5) == [1, 2, 4, 5, 5, 5, 4, 2, 1]
    dims = orng.bond_dims_c_style(12, 2, 32)
    assert bond_capacities(dims, 2, 32) == dims


def _c_struct_fields(name):
    """(type, field) pairs of a typedef'd struct in ctdmrg.h, in declaration order."""
    text = (ROOT / "include" / "ctdmrg.h").read_text()
    m = re.search(r"typedef\s+struct\s*(?:\w+\s*)?\{([^{}]*)\}\s*" + name + r"\s*;", text)
    assert m, name
    body = re.sub(r"/\*.*?\*/", "", m.group(1), flags=re.S)
    return [(t, f) for t, f in re.findall(r"(int64_t|int|double)\s+(\w+)\s*;", body)]


@pytest.mark.parametrize("cname,pyname", [("ct_dmrg_params", "ct_dmrg_params"), ("ct_dmrg_stats", "ct_dmrg_stats")])
def test_ctypes_structs_match_header(cname, pyname):
    """The ctypes mirrors of the parameter and statistics structs have the header's fields, in
    order and with the same C types (an ABI drift here would corrupt every sweep call)."""
    from chemtensor_mojo_gb300 import _lib
    ctype = {"int": C.c_int, "int64_t": C.c_int64, "double": C.c_double}
    cfields = _c_struct_fields(cname)
    pyfields = getattr(_lib, pyname)._fields_
    assert [f for _, f in cfields] == [f for f, _ in pyfields]
    for (t, f), (pf, pt) in zip(cfields, pyfields):
        assert C.sizeof(ctype[t]) == C.sizeof(pt) and ctype[t]._type_ == pt._type_, f


def test_python_stats_mirror_the_c_struct():
    """Every field of ct_dmrg_stats reaches DMRGStats."""
    from chemtensor_mojo_gb300 import _lib
    from chemtensor_mojo_gb300.dmrg import DMRGStats
    names = {f for f, _ in _lib.ct_dmrg_stats._fields_}
    assert names <= set(DMRGStats().__dict__)


def test_flop_counts_match_oracle():
    import bench
    from oracle import dmrg as od
    for chi_l, chi_r in ((1024, 1024), (512, 1024), (64, 16)):
        assert bench.heff_flops(chi_l, chi_r) == pytest.approx(od.heff_flops(chi_l, chi_r, 5, 2))
    # the centre-bond apply of the benchmark: 86.7 GFLOP
    assert bench.heff_flops(1024, 1024) == pytest.approx(86.7e9, rel=2e-3)
