"""Host logic of the TF32x3 GEMM launcher, through ct_tc_gemm_plan (no GPU): the tile width
and orientation it picks for the H_eff products, the tuning switches, and the hybrid
schedule -- whole waves of tiles, then the last partial wave's k-blocks shared out over the
SMs -- checked for exact coverage by a restatement of the kernel's work walk (TcCursor in
csrc/ct_tc.cu): every (tile, k-block) exactly once, each split tile's pieces numbered
0..n-1 with one n, and n never above the plan's slot count."""
import ctypes as C

import numpy as np
import pytest

SWITCHES = ("CTDMRG_TC_BN", "CTDMRG_TC_TRANS", "CTDMRG_TC_HYBRID", "CTDMRG_TC_KCHUNK", "CTDMRG_TC_STREAM_K",
            "CTDMRG_TC_TILE_PER_CTA")


@pytest.fixture(scope="module")
def lib():
    from chemtensor_mojo_gb300 import _lib
    if not _lib.LIB_PATH.exists():
        from chemtensor_mojo_gb300 import build
        build.build()
    return _lib.load()


@pytest.fixture(autouse=True)
def defaults(monkeypatch):
    for v in SWITCHES:
        monkeypatch.delenv(v, raising=False)


def plan(lib, m, n, k, sms=152):
    out = (C.c_int64 * 8)()
    assert lib.ct_tc_gemm_plan(m, n, k, sms, out) == 0
    keys = ("bn", "trans", "tiles", "tiles_dp", "gsk", "units", "maxp", "nkb")
    return dict(zip(keys, list(out)))


def walk(p, sms):
    """(cta, tile, kb0, kb1, piece, pieces) in each CTA's processing order, as TcCursor::next."""
    tiles_dp, gsk, units, nkb = p["tiles_dp"], p["gsk"], p["units"], p["nkb"]
    grid = min(p["tiles"], sms) if gsk == 0 else (sms if tiles_dp > 0 else gsk)
    for c in range(grid):
        for t in range(c, tiles_dp, grid):
            yield c, t, 0, nkb, 0, 1
        if c >= gsk:
            continue
        u, ue = c * units // gsk, (c + 1) * units // gsk
        while u < ue:
            st = u // nkb
            k0 = u - st * nkb
            k1 = min(nkb, k0 + (ue - u))
            base = st * nkb
            cf = ((base + 1) * gsk - 1) // units
            cl = ((base + nkb) * gsk - 1) // units
            yield c, tiles_dp + st, k0, k1, c - cf, cl - cf + 1
            u += k1 - k0


def check_cover(p, sms):
    seen = np.zeros((p["tiles"], p["nkb"]), dtype=np.int32)
    pieces = {}
    for _, t, k0, k1, piece, n in walk(p, sms):
        assert 0 <= t < p["tiles"] and 0 <= k0 < k1 <= p["nkb"] and 0 <= piece < n <= p["maxp"]
        seen[t, k0:k1] += 1
        pieces.setdefault(t, {})[piece] = n
    assert np.all(seen == 1)
    for t, d in pieces.items():
        ns = set(d.values())
        assert len(ns) == 1 and sorted(d) == list(range(ns.pop())), (t, d)


def test_heff_products_at_chi_1024(lib):
    # GEMM 1 (wL Dl x d^2 Dr x Dl): 760 tiles of 128 x 224 fill 5 waves of 152 exactly
    p = plan(lib, 5120, 4096, 1024)
    assert (p["bn"], p["trans"], p["tiles"], p["gsk"]) == (224, 0, 760, 0)
    # GEMM 4 (Dl d^2 x Dr x wR Dr): its transpose 1024 x 4096 is one wave of 152 tiles of 128 x 224
    p = plan(lib, 4096, 1024, 5120)
    assert (p["bn"], p["trans"], p["tiles"], p["gsk"]) == (224, 1, 152, 0)
    # 8192 x 2048 x 8192: 512 tiles of 128 x 256, the last partial wave shared out
    p = plan(lib, 8192, 2048, 8192)
    assert p["bn"] == 256 and p["tiles"] == 512 and p["tiles_dp"] == 456 and p["gsk"] == 152
    check_cover(p, 152)


def test_switches(lib, monkeypatch):
    monkeypatch.setenv("CTDMRG_TC_TRANS", "0")
    assert plan(lib, 4096, 1024, 5120)["trans"] == 0
    monkeypatch.setenv("CTDMRG_TC_TRANS", "1")
    assert plan(lib, 5120, 4096, 1024)["trans"] == 1
    monkeypatch.delenv("CTDMRG_TC_TRANS")
    monkeypatch.setenv("CTDMRG_TC_HYBRID", "0")
    p = plan(lib, 8192, 2048, 8192)
    assert p["gsk"] == 0 and p["tiles_dp"] == p["tiles"]
    monkeypatch.delenv("CTDMRG_TC_HYBRID")
    for bn in ("128", "192", "224", "256"):
        monkeypatch.setenv("CTDMRG_TC_BN", bn)
        p = plan(lib, 2500, 1700, 999)
        assert p["bn"] == int(bn) and p["trans"] == 0
    monkeypatch.delenv("CTDMRG_TC_BN")
    # the single-accumulator kernel has no 192 / 224 tiles, no transposed form, no stream-K part
    monkeypatch.setenv("CTDMRG_TC_KCHUNK", "0")
    for shape in ((5120, 4096, 1024), (4096, 1024, 5120), (8192, 2048, 8192)):
        p = plan(lib, *shape)
        assert p["bn"] in (128, 256) and p["trans"] == 0 and p["gsk"] == 0


@pytest.mark.parametrize("sms", [152, 148, 132])
def test_hybrid_schedule_covers_every_k_block(lib, sms):
    rng = np.random.default_rng(sms)
    with_sk = 0
    for _ in range(300):
        m, n = int(rng.integers(1, 12000)), int(rng.integers(1, 9000))
        k = int(rng.integers(1, 12000))
        p = plan(lib, m, n, k, sms)
        assert p["bn"] in (128, 192, 224, 256)
        assert p["nkb"] == -(-k // 32)
        rows, cols = (n, m) if p["trans"] else (m, n)
        assert p["tiles"] == -(-rows // 128) * -(-cols // p["bn"])
        if p["gsk"]:
            with_sk += 1
            # only next to whole waves, each CTA's share at least 8 k-blocks
            assert p["tiles_dp"] > 0 and p["tiles_dp"] % sms == 0 and p["tiles"] - p["tiles_dp"] < sms
            assert p["units"] == (p["tiles"] - p["tiles_dp"]) * p["nkb"]
            assert p["units"] // p["gsk"] >= 8
        check_cover(p, sms)
    assert with_sk > 20
