"""Seeded random MPS, restating src/tests/benchmarks/rng_c_compat.mojo.

PCG32 is O'Neill's published generator (pcg_basic); the seeding, the two-stream
state, Floyd-style ``rand_choice`` advancing and the Box-Muller ``randnf`` follow
the reference's Mojo restatement of ChemTensor's rng.c line by line:

* ``_pcg32_step``           rng_c_compat.mojo:21-30
* ``pcg32_seed``            rng_c_compat.mojo:49-56
* ``RngState.rand_uint64``  rng_c_compat.mojo:69-74
* ``rand_interval``         rng_c_compat.mojo:76-84
* ``rand_choice_advance``   rng_c_compat.mojo:86-96
* ``randnf``                rng_c_compat.mojo:98-108 (float32 arithmetic)
* ``seed_rng_state``        rng_c_compat.mojo:129-149
* ``bond_dims_c_style``     rng_c_compat.mojo:152-171
* ``create_random_mps_c_compatible`` rng_c_compat.mojo:174-231

Test infrastructure only (see oracle/__init__.py).
"""
from __future__ import annotations

import numpy as np

MASK64 = (1 << 64) - 1
MASK32 = (1 << 32) - 1
PCG32_MULT = 6364136223846793005


def _pcg32_step(state: int, inc: int):
    new_state = (state * PCG32_MULT + inc) & MASK64
    xorshifted = (((state >> 18) ^ state) >> 27) & MASK32
    rot = state >> 59
    out = ((xorshifted >> rot) | (xorshifted << ((-rot) & 31))) & MASK32
    return new_state, out


def pcg32_seed(initstate: int, initseq: int):
    inc = ((initseq << 1) | 1) & MASK64
    state, _ = _pcg32_step(0, inc)
    state = (state + initstate) & MASK64
    state, _ = _pcg32_step(state, inc)
    return [state, inc]


class RngState:
    """Two PCG32 streams; ``randnf`` only draws from the first one."""

    def __init__(self, gen0, gen1):
        self.gen0 = list(gen0)
        self.gen1 = list(gen1)

    def rand_uint32(self) -> int:
        self.gen0[0], v = _pcg32_step(self.gen0[0], self.gen0[1])
        return v

    def rand_uint64(self) -> int:
        self.gen0[0], v0 = _pcg32_step(self.gen0[0], self.gen0[1])
        self.gen1[0], v1 = _pcg32_step(self.gen1[0], self.gen1[1])
        return (v0 << 32) | v1

    def rand_interval(self, bound: int) -> int:
        threshold = ((~bound + 1) & MASK64) % bound
        while True:
            r = self.rand_uint64()
            if r >= threshold:
                return r % bound

    def rand_choice_advance(self, bound: int, num_samples: int) -> None:
        for i in range(num_samples):
            self.rand_interval(bound - num_samples + 1 + i)

    def randnf(self) -> np.float32:
        inv_2p32 = np.float32(2.32830644e-10)
        u1 = np.float32(self.rand_uint32()) * inv_2p32
        u2 = np.float32(self.rand_uint32()) * inv_2p32
        if u1 == 0.0:
            u1 = np.float32(1.0)
        r = np.sqrt(np.float32(-2.0) * np.log(np.float32(u1)))
        g = r * np.sin(np.float32(6.2831853071795864769) * np.float32(u2))
        return np.float32(g)


def seed_rng_state(seed: int) -> RngState:
    mult = 6364136223846793005
    inc = 1442695040888963407
    g = pcg32_seed(seed, (mult * seed + inc) & MASK64)
    vals = []
    for _ in range(8):
        g[0], v = _pcg32_step(g[0], g[1])
        vals.append(v)
    seed1 = (vals[0] << 32) | vals[1]
    seed2 = (vals[2] << 32) | vals[3]
    seq1 = (vals[4] << 32) | vals[5]
    seq2 = (vals[6] << 32) | vals[7]
    mask = 0x7FFF_FFFF_FFFF_FFFF
    if (seq1 & mask) == (seq2 & mask):
        seq2 = (~seq2) & MASK64
    return RngState(pcg32_seed(seed1, seq1), pcg32_seed(seed2, seq2))


def bond_dims_c_style(nsites: int, d: int, chi_max: int):
    """min(d^k, d^(L-k), chi_max) with 1 at both ends (rng_c_compat.mojo:152-171)."""
    b = [0] * (nsites + 1)
    b[0] = 1
    b[nsites] = 1
    mid = (nsites + 1) // 2
    for l in range(1, mid):
        b[l] = min(b[l - 1] * d, chi_max)
    for l in range(nsites - 1, mid - 1, -1):
        b[l] = min(b[l + 1] * d, chi_max)
    return b


def create_random_mps_c_compatible(nsites: int, d: int, chi_max: int, seed: int):
    """List of float32-valued site tensors [Dl, d, Dr], entries N(0,1)/sqrt(nelem).

    Returned as float64 arrays holding the float32 values (the reference builds
    them in float32, rng_c_compat.mojo:216-230).
    """
    rng = seed_rng_state(seed)
    dims = [0] * (nsites + 1)
    dims[0] = 1
    dims[nsites] = 1
    mid = (nsites + 1) // 2
    for l in range(1, mid):
        full = dims[l - 1] * d
        dims[l] = min(full, chi_max)
        if full > chi_max:
            rng.rand_choice_advance(full, chi_max)
    for l in range(nsites - 1, mid - 1, -1):
        full = dims[l + 1] * d
        dims[l] = min(full, chi_max)
        if full > chi_max:
            rng.rand_choice_advance(full, chi_max)
    sites = []
    for i in range(nsites):
        dl, dr = dims[i], dims[i + 1]
        nelem = dl * d * dr
        scale = np.float32(1.0 / np.sqrt(float(nelem)))
        data = np.empty(nelem, dtype=np.float32)
        for k in range(nelem):
            data[k] = rng.randnf() * scale
        sites.append(data.astype(np.float64).reshape(dl, d, dr))
    return sites, dims


def gaussian_mps(nsites: int, d: int, chi_max: int, seed: int):
    """Fast seeded Gaussian MPS with the same bond dimensions (large chains).

    The pure-Python PCG32 stream is too slow for chi ~ 1000 tensors; this draws
    N(0,1) entries from NumPy's PCG64 with the same seed and the same
    1/sqrt(nelem) scaling.  Used for the large synthetic workloads only.
    """
    dims = bond_dims_c_style(nsites, d, chi_max)
    g = np.random.Generator(np.random.PCG64(seed))
    sites = []
    for i in range(nsites):
        dl, dr = dims[i], dims[i + 1]
        a = g.standard_normal((dl, d, dr)) / np.sqrt(dl * d * dr)
        sites.append(a)
    return sites, dims
