// Mixed-precision form: TF32x3 contractions on the sm_103a tensor cores.
//
// GEMM: C[M,N] = sum_k A[m,k] B[n,k] with both operands K-major, each split
// into two TF32 planes (x = hi + lo, both exactly representable in TF32) so
// that hi*hi + hi*lo + lo*hi accumulated in FP32 recovers ~FP32 accuracy.
//   * one CTA per 128 x BN output tile, 6 warps:
//       warp 0      TMA producer (cp.async.bulk.tensor, 128B swizzle)
//       warp 1      TMEM allocator + single-thread tcgen05.mma issuer
//       warps 2..5  epilogue (tcgen05.ld 32x32b, one TMEM lane quadrant each)
//   * STAGES-deep smem ring guarded by full/empty mbarriers; MMAs release a
//     stage through tcgen05.commit; the accumulator lives in TMEM.
//   * every mbarrier wait is bounded by %globaltimer (2 s); a timeout sets the
//     device status word and the CTA falls through to TMEM release and exit.
//
// Contraction chains (see ct_ops.cu for the FP64 form) are the same, with the
// permutes folded into the operand packers (FP64 -> split TF32, K-major,
// K padded to 32) and into the GEMM epilogue's row mapping.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <stdlib.h>

#include <algorithm>
#include <new>

#include "ct_ops.cuh"
#include "ct_tc_ptx.cuh"

namespace {

constexpr int TC_BM = 128;
constexpr int TC_BK = 32;             // fp32 elements per 128-byte swizzle row
constexpr int TC_THREADS = 192;

// round-to-nearest-even to TF32 (10 explicit mantissa bits), kept in an fp32 container
__device__ __forceinline__ float tf32_rne(float x) {
    uint32_t u = __float_as_uint(x);
    if ((u & 0x7F800000u) == 0x7F800000u) return x;   // inf / nan unchanged
    u += 0xFFFu + ((u >> 13) & 1u);
    u &= 0xFFFFE000u;
    return __uint_as_float(u);
}

// x = hi + lo with both halves TF32-representable.  All in FP32: x - hi is
// exact in FP32, and lo keeps 11 significant bits, so rounding an FP64 value to
// FP32 first loses nothing that the pair could hold.  (FP64 arithmetic issues
// at a small fraction of the FP32 rate on this part; the packers stay clear
// of it apart from the one conversion.)
__device__ __forceinline__ void split_tf32(float x, float& hi, float& lo) {
    hi = tf32_rne(x);
    lo = tf32_rne(x - hi);
}

// ---------------------------------------------------------------------------
// GEMM kernel
// ---------------------------------------------------------------------------
struct TcEpi {
    void* C;
    int out_fp64;        // 1: double, 0: float
    int64_t M0;          // row m -> (m / M0) * sCm1 + (m % M0) * sCm0
    int64_t sCm1, sCm0;
    double alpha, beta;  // C = alpha * acc + beta * C
    int vec;             // set by the launcher: C and both row strides 16-byte aligned
    // set by the launcher (chunked kernel only): the kernel computes the transposed
    // product, its element (i, j) is the caller's C(j, i), stored at j * sCm0 + i
    // (single-level rows: M0 >= the caller's M)
    int trans;
};

template <int BN, int STAGES>
struct TcSmem {
    static constexpr int A_BYTES = TC_BM * TC_BK * 4;       // 16 KB per plane
    static constexpr int B_BYTES = BN * TC_BK * 4;
    static constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;
    static constexpr int TILE_BYTES = STAGES * STAGE_BYTES;
    static constexpr int TOTAL = TILE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
};

template <int BN, int STAGES>
__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap tmAh, const __grid_constant__ CUtensorMap tmAl,
                   const __grid_constant__ CUtensorMap tmBh, const __grid_constant__ CUtensorMap tmBl, int M, int N,
                   int Kpad, TcEpi epi, const int* skip, int* status) {
    using L = TcSmem<BN, STAGES>;
    if (ct_skip(skip)) return;
    extern __shared__ uint8_t tc_smem_raw[];
    // 128-byte swizzled tiles need 1024-byte alignment in the shared window
    uint8_t* smem = tc_smem_raw + ((1024u - (smem_u32(tc_smem_raw) & 1023u)) & 1023u);
    uint64_t* full = (uint64_t*)(smem + L::TILE_BYTES);
    uint64_t* empty = full + STAGES;
    uint64_t* done = empty + STAGES;
    uint32_t* tmem_slot = (uint32_t*)(done + 1);
    volatile int* abort_flag = (volatile int*)(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.y * TC_BM, n0 = blockIdx.x * BN;
    const int nkb = Kpad / TC_BK;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"((uint32_t)BN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            for (int kb = 0; kb < nkb; ++kb) {
                const int s = kb % STAGES;
                const uint32_t ph = (uint32_t)(kb / STAGES) & 1u;
                if (kb >= STAGES && !mbar_wait(&empty[s], ph ^ 1u, abort_flag)) {
                    *abort_flag = 1;
                    ct_set_status(status, CT_ERR_CUDA);
                    break;
                }
                uint8_t* st = smem + s * L::STAGE_BYTES;
                mbar_expect_tx(&full[s], L::STAGE_BYTES);
                const int x = kb * TC_BK;
                tma_load_2d(st, &tmAh, x, m0, &full[s]);
                tma_load_2d(st + L::A_BYTES, &tmAl, x, m0, &full[s]);
                tma_load_2d(st + 2 * L::A_BYTES, &tmBh, x, n0, &full[s]);
                tma_load_2d(st + 2 * L::A_BYTES + L::B_BYTES, &tmBl, x, n0, &full[s]);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = idesc_tf32(TC_BM, BN);
            bool ok = true;
            for (int kb = 0; kb < nkb; ++kb) {
                const int s = kb % STAGES;
                const uint32_t ph = (uint32_t)(kb / STAGES) & 1u;
                if (!mbar_wait(&full[s], ph, abort_flag)) {
                    *abort_flag = 1;
                    ct_set_status(status, CT_ERR_CUDA);
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t a_hi = smem_u32(smem + s * L::STAGE_BYTES);
                const uint32_t a_lo = a_hi + L::A_BYTES;
                const uint32_t b_hi = a_hi + 2 * L::A_BYTES;
                const uint32_t b_lo = b_hi + L::B_BYTES;
#pragma unroll
                for (int kk = 0; kk < TC_BK / 8; ++kk) {
                    const uint32_t off = kk * 32;   // 8 tf32 = 32 bytes of K per MMA
                    const uint32_t acc0 = (kb > 0 || kk > 0) ? 1u : 0u;
                    mma_tf32(tmem, sw128_desc(a_lo + off), sw128_desc(b_hi + off), idesc, acc0);
                    mma_tf32(tmem, sw128_desc(a_hi + off), sw128_desc(b_lo + off), idesc, 1u);
                    mma_tf32(tmem, sw128_desc(a_hi + off), sw128_desc(b_hi + off), idesc, 1u);
                }
                mma_commit(&empty[s]);
            }
            if (ok) mma_commit(done);
        }
    } else {
        // epilogue warps 2..5 -> TMEM lane quadrants 2,3,0,1
        const int q = warp & 3;
        const bool ok = mbar_wait(done, 0, abort_flag);
        if (!ok) {
            *abort_flag = 1;
            ct_set_status(status, CT_ERR_CUDA);
        }
        __syncwarp();
        tc_fence_after();
        if (ok) {
            const int row = q * 32 + lane;
            const int64_t m = (int64_t)m0 + row;
            const bool mvalid = m < M;
            int64_t rbase = 0;
            if (mvalid) rbase = (m / epi.M0) * epi.sCm1 + (m % epi.M0) * epi.sCm0;
            const uint32_t tq = tmem + ((uint32_t)(q * 32) << 16);
#pragma unroll 1
            for (int c = 0; c < BN; c += 16) {
                uint32_t r[16];
                tmem_ld16(tq + (uint32_t)c, r);
                if (!mvalid) continue;
                if (epi.out_fp64) {
                    double* Cd = (double*)epi.C + rbase;
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        const int64_t n = (int64_t)n0 + c + j;
                        if (n < N) {
                            double v = epi.alpha * (double)__uint_as_float(r[j]);
                            if (epi.beta != 0.0) v = fma(epi.beta, Cd[n], v);
                            Cd[n] = v;
                        }
                    }
                } else {
                    float* Cf = (float*)epi.C + rbase;
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        const int64_t n = (int64_t)n0 + c + j;
                        if (n < N) Cf[n] = (float)epi.alpha * __uint_as_float(r[j]);
                    }
                }
            }
        }
        tc_fence_before();
    }
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)BN)
                     : "memory");
    }
}

// Persistent variant: one CTA per SM walks its work items.  The accumulator is
// double-buffered in TMEM (2 x BN columns), so the epilogue of item i (TMEM ->
// global) overlaps the MMAs of item i+1; the smem ring and its phases run on
// across items.  acc_full[b] is committed by the MMA thread, acc_empty[b] is
// released by the four epilogue warps.
//
// Schedules.  Tile-per-item: CTA c takes tiles c, c + G, ...  Stream-K (sk
// != null): the tiles x nkb k-blocks are cut into G equal contiguous ranges,
// one per CTA, so a last partial wave of tiles no longer leaves SMs idle.  A
// range of at least nkb + 1 k-blocks splits a tile between at most two CTAs:
// the head (k-blocks from 0) ends CTA c's range, the tail starts CTA c+1's.
// Each CTA walks its range backwards, tile by tile: its head fragment first,
// which it stores raw (FP32) to sk->part[c] and flags per TMEM lane quadrant;
// its tail fragment last, which adds the head that CTA c-1 stored long before
// (a bounded wait on the flag) -- always in the same order, so the result is
// deterministic.  All CTAs are resident (one per SM), so no wait depends on a
// CTA that cannot run.

struct TcStreamK {
    float* part;     // [G][TC_BM][BN] head partials
    int* flag;       // [G][4]: 1 when quadrant q of CTA c's head partial is stored
    int64_t total;   // tiles * nkb
};

struct TcItem {
    int t, kb0, kb1;
};

// Number of work items of CTA c, and item j (0-based, in processing order).
__device__ __forceinline__ int tc_items(const TcStreamK* sk, int tiles, int nkb, int c, int G) {
    if (!sk) return c < tiles ? (tiles - 1 - c) / G + 1 : 0;
    const int64_t w0 = (int64_t)c * sk->total / G, w1 = (int64_t)(c + 1) * sk->total / G;
    if (w1 <= w0) return 0;
    return (int)((w1 - 1) / nkb - w0 / nkb + 1);
}
__device__ __forceinline__ TcItem tc_item(const TcStreamK* sk, int nkb, int c, int G, int j) {
    TcItem it;
    if (!sk) {
        it.t = c + j * G;
        it.kb0 = 0;
        it.kb1 = nkb;
        return it;
    }
    const int64_t w0 = (int64_t)c * sk->total / G, w1 = (int64_t)(c + 1) * sk->total / G;
    const int64_t t = (w1 - 1) / nkb - j;   // backwards: head fragment first, tail last
    const int64_t b = t * nkb;
    it.t = (int)t;
    it.kb0 = (int)(w0 > b ? w0 - b : 0);
    it.kb1 = (int)(w1 - b < nkb ? w1 - b : nkb);
    return it;
}

__device__ __forceinline__ int ld_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

template <int BN, int STAGES>
__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_gemm_persist_kernel(const __grid_constant__ CUtensorMap tmAh, const __grid_constant__ CUtensorMap tmAl,
                           const __grid_constant__ CUtensorMap tmBh, const __grid_constant__ CUtensorMap tmBl, int M,
                           int N, int Kpad, TcEpi epi, TcStreamK skd, int use_sk, const int* skip, int* status) {
    using L = TcSmem<BN, STAGES>;
    if (ct_skip(skip)) return;
    extern __shared__ uint8_t tc_smem_raw[];
    uint8_t* smem = tc_smem_raw + ((1024u - (smem_u32(tc_smem_raw) & 1023u)) & 1023u);
    uint64_t* full = (uint64_t*)(smem + L::TILE_BYTES);
    uint64_t* empty = full + STAGES;
    uint64_t* acc_full = empty + STAGES;
    uint64_t* acc_empty = acc_full + 2;
    uint32_t* tmem_slot = (uint32_t*)(acc_empty + 2);
    volatile int* abort_flag = (volatile int*)(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tiles_n = (N + BN - 1) / BN;
    const int tiles = tiles_n * ((M + TC_BM - 1) / TC_BM);
    const int nkb = Kpad / TC_BK;
    const TcStreamK* sk = use_sk ? &skd : nullptr;
    const int c = blockIdx.x, G = gridDim.x;
    const int nitems = tc_items(sk, tiles, nkb, c, G);

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], 4);
        }
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"((uint32_t)(2 * BN))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            int g = 0;
            bool ok = true;
            for (int j = 0; j < nitems && ok; ++j) {
                const TcItem it = tc_item(sk, nkb, c, G, j);
                const int m0 = (it.t / tiles_n) * TC_BM, n0 = (it.t % tiles_n) * BN;
                for (int kb = it.kb0; kb < it.kb1; ++kb, ++g) {
                    const int s = g % STAGES;
                    const uint32_t ph = (uint32_t)(g / STAGES) & 1u;
                    if (g >= STAGES && !mbar_wait(&empty[s], ph ^ 1u, abort_flag)) {
                        *abort_flag = 1;
                        ct_set_status(status, CT_ERR_CUDA);
                        ok = false;
                        break;
                    }
                    uint8_t* st = smem + s * L::STAGE_BYTES;
                    mbar_expect_tx(&full[s], L::STAGE_BYTES);
                    const int x = kb * TC_BK;
                    tma_load_2d(st, &tmAh, x, m0, &full[s]);
                    tma_load_2d(st + L::A_BYTES, &tmAl, x, m0, &full[s]);
                    tma_load_2d(st + 2 * L::A_BYTES, &tmBh, x, n0, &full[s]);
                    tma_load_2d(st + 2 * L::A_BYTES + L::B_BYTES, &tmBl, x, n0, &full[s]);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = idesc_tf32(TC_BM, BN);
            int g = 0;
            bool ok = true;
            for (int i = 0; i < nitems && ok; ++i) {
                const TcItem it = tc_item(sk, nkb, c, G, i);
                const int b = i & 1, u = i >> 1;
                if (u > 0 && !mbar_wait(&acc_empty[b], (uint32_t)((u - 1) & 1), abort_flag)) {
                    *abort_flag = 1;
                    ct_set_status(status, CT_ERR_CUDA);
                    break;
                }
                tc_fence_after();
                const uint32_t dt = tmem + (uint32_t)(b * BN);
                for (int kb = it.kb0; kb < it.kb1; ++kb, ++g) {
                    const int s = g % STAGES;
                    const uint32_t ph = (uint32_t)(g / STAGES) & 1u;
                    if (!mbar_wait(&full[s], ph, abort_flag)) {
                        *abort_flag = 1;
                        ct_set_status(status, CT_ERR_CUDA);
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t a_hi = smem_u32(smem + s * L::STAGE_BYTES);
                    const uint32_t a_lo = a_hi + L::A_BYTES;
                    const uint32_t b_hi = a_hi + 2 * L::A_BYTES;
                    const uint32_t b_lo = b_hi + L::B_BYTES;
#pragma unroll
                    for (int kk = 0; kk < TC_BK / 8; ++kk) {
                        const uint32_t off = kk * 32;
                        const uint32_t acc0 = (kb > it.kb0 || kk > 0) ? 1u : 0u;
                        mma_tf32(dt, sw128_desc(a_lo + off), sw128_desc(b_hi + off), idesc, acc0);
                        mma_tf32(dt, sw128_desc(a_hi + off), sw128_desc(b_lo + off), idesc, 1u);
                        mma_tf32(dt, sw128_desc(a_hi + off), sw128_desc(b_hi + off), idesc, 1u);
                    }
                    mma_commit(&empty[s]);
                }
                if (ok) mma_commit(&acc_full[b]);
            }
        }
    } else {
        const int q = warp & 3;
        const int row = q * 32 + lane;
        for (int i = 0; i < nitems; ++i) {
            const TcItem it = tc_item(sk, nkb, c, G, i);
            const int b = i & 1, u = i >> 1;
            const bool ok = mbar_wait(&acc_full[b], (uint32_t)(u & 1), abort_flag);
            if (!ok) {
                *abort_flag = 1;
                ct_set_status(status, CT_ERR_CUDA);
                break;
            }
            __syncwarp();
            tc_fence_after();
            const bool head = sk && it.kb0 == 0 && it.kb1 < nkb;   // the rest of this tile is CTA c+1's
            const bool tail = sk && it.kb0 > 0;                    // CTA c-1 holds this tile's head
            const float* prev = nullptr;
            if (tail) {
                // CTA c-1 stored its head of this tile as its first item; wait for quadrant q
                const int* f = skd.flag + (int64_t)(c - 1) * 4 + q;
                bool seen = ld_acquire(f) != 0;
                if (!seen) {
                    const unsigned long long t0 = gtimer();
                    while (!(seen = ld_acquire(f) != 0)) {
                        if (*abort_flag || gtimer() - t0 > TC_WAIT_NS) break;
                    }
                }
                if (!seen) {
                    *abort_flag = 1;
                    ct_set_status(status, CT_ERR_CUDA);
                    break;
                }
                prev = skd.part + ((int64_t)(c - 1) * TC_BM + row) * BN;
            }
            const int m0 = (it.t / tiles_n) * TC_BM, n0 = (it.t % tiles_n) * BN;
            const int64_t m = (int64_t)m0 + row;
            const bool mvalid = m < M;
            int64_t rbase = 0;
            if (mvalid) rbase = (m / epi.M0) * epi.sCm1 + (m % epi.M0) * epi.sCm0;
            const uint32_t tq = tmem + (uint32_t)(b * BN) + ((uint32_t)(q * 32) << 16);
            float* mine = head ? skd.part + ((int64_t)c * TC_BM + row) * BN : nullptr;
#pragma unroll 1
            for (int cc = 0; cc < BN; cc += 16) {
                uint32_t r[16];
                tmem_ld16(tq + (uint32_t)cc, r);
                if (head) {
                    // raw partial of k-blocks [0, kb1), every row (the tail CTA masks)
#pragma unroll
                    for (int j = 0; j < 16; ++j) mine[cc + j] = __uint_as_float(r[j]);
                    continue;
                }
                if (!mvalid) continue;
                float v32[16];
#pragma unroll
                for (int j = 0; j < 16; ++j) v32[j] = prev ? prev[cc + j] + __uint_as_float(r[j]) : __uint_as_float(r[j]);
                const int64_t nb = (int64_t)n0 + cc;
                if (epi.vec && nb + 16 <= N) {
                    // 16-byte stores: a warp writes 32 rows x 64 B (FP32) or 128 B (FP64)
                    // per group of 4 / 8 instructions instead of one 4-byte word per row
                    if (epi.out_fp64) {
                        double2* Cd = (double2*)((double*)epi.C + rbase + nb);
#pragma unroll
                        for (int j = 0; j < 8; ++j) {
                            double2 o;
                            o.x = epi.alpha * (double)v32[2 * j];
                            o.y = epi.alpha * (double)v32[2 * j + 1];
                            if (epi.beta != 0.0) {
                                const double2 c0 = Cd[j];
                                o.x = fma(epi.beta, c0.x, o.x);
                                o.y = fma(epi.beta, c0.y, o.y);
                            }
                            Cd[j] = o;
                        }
                    } else {
                        float4* Cf = (float4*)((float*)epi.C + rbase + nb);
                        const float a = (float)epi.alpha;
#pragma unroll
                        for (int j = 0; j < 4; ++j)
                            Cf[j] = make_float4(a * v32[4 * j], a * v32[4 * j + 1], a * v32[4 * j + 2], a * v32[4 * j + 3]);
                    }
                    continue;
                }
                if (epi.out_fp64) {
                    double* Cd = (double*)epi.C + rbase;
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        const int64_t n = (int64_t)n0 + cc + j;
                        if (n < N) {
                            double v = epi.alpha * (double)v32[j];
                            if (epi.beta != 0.0) v = fma(epi.beta, Cd[n], v);
                            Cd[n] = v;
                        }
                    }
                } else {
                    float* Cf = (float*)epi.C + rbase;
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        const int64_t n = (int64_t)n0 + cc + j;
                        if (n < N) Cf[n] = (float)epi.alpha * v32[j];
                    }
                }
            }
            if (head) {
                __syncwarp();
                __threadfence();
                if (lane == 0) st_release(skd.flag + (int64_t)c * 4 + q, 1);
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&acc_empty[b]);
        }
    }
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)(2 * BN))
                     : "memory");
    }
}

// Chunked accumulation.  The tensor cores add into the FP32 accumulator with
// truncation (round toward zero): every MMA shrinks the running sum's magnitude
// by a fraction of an ulp, so a product summed over K in one accumulator comes
// out too small by ~6e-9 per unit of K (-3e-5 relative at K = 5120).  This
// variant bounds the number of adds into any accumulator: each tile's K range is
// cut into chunks of `kc` k-blocks (kc * 32 of K); every chunk starts a fresh
// TMEM accumulator, cycling through 512 / BN BN-column buffers, and the epilogue
// warps add the chunks in FP32 registers with round-to-nearest, whose errors
// have no sign preference.  The bias left is that of one chunk, kc times that of
// one 32-wide k-block (~1.8e-7).
//   * one CTA per SM; the schedule is hybrid (TcHybrid below): whole tiles
//     c, c + G, ... for the full waves, then the last partial wave's k-blocks
//     shared out evenly over the CTAs (stream-K);
//   * warps: 0 TMA producer, 1 TMEM allocator + MMA issuer, then 4 EPW epilogue
//     warps; epilogue warp w reads TMEM lane quadrant w % 4 (the quadrant a warp
//     may access) and column group (w - 2) / 4 of the tile, holding BN / EPW
//     FP32 running sums per thread.  EPW = 4 for the 128 x 128 tile (a chunk of
//     64 of K is ~2000 cycles of MMAs there, so the per-chunk epilogue must be
//     short), 2 for the 128 x 192 / 224 / 256 tiles (their 96 to 128 sums per
//     thread leave no room for more warps in the register file);
//   * acc_full[b] is committed by the MMA thread after a chunk's last MMA,
//     acc_empty[b] released by the epilogue warps once the chunk is in
//     registers, so the MMAs of the next chunks run while chunk i is read (with
//     four buffers -- two for the wide tiles -- the MMA thread is three chunks
//     -- one -- ahead, which hides the commit -> epilogue -> release latency of a
//     short chunk); a tile's stores overlap the next tile's first chunks;
//   * with epi.trans the kernel's tile rows are C's columns: each thread stores
//     its row's values down a column of C, so a warp store covers 32 consecutive
//     words.
__host__ __device__ constexpr int tc_chunk_epw(int BN) { return BN >= 192 ? 2 : 4; }
// tcgen05.alloc takes a power of two (>= 32) of columns
__host__ __device__ constexpr uint32_t tc_pow2_cols(int n) { return n <= 32 ? 32u : 2u * tc_pow2_cols((n + 1) / 2); }
__host__ __device__ constexpr int tc_chunk_threads(int BN) { return 32 * (2 + 4 * tc_chunk_epw(BN)); }

// Hybrid schedule.  Tiles [0, tiles_dp) (whole waves, tiles_dp a multiple of G)
// go round-robin, one whole tile per turn, so that the CTAs of a wave read the
// same operand rows at the same time (L2 reuse).  The k-blocks of the remaining
// tiles, units = (tiles - tiles_dp) * nkb of them in tile-major order, are cut
// into gsk equal contiguous ranges, CTA c < gsk taking [c*units/gsk,
// (c+1)*units/gsk); a tile whose k-blocks span several ranges is a set of
// pieces, numbered in k order.  Each piece's epilogue warp (region = lane
// quadrant x column group) stores its FP32 sums to its own partial slot, then
// counts itself in the tile-region's arrival counter; the warp that arrives
// last adds all pieces' partials in piece order and stores the result.  No CTA
// waits for another, and the sum is the same FP32 expression whichever piece
// arrives last (deterministic).  Counters carry the launch's epoch in their high
// half, so a counter left by an earlier (even an aborted) launch reads as zero
// and no reset is needed between launches.
struct TcHybrid {
    int tiles_dp;               // whole-tile part; == tiles when there is no stream-K part
    int gsk;                    // CTAs sharing the stream-K units (0: none)
    int64_t units;              // (tiles - tiles_dp) * nkb
    int maxp;                   // partial slots per stream-K tile (most pieces of any tile)
    unsigned epoch;             // nonzero tag of this launch
    float* part;                // [(tiles - tiles_dp) * maxp][regions][HC / 4][32] float4
    unsigned long long* cnt;    // [(tiles - tiles_dp) * regions]: epoch << 32 | arrivals
};

struct TcPiece {
    int t, kb0, kb1;   // tile, k-block range
    int p, n;          // piece index, pieces of the tile (n = 1: the whole tile)
    int st;            // stream-K tile index (t - tiles_dp), -1 for a whole tile
};

// Walks CTA c's work in processing order: its whole tiles, then its stream-K range.
struct TcCursor {
    int t;
    int64_t u, ue;
    __device__ TcCursor(const TcHybrid& hy, int c) : t(c), u(0), ue(0) {
        if (c < hy.gsk) {
            u = (int64_t)c * hy.units / hy.gsk;
            ue = (int64_t)(c + 1) * hy.units / hy.gsk;
        }
    }
    __device__ bool next(const TcHybrid& hy, int nkb, int G, int c, TcPiece& w) {
        if (t < hy.tiles_dp) {
            w.t = t;
            w.kb0 = 0;
            w.kb1 = nkb;
            w.p = 0;
            w.n = 1;
            w.st = -1;
            t += G;
            return true;
        }
        if (u >= ue) return false;
        const int st = (int)(u / nkb);
        const int k0 = (int)(u - (int64_t)st * nkb);
        const int64_t left = ue - u;
        const int k1 = left < nkb - k0 ? k0 + (int)left : nkb;
        // owner of unit x: the largest c with c*units/gsk <= x, i.e. ((x+1)*gsk - 1) / units
        const int64_t base = (int64_t)st * nkb;
        const int cf = (int)(((base + 1) * hy.gsk - 1) / hy.units);
        const int cl = (int)(((base + nkb) * hy.gsk - 1) / hy.units);
        w.t = hy.tiles_dp + st;
        w.kb0 = k0;
        w.kb1 = k1;
        w.p = c - cf;
        w.n = cl - cf + 1;
        w.st = st;
        u += k1 - k0;
        return true;
    }
};

// Count one arrival of this launch (epoch) at *p; returns the arrivals so far
// including this one, 0 if the CAS loop did not settle (it needs at most one
// retry per other piece of the tile).
__device__ __forceinline__ unsigned tc_arrive(unsigned long long* p, unsigned epoch) {
    unsigned long long old = *(volatile unsigned long long*)p;
    for (int i = 0; i < 1024; ++i) {
        const unsigned cnt = (unsigned)(old >> 32) == epoch ? (unsigned)old : 0u;
        const unsigned long long nw = ((unsigned long long)epoch << 32) | (unsigned long long)(cnt + 1u);
        const unsigned long long prev = atomicCAS(p, old, nw);
        if (prev == old) return cnt + 1u;
        old = prev;
    }
    return 0u;
}


// Registers: each SM sub-partition holds 16K of them; 10 warps put 3 on some
// sub-partitions (168 per thread), 18 warps put 5 (96 per thread, enough for 32
// sums and 32 loaded columns).
template <int BN, int STAGES>
__global__ void __launch_bounds__(tc_chunk_threads(BN), 1)
    tc_gemm_chunk_kernel(const __grid_constant__ CUtensorMap tmAh, const __grid_constant__ CUtensorMap tmAl,
                         const __grid_constant__ CUtensorMap tmBh, const __grid_constant__ CUtensorMap tmBl, int M,
                         int N, int Kpad, int kc, TcEpi epi, TcHybrid hy, const int* skip, int* status) {
    using L = TcSmem<BN, STAGES>;
    constexpr int EPW = tc_chunk_epw(BN);
    constexpr int HC = BN / EPW;   // columns per epilogue warp
    constexpr int NB = 512 / BN;   // chunk accumulators in TMEM (all 512 columns)
    constexpr uint32_t TMEM_COLS = tc_pow2_cols(NB * BN);
    if (ct_skip(skip)) return;
    extern __shared__ uint8_t tc_smem_raw[];
    uint8_t* smem = tc_smem_raw + ((1024u - (smem_u32(tc_smem_raw) & 1023u)) & 1023u);
    uint64_t* full = (uint64_t*)(smem + L::TILE_BYTES);
    uint64_t* empty = full + STAGES;
    uint64_t* acc_full = empty + STAGES;
    uint64_t* acc_empty = acc_full + NB;
    uint32_t* tmem_slot = (uint32_t*)(acc_empty + NB);
    volatile int* abort_flag = (volatile int*)(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tiles_n = (N + BN - 1) / BN;
    const int nkb = Kpad / TC_BK;
    const int c = blockIdx.x, G = gridDim.x;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < NB; ++b) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], 4 * EPW);
        }
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            int g = 0;
            bool ok = true;
            TcCursor cur(hy, c);
            TcPiece w;
            while (ok && cur.next(hy, nkb, G, c, w)) {
                const int m0 = (w.t / tiles_n) * TC_BM, n0 = (w.t % tiles_n) * BN;
                for (int kb = w.kb0; kb < w.kb1; ++kb, ++g) {
                    const int s = g % STAGES;
                    const uint32_t ph = (uint32_t)(g / STAGES) & 1u;
                    if (g >= STAGES && !mbar_wait(&empty[s], ph ^ 1u, abort_flag)) {
                        *abort_flag = 1;
                        ct_set_status(status, CT_ERR_CUDA);
                        ok = false;
                        break;
                    }
                    uint8_t* st = smem + s * L::STAGE_BYTES;
                    mbar_expect_tx(&full[s], L::STAGE_BYTES);
                    const int x = kb * TC_BK;
                    tma_load_2d(st, &tmAh, x, m0, &full[s]);
                    tma_load_2d(st + L::A_BYTES, &tmAl, x, m0, &full[s]);
                    tma_load_2d(st + 2 * L::A_BYTES, &tmBh, x, n0, &full[s]);
                    tma_load_2d(st + 2 * L::A_BYTES + L::B_BYTES, &tmBl, x, n0, &full[s]);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = idesc_tf32(TC_BM, BN);
            int g = 0, gc = 0;
            bool ok = true;
            TcCursor cur(hy, c);
            TcPiece w;
            while (ok && cur.next(hy, nkb, G, c, w)) {
                for (int kb0 = w.kb0; kb0 < w.kb1 && ok; kb0 += kc, ++gc) {
                    const int b = gc % NB, u = gc / NB;
                    if (u > 0 && !mbar_wait(&acc_empty[b], (uint32_t)((u - 1) & 1), abort_flag)) {
                        *abort_flag = 1;
                        ct_set_status(status, CT_ERR_CUDA);
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t dt = tmem + (uint32_t)(b * BN);
                    const int kb1 = kb0 + kc < w.kb1 ? kb0 + kc : w.kb1;
                    for (int kb = kb0; kb < kb1; ++kb, ++g) {
                        const int s = g % STAGES;
                        const uint32_t ph = (uint32_t)(g / STAGES) & 1u;
                        if (!mbar_wait(&full[s], ph, abort_flag)) {
                            *abort_flag = 1;
                            ct_set_status(status, CT_ERR_CUDA);
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                        const uint32_t a_hi = smem_u32(smem + s * L::STAGE_BYTES);
                        const uint32_t a_lo = a_hi + L::A_BYTES;
                        const uint32_t b_hi = a_hi + 2 * L::A_BYTES;
                        const uint32_t b_lo = b_hi + L::B_BYTES;
#pragma unroll
                        for (int kk = 0; kk < TC_BK / 8; ++kk) {
                            const uint32_t off = kk * 32;
                            const uint32_t acc0 = (kb > kb0 || kk > 0) ? 1u : 0u;
                            mma_tf32(dt, sw128_desc(a_lo + off), sw128_desc(b_hi + off), idesc, acc0);
                            mma_tf32(dt, sw128_desc(a_hi + off), sw128_desc(b_lo + off), idesc, 1u);
                            mma_tf32(dt, sw128_desc(a_hi + off), sw128_desc(b_hi + off), idesc, 1u);
                        }
                        mma_commit(&empty[s]);
                    }
                    if (ok) mma_commit(&acc_full[b]);
                }
            }
        }
    } else {
        const int q = warp & 3;              // TMEM lane quadrant of this warp
        const int hf = (warp - 2) >> 2;      // column group of the tile
        const int row = q * 32 + lane;
        float sum[HC];
        int gc = 0;
        bool ok = true;
        TcCursor cur(hy, c);
        TcPiece w;
        while (ok && cur.next(hy, nkb, G, c, w)) {
#pragma unroll
            for (int j = 0; j < HC; ++j) sum[j] = 0.f;
            for (int kb0 = w.kb0; kb0 < w.kb1; kb0 += kc, ++gc) {
                const int b = gc % NB, u = gc / NB;
                if (!mbar_wait(&acc_full[b], (uint32_t)(u & 1), abort_flag)) {
                    *abort_flag = 1;
                    ct_set_status(status, CT_ERR_CUDA);
                    ok = false;
                    break;
                }
                __syncwarp();
                tc_fence_after();
                const uint32_t tq = tmem + (uint32_t)(b * BN + hf * HC) + ((uint32_t)(q * 32) << 16);
                // LB columns per wait: several TMEM loads in flight before one
                // tcgen05.wait::ld (fewer for the wide tile, whose 128 sums leave
                // room for 32 more registers only)
                constexpr int LB = HC >= 96 ? (HC % 32 == 0 ? 32 : 16) : HC;
#pragma unroll
                for (int cc = 0; cc < HC; cc += LB) {
                    uint32_t r[LB];
#pragma unroll
                    for (int q8 = 0; q8 < LB; q8 += 8)
                        tmem_ld8_nowait(tq + (uint32_t)(cc + q8), *reinterpret_cast<uint32_t(*)[8]>(&r[q8]));
                    tmem_wait_ld();
#pragma unroll
                    for (int j = 0; j < LB; ++j) sum[cc + j] += __uint_as_float(r[j]);
                }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&acc_empty[b]);
            }
            if (!ok) break;
            if (w.n > 1) {
                // a piece of a stream-K tile: FP32 sums to this piece's slot (lane-interleaved
                // float4, so a warp's store covers 512 contiguous bytes), then the arrival count
                constexpr int NREG = 4 * EPW;
                constexpr int64_t REG4 = (int64_t)(HC / 4) * 32;       // float4 per region
                const int region = warp - 2;
                if (w.n > hy.maxp) {
                    *abort_flag = 1;
                    ct_set_status(status, CT_ERR_CUDA);
                    ok = false;
                    break;
                }
                float4* slot0 = (float4*)hy.part + ((int64_t)w.st * hy.maxp * NREG + region) * REG4 + lane;
                float4* mine = slot0 + (int64_t)w.p * NREG * REG4;
#pragma unroll
                for (int j4 = 0; j4 < HC / 4; ++j4)
                    __stcg(mine + j4 * 32, make_float4(sum[4 * j4], sum[4 * j4 + 1], sum[4 * j4 + 2], sum[4 * j4 + 3]));
                __threadfence();
                __syncwarp();
                unsigned arrived = 0;
                if (lane == 0) {
                    arrived = tc_arrive(hy.cnt + (int64_t)w.st * NREG + region, hy.epoch);
                    __threadfence();
                }
                arrived = __shfl_sync(0xffffffffu, arrived, 0);
                if (arrived == 0) {
                    *abort_flag = 1;
                    ct_set_status(status, CT_ERR_CUDA);
                    ok = false;
                    break;
                }
                if ((int)arrived < w.n) continue;   // a later piece stores the tile
                __threadfence();
                // the last piece: sum the n partials in piece order, LG columns at a time
                constexpr int LG = HC >= 128 ? 32 : 16;
#pragma unroll
                for (int cg = 0; cg < HC; cg += LG) {
#pragma unroll
                    for (int j4 = 0; j4 < LG / 4; ++j4) {
                        const float4 v = __ldcg(slot0 + (cg / 4 + j4) * 32);
                        sum[cg + 4 * j4] = v.x;
                        sum[cg + 4 * j4 + 1] = v.y;
                        sum[cg + 4 * j4 + 2] = v.z;
                        sum[cg + 4 * j4 + 3] = v.w;
                    }
                    for (int q = 1; q < w.n; ++q) {
                        const float4* sq = slot0 + (int64_t)q * NREG * REG4;
#pragma unroll
                        for (int j4 = 0; j4 < LG / 4; ++j4) {
                            const float4 v = __ldcg(sq + (cg / 4 + j4) * 32);
                            sum[cg + 4 * j4] += v.x;
                            sum[cg + 4 * j4 + 1] += v.y;
                            sum[cg + 4 * j4 + 2] += v.z;
                            sum[cg + 4 * j4 + 3] += v.w;
                        }
                    }
                }
            }
            const int m0 = (w.t / tiles_n) * TC_BM;
            const int n0 = (w.t % tiles_n) * BN + hf * HC;
            const int64_t m = (int64_t)m0 + row;
            if (m >= M) continue;
            if (epi.trans) {
                // element (m, n) to C[n][m]: for each n the warp's 32 rows are 32 consecutive words
#pragma unroll
                for (int j = 0; j < HC; ++j) {
                    const int64_t n = (int64_t)n0 + j;
                    if (n >= N) break;
                    const int64_t a = n * epi.sCm0 + m;
                    if (epi.out_fp64) {
                        double* Cd = (double*)epi.C;
                        double v = epi.alpha * (double)sum[j];
                        if (epi.beta != 0.0) v = fma(epi.beta, Cd[a], v);
                        Cd[a] = v;
                    } else {
                        ((float*)epi.C)[a] = (float)epi.alpha * sum[j];
                    }
                }
                continue;
            }
            const int64_t rbase = (m / epi.M0) * epi.sCm1 + (m % epi.M0) * epi.sCm0;
#pragma unroll
            for (int cc = 0; cc < HC; cc += 16) {
                const int64_t nb = (int64_t)n0 + cc;
                if (epi.vec && nb + 16 <= N) {
                    if (epi.out_fp64) {
                        double2* Cd = (double2*)((double*)epi.C + rbase + nb);
#pragma unroll
                        for (int j = 0; j < 8; ++j) {
                            double2 o;
                            o.x = epi.alpha * (double)sum[cc + 2 * j];
                            o.y = epi.alpha * (double)sum[cc + 2 * j + 1];
                            if (epi.beta != 0.0) {
                                const double2 c0 = Cd[j];
                                o.x = fma(epi.beta, c0.x, o.x);
                                o.y = fma(epi.beta, c0.y, o.y);
                            }
                            Cd[j] = o;
                        }
                    } else {
                        float4* Cf = (float4*)((float*)epi.C + rbase + nb);
                        const float a = (float)epi.alpha;
#pragma unroll
                        for (int j = 0; j < 4; ++j)
                            Cf[j] = make_float4(a * sum[cc + 4 * j], a * sum[cc + 4 * j + 1], a * sum[cc + 4 * j + 2],
                                                a * sum[cc + 4 * j + 3]);
                    }
                    continue;
                }
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int64_t n = nb + j;
                    if (n >= N) break;
                    if (epi.out_fp64) {
                        double* Cd = (double*)epi.C + rbase;
                        double v = epi.alpha * (double)sum[cc + j];
                        if (epi.beta != 0.0) v = fma(epi.beta, Cd[n], v);
                        Cd[n] = v;
                    } else {
                        ((float*)epi.C)[rbase + n] = (float)epi.alpha * sum[cc + j];
                    }
                }
            }
        }
    }
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS)
                     : "memory");
    }
}

// ---------------------------------------------------------------------------
// operand packer: FP64 source -> split TF32 planes [rows][ldk], K-major.
// row r = r1 * R0 + r0 ; col k = k1 * K0p + k0 (k0 < K0 valid, K0..K0p zero)
// src address = r1*s_r1 + r0*s_r0 + k1*s_k1 + k0*s_k0
// ---------------------------------------------------------------------------
struct PackDesc {
    const double* src;
    int64_t rows, R0, s_r1, s_r0;
    int64_t K1, K0, K0p, s_k1, s_k0;
    float* hi;
    float* lo;
    int64_t ldk;   // = K1 * K0p rounded up to 32
    double scale;
    const double* scale_ptr;   // optional device scalar multiplier
};

// 32 x 32 tiles through shared memory; K_FAST: source contiguous along k0.
// The tile's 32 row offsets and 32 column offsets are computed once per block
// (the 64-bit divisions of the index split would otherwise dominate).
template <bool K_FAST>
__global__ void __launch_bounds__(256) pack_split_kernel(PackDesc p, const int* skip) {
    if (ct_skip(skip)) return;
    __shared__ double tile[32][33];
    __shared__ int64_t roff[32], koff[32];
    const int64_t rb = (int64_t)blockIdx.y * 32;
    const int64_t kb = (int64_t)blockIdx.x * 32;   // in padded k space
    const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
    if (ty == 0) {
        const int64_t r = rb + tx;
        roff[tx] = (r < p.rows) ? (r / p.R0) * p.s_r1 + (r % p.R0) * p.s_r0 : -1;
    } else if (ty == 1) {
        const int64_t k = kb + tx;
        int64_t o = -1;
        if (k < p.ldk) {
            const int64_t k1 = k / p.K0p, k0 = k % p.K0p;
            if (k1 < p.K1 && k0 < p.K0) o = k1 * p.s_k1 + k0 * p.s_k0;
        }
        koff[tx] = o;
    }
    double scd = p.scale;
    if (p.scale_ptr) scd *= *p.scale_ptr;
    const float sc = (float)scd;
    __syncthreads();
    for (int i = ty; i < 32; i += 8) {
        const int ri = K_FAST ? i : tx, ki = K_FAST ? tx : i;
        const int64_t ro = roff[ri], ko = koff[ki];
        const double v = (ro >= 0 && ko >= 0) ? p.src[ro + ko] : 0.0;
        if (K_FAST) tile[i][tx] = v;
        else tile[tx][i] = v;
    }
    __syncthreads();
    for (int i = ty; i < 32; i += 8) {
        const int64_t r = rb + i, k = kb + tx;
        if (r < p.rows && k < p.ldk) {
            float h, l;
            split_tf32((float)tile[i][tx] * sc, h, l);
            p.hi[r * p.ldk + k] = h;
            p.lo[r * p.ldk + k] = l;
        }
    }
}

// MPO leg in FP32 with split-TF32 output: out(o, j, i) = sum_k Wt[j,k] in(o,k,i)
struct MpoTcDesc {
    int64_t O, K, J, I;
    const float* in; int64_t sIo, sIk, sIi;
    float* hi; float* lo; int64_t sOo, sOi, J0, sOj1, sOj0;
    const double* Wt;
    const int* skip;
};

constexpr int MPOT_NT = 128, MPOT_JC = 32;

// Block (x, o, z) handles columns i of slab o for the output rows j in chunk z
// ([z * jch, z * jch + jch) of J).  Dynamic shared memory: that chunk of Wt as
// FP32 [jch][K], then its jch output offsets (int64).
__global__ void __launch_bounds__(MPOT_NT) mpo_tc_kernel(MpoTcDesc m, int64_t jch) {
    if (ct_skip(m.skip)) return;
    extern __shared__ float wsf[];
    const int64_t jbeg = (int64_t)blockIdx.z * jch;
    const int64_t jn = (m.J - jbeg) < jch ? (m.J - jbeg) : jch;
    const int64_t JK = jn * m.K;
    int64_t* joff = reinterpret_cast<int64_t*>(wsf + ((jch * m.K + 1) & ~(int64_t)1));
    for (int64_t t = threadIdx.x; t < JK; t += MPOT_NT) wsf[t] = (float)m.Wt[jbeg * m.K + t];
    for (int64_t j = threadIdx.x; j < jn; j += MPOT_NT) {
        const int64_t jj = jbeg + j;
        joff[j] = (jj / m.J0) * m.sOj1 + (jj % m.J0) * m.sOj0;
    }
    __syncthreads();
    const int64_t o = blockIdx.y;
    const int64_t i = (int64_t)blockIdx.x * MPOT_NT + threadIdx.x;
    if (i >= m.I) return;
    const float* in = m.in + o * m.sIo + i * m.sIi;
    const int64_t obase = o * m.sOo + i * m.sOi;
    for (int64_t j0 = 0; j0 < jn; j0 += MPOT_JC) {
        float acc[MPOT_JC];
#pragma unroll
        for (int jj = 0; jj < MPOT_JC; ++jj) acc[jj] = 0.f;
        const int nj = (int)((jn - j0) < MPOT_JC ? (jn - j0) : MPOT_JC);
        for (int64_t k = 0; k < m.K; ++k) {
            const float x = in[k * m.sIk];
#pragma unroll
            for (int jj = 0; jj < MPOT_JC; ++jj)
                if (jj < nj) acc[jj] = fmaf(wsf[(j0 + jj) * m.K + k], x, acc[jj]);
        }
#pragma unroll
        for (int jj = 0; jj < MPOT_JC; ++jj) {
            if (jj >= nj) break;
            const int64_t off = obase + joff[j0 + jj];
            float h, l;
            split_tf32(acc[jj], h, l);
            m.hi[off] = h;
            m.lo[off] = l;
        }
    }
}

// Two adjacent columns per thread (float2 loads and stores) and the weights
// stored k-major in shared memory, read four at a time: per k one global load
// and JT/4 shared loads feed 2 JT FMAs.  Block (x, o, z): columns
// [2 (x * MPOT_NT + tid), +2) of slab o, output rows [z JT, z JT + JT) of J.
// Needs unit column strides and even I, sIo, sIk, sOo and output offsets.
template <int JT>
__global__ void __launch_bounds__(MPOT_NT) mpo_tc2_kernel(MpoTcDesc m) {
    if (ct_skip(m.skip)) return;
    extern __shared__ __align__(16) float wk[];   // [K][JT], then JT int64 offsets
    const int64_t jbeg = (int64_t)blockIdx.z * JT;
    const int jn = (int)((m.J - jbeg) < JT ? (m.J - jbeg) : JT);
    int64_t* joff = reinterpret_cast<int64_t*>(wk + ((m.K * JT + 3) & ~(int64_t)3));
    for (int64_t t = threadIdx.x; t < m.K * JT; t += MPOT_NT) {
        const int64_t k = t / JT, jj = t % JT;
        wk[t] = (jj < jn) ? (float)m.Wt[(jbeg + jj) * m.K + k] : 0.f;
    }
    for (int j = threadIdx.x; j < jn; j += MPOT_NT) {
        const int64_t jj = jbeg + j;
        joff[j] = (jj / m.J0) * m.sOj1 + (jj % m.J0) * m.sOj0;
    }
    __syncthreads();
    const int64_t o = blockIdx.y;
    const int64_t i = 2 * ((int64_t)blockIdx.x * MPOT_NT + threadIdx.x);
    if (i >= m.I) return;
    const float* in = m.in + o * m.sIo + i;
    float acc[JT][2];
#pragma unroll
    for (int j = 0; j < JT; ++j) acc[j][0] = acc[j][1] = 0.f;
    for (int64_t k = 0; k < m.K; ++k) {
        const float2 x = *reinterpret_cast<const float2*>(in + k * m.sIk);
        const float4* w = reinterpret_cast<const float4*>(wk + k * JT);
#pragma unroll
        for (int j4 = 0; j4 < JT / 4; ++j4) {
            const float4 v = w[j4];
            acc[4 * j4 + 0][0] = fmaf(v.x, x.x, acc[4 * j4 + 0][0]);
            acc[4 * j4 + 0][1] = fmaf(v.x, x.y, acc[4 * j4 + 0][1]);
            acc[4 * j4 + 1][0] = fmaf(v.y, x.x, acc[4 * j4 + 1][0]);
            acc[4 * j4 + 1][1] = fmaf(v.y, x.y, acc[4 * j4 + 1][1]);
            acc[4 * j4 + 2][0] = fmaf(v.z, x.x, acc[4 * j4 + 2][0]);
            acc[4 * j4 + 2][1] = fmaf(v.z, x.y, acc[4 * j4 + 2][1]);
            acc[4 * j4 + 3][0] = fmaf(v.w, x.x, acc[4 * j4 + 3][0]);
            acc[4 * j4 + 3][1] = fmaf(v.w, x.y, acc[4 * j4 + 3][1]);
        }
    }
    const int64_t obase = o * m.sOo + i;
#pragma unroll
    for (int j = 0; j < JT; ++j) {
        if (j >= jn) break;
        float2 hv, lv;
        split_tf32(acc[j][0], hv.x, lv.x);
        split_tf32(acc[j][1], hv.y, lv.y);
        *reinterpret_cast<float2*>(m.hi + obase + joff[j]) = hv;
        *reinterpret_cast<float2*>(m.lo + obase + joff[j]) = lv;
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

bool get_encoder() {
    if (g_encode) return true;
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess || fn == nullptr) {
        (void)cudaGetLastError();
        return false;
    }
    g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    return true;
}

}  // namespace

// the driver's cuTensorMapEncodeTiled for the other tensor-core translation units (null when absent)
PFN_cuTensorMapEncodeTiled_v12000 ct_tma_encoder() { return get_encoder() ? g_encode : nullptr; }

namespace {

int make_map(ct_handle* h, CUtensorMap* m, const float* base, int64_t rows, int64_t ldk, int box_rows) {
    if (((uintptr_t)base & 15) || (ldk % TC_BK)) {
        ct_seterr(h, "TMA operand misaligned (base %p, ldk %lld)", (const void*)base, (long long)ldk);
        return CT_ERR_INVALID;
    }
    cuuint64_t dims[2] = {(cuuint64_t)ldk, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)(ldk * 4)};
    cuuint32_t box[2] = {(cuuint32_t)TC_BK, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)base, dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        ct_seterr(h, "cuTensorMapEncodeTiled failed (%d)", (int)r);
        return CT_ERR_CUDA;
    }
    return CT_OK;
}

// Tile shapes of the GEMM: 128 x 128 with a 3-stage ring (64 KB stages), or 128 x 192 / 128 x 256
// with a 2-stage ring (80 / 96 KB stages; 192 in the chunked kernel only).  The wide tile reads
// 25% fewer operand bytes from shared memory and L2 per MMA flop; the narrow one leaves smaller
// partial waves.  CTDMRG_TC_BN=128, 192 or 256 forces one; otherwise tc_pick_bn chooses per shape.
constexpr int GEMM_STAGES_N = 3;
constexpr int GEMM_STAGES_W = 2;

// read on every launch (one environment scan, next to a launch of tens of microseconds), so a
// test can switch tile shapes inside one process
int tc_bn_mode() {
    const char* e = getenv("CTDMRG_TC_BN");
    if (!e) return 0;
    const int b = atoi(e);
    return (b == 128 || b == 192 || b == 224 || b == 256) ? b : 0;
}

// persistent kernel by default; CTDMRG_TC_TILE_PER_CTA=1 selects the one-tile-per-CTA kernel
bool tc_use_persistent() {
    static const bool v = [] {
        const char* e = getenv("CTDMRG_TC_TILE_PER_CTA");
        return !(e && e[0] == '1');
    }();
    return v;
}

// stream-K schedule of the persistent kernel only on request (CTDMRG_TC_STREAM_K=1): measured
// on the H_eff shapes it did not pay (4096x1024x5120: 0.192 vs 0.191 ms; 5120x4096x1024:
// 0.242 vs 0.217 ms), the contiguous per-CTA ranges lose the L2 reuse of neighbouring tiles
bool tc_use_stream_k() {
    static const bool v = [] {
        const char* e = getenv("CTDMRG_TC_STREAM_K");
        return e && e[0] == '1';
    }();
    return v;
}

// K-blocks (32 of K each) per TMEM accumulator of the chunked kernel: CTDMRG_TC_KCHUNK=n, read
// on every launch like CTDMRG_TC_BN; 0 selects the single-accumulator persistent kernel.
int tc_kchunk() {
    const char* e = getenv("CTDMRG_TC_KCHUNK");
    if (!e) return 2;
    const int k = atoi(e);
    return k < 0 ? 0 : (k > 1024 ? 1024 : k);
}

// The chunked kernel's hybrid schedule (TcHybrid): on unless CTDMRG_TC_HYBRID=0, read on every
// launch like CTDMRG_TC_BN.
bool tc_hybrid_on() {
    const char* e = getenv("CTDMRG_TC_HYBRID");
    return !(e && e[0] == '0');
}

// Plans the stream-K part for `tiles` tiles of nkb k-blocks on G SMs.  False (hy: whole tiles
// only) when the last wave is full, when ranges of at least max(8, 2 kc) k-blocks would still be
// whole tiles, or when the shared-out last wave would not be clearly shorter than one tile
// (its longest range above 0.85 nkb).
bool tc_plan_hybrid(int64_t tiles, int G, int64_t nkb, int kc, TcHybrid& hy) {
    hy = TcHybrid{};
    hy.tiles_dp = (int)tiles;
    hy.maxp = 1;
    if (!tc_hybrid_on() || G <= 0 || nkb <= 0) return false;
    const int64_t r = tiles % G;
    // not without whole waves: a schedule of pieces only (tiles < G) made the CTAs sharing an
    // operand row read it at different k (4096x1024x5120 in 128 x 256 tiles: 205 against 238
    // TFLOP/s for one partial wave of whole tiles)
    if (r == 0 || tiles < G) return false;
    const int64_t units = r * nkb;
    const int64_t minu = 2 * kc > 8 ? 2 * kc : 8;
    const int64_t gsk = units / minu < G ? units / minu : G;
    if (gsk <= r) return false;
    if (ct_cdiv(units, gsk) * 20 > nkb * 17) return false;
    int64_t maxp = 1;
    for (int64_t st = 0; st < r; ++st) {
        const int64_t base = st * nkb;
        const int64_t cf = ((base + 1) * gsk - 1) / units, cl = ((base + nkb) * gsk - 1) / units;
        if (cl - cf + 1 > maxp) maxp = cl - cf + 1;
    }
    hy.tiles_dp = (int)(tiles - r);
    hy.gsk = (int)gsk;
    hy.units = units;
    hy.maxp = (int)maxp;
    return true;
}

// Grows the handle's stream-K partials / counters (after a synchronisation of the handle's
// stream, so no running launch uses the old ones); new counters start at zero (epoch 0, stale).
int tc_hybrid_scratch(ct_handle* h, int64_t part_floats, int64_t cnt_n) {
    if (h->tc_hy_part_floats >= part_floats && h->tc_hy_cnt_n >= cnt_n) return CT_OK;
    CT_CUDA(h, cudaStreamSynchronize(h->stream));
    if (h->tc_hy_part_floats < part_floats) {
        cudaFree(h->tc_hy_part);
        h->tc_hy_part = nullptr;
        h->tc_hy_part_floats = 0;
        CT_CUDA(h, cudaMalloc((void**)&h->tc_hy_part, (size_t)part_floats * sizeof(float)));
        h->tc_hy_part_floats = part_floats;
    }
    if (h->tc_hy_cnt_n < cnt_n) {
        cudaFree(h->tc_hy_cnt);
        h->tc_hy_cnt = nullptr;
        h->tc_hy_cnt_n = 0;
        CT_CUDA(h, cudaMalloc((void**)&h->tc_hy_cnt, (size_t)cnt_n * sizeof(unsigned long long)));
        CT_CUDA(h, cudaMemsetAsync(h->tc_hy_cnt, 0, (size_t)cnt_n * sizeof(unsigned long long), h->stream));
        h->tc_hy_cnt_n = cnt_n;
    }
    return CT_OK;
}

// Tile width per shape: the least (waves x BN / speed(BN)), waves counted whole.  Speed is a
// width's rate per flop relative to 128.  Single-accumulator kernels: at K <= 2048 the wide
// tile's fixed per-tile cost (pipeline fill, epilogue) is spread over twice the MMAs, measured as
// 1.12x (5120x4096x1024: 0.164 vs 0.166 ms; 2048x2048x1024: 0.037 vs 0.041 ms); at K = 5120 both
// run at the same rate.  Chunked kernel: each chunk boundary costs a fixed ~0.2 us of tensor time
// whatever the width, so wide tiles gain at every K; measured on 5120x4096x1024, 4096x1024x5120,
// 2048x2048x1024 and 8192x2048x8192 with whole waves counted, 192 runs at 1.13-1.30x and 256 at
// 1.24-1.33x the 128-wide rate (used: 1.2, 1.25 for 224, 1.28).
// With the hybrid schedule (hybrid_kc > 0: the chunk width) a partial last wave costs its
// longest shared-out range plus the partial sums' store and reload, ~15 us measured, in units
// of one tile's time (~36 us for a 128 x 256 x 1024 tile at 1.28).
double tc_width_speed(int bn, int64_t K, bool chunked) {
    if (bn <= 128) return 1.0;
    if (!chunked) return K <= 2048 ? 1.12 : 1.0;
    return bn >= 256 ? 1.28 : bn >= 224 ? 1.25 : 1.2;
}

int tc_pick_bn(int64_t M, int64_t N, int64_t K, int num_sms, bool chunked, int hybrid_kc, double* cost_out) {
    const int mode = tc_bn_mode();
    if (mode) return mode;
    const int64_t tm = ct_cdiv(M, TC_BM);
    const int64_t nkb = ct_cdiv(K, TC_BK);
    auto cost = [&](int bn) {
        const double speed = tc_width_speed(bn, K, chunked);
        const int64_t tiles = tm * ct_cdiv(N, bn);
        double waves = (double)ct_cdiv(tiles, num_sms);
        TcHybrid hy;
        if (hybrid_kc > 0 && tc_plan_hybrid(tiles, num_sms, nkb, hybrid_kc, hy)) {
            const double tile_us = 36.0 * ((double)nkb / 32.0) * ((double)bn / 256.0) * (1.28 / speed);
            const double sk = (double)(hy.tiles_dp / num_sms) + (double)ct_cdiv(hy.units, hy.gsk) / (double)nkb +
                              15.0 / tile_us;
            if (sk < waves) waves = sk;
        }
        return waves * (double)bn / speed;
    };
    int best = 128;
    double c = cost(128);
    // 192 / 224 (chunked kernel only) fill waves that 256 leaves partial: 5120 x 4096 takes 640
    // tiles of 256 (4.2 waves on 152 SMs), 880 of 192 (5.8), 760 of 224 (5.0)
    for (int bn : {256, 224, 192}) {
        if (N <= 128 || (bn < 256 && !chunked)) continue;
        const double cb = cost(bn);
        if (cb < c) {
            c = cb;
            best = bn;
        }
    }
    if (cost_out) *cost_out = c;
    return best;
}

// CTDMRG_TC_TRANS: 0 never computes the transposed product, 1 always where it may (chunked
// kernel, single-level rows), unset chooses by the tile cost; read on every launch.
int tc_trans_mode() {
    const char* e = getenv("CTDMRG_TC_TRANS");
    if (!e) return -1;
    return e[0] == '1' ? 1 : 0;
}

struct SplitOperand {
    float* hi = nullptr;
    float* lo = nullptr;
    int64_t rows = 0, ldk = 0;
};

template <int BN, int STAGES>
int tc_gemm_run(ct_handle* h, const SplitOperand& A, const SplitOperand& B, int64_t M, int64_t N,
                const TcEpi& epi, const int* skip) {
    CUtensorMap ta_h, ta_l, tb_h, tb_l;
    CT_TRY(make_map(h, &ta_h, A.hi, A.rows, A.ldk, TC_BM));
    CT_TRY(make_map(h, &ta_l, A.lo, A.rows, A.ldk, TC_BM));
    CT_TRY(make_map(h, &tb_h, B.hi, B.rows, B.ldk, BN));
    CT_TRY(make_map(h, &tb_l, B.lo, B.rows, B.ldk, BN));
    using L = TcSmem<BN, STAGES>;
    static int attr_dev = -1;
    if (attr_dev != h->device) {
        CT_CUDA(h, cudaFuncSetAttribute(tc_gemm_kernel<BN, STAGES>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        L::TOTAL));
        CT_CUDA(h, cudaFuncSetAttribute(tc_gemm_persist_kernel<BN, STAGES>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, L::TOTAL));
        CT_CUDA(h, cudaFuncSetAttribute(tc_gemm_chunk_kernel<BN, STAGES>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, L::TOTAL));
        attr_dev = h->device;
    }
    const int64_t tiles = ct_cdiv(N, BN) * ct_cdiv(M, TC_BM);
    const int kc = tc_kchunk();
    if ((BN == 192 || BN == 224) && !(tc_use_persistent() && kc > 0 && !tc_use_stream_k())) {
        ct_seterr(h, "128 x 192 and 128 x 224 tiles exist only in the chunked kernel");
        return CT_ERR_UNSUPPORTED;
    }
    if (tc_use_persistent() && kc > 0 && !tc_use_stream_k()) {
        int64_t grid = tiles < h->num_sms ? tiles : h->num_sms;
        TcHybrid hy;
        if (!tc_plan_hybrid(tiles, h->num_sms, A.ldk / TC_BK, kc, hy) || h->no_alloc) {
            hy = TcHybrid{};
            hy.tiles_dp = (int)tiles;
            hy.maxp = 1;
        } else {
            const int64_t r = tiles - hy.tiles_dp;
            CT_TRY(tc_hybrid_scratch(h, r * hy.maxp * TC_BM * BN, r * 4 * tc_chunk_epw(BN)));
            if (++h->tc_hy_epoch == 0) h->tc_hy_epoch = 1;
            hy.epoch = h->tc_hy_epoch;
            hy.part = h->tc_hy_part;
            hy.cnt = h->tc_hy_cnt;
            grid = hy.tiles_dp > 0 ? h->num_sms : hy.gsk;
        }
        tc_gemm_chunk_kernel<BN, STAGES><<<(unsigned)grid, tc_chunk_threads(BN), L::TOTAL, h->stream>>>(
            ta_h, ta_l, tb_h, tb_l, (int)M, (int)N, (int)A.ldk, kc, epi, hy, skip, h->d_status);
        ct_note_launch();
    } else if (tc_use_persistent()) {
        const int64_t grid = tiles < h->num_sms ? tiles : h->num_sms;
        // stream-K when the tiles leave a partial last wave and every CTA's share
        // of k-blocks covers at least one whole tile (so a tile has at most two owners)
        const int64_t nkb = A.ldk / TC_BK;
        TcStreamK sk{};
        sk.total = tiles * nkb;
        const bool use_sk = tc_use_stream_k() && tiles > grid && (tiles % grid) != 0 && sk.total / grid >= nkb + 1;
        if (use_sk) {
            const size_t need = (size_t)grid * TC_BM * BN;
            if (h->tc_sk_floats < (int64_t)need) {
                if (h->tc_sk_part) cudaFree(h->tc_sk_part);
                if (h->tc_sk_flag) cudaFree(h->tc_sk_flag);
                h->tc_sk_part = nullptr;
                h->tc_sk_flag = nullptr;
                h->tc_sk_floats = 0;
                CT_CUDA(h, cudaMalloc((void**)&h->tc_sk_part, need * sizeof(float)));
                CT_CUDA(h, cudaMalloc((void**)&h->tc_sk_flag, (size_t)h->num_sms * 4 * sizeof(int)));
                h->tc_sk_floats = (int64_t)need;
            }
            CT_CUDA(h, cudaMemsetAsync(h->tc_sk_flag, 0, (size_t)grid * 4 * sizeof(int), h->stream));
            sk.part = h->tc_sk_part;
            sk.flag = h->tc_sk_flag;
        }
        tc_gemm_persist_kernel<BN, STAGES><<<(unsigned)grid, TC_THREADS, L::TOTAL, h->stream>>>(
            ta_h, ta_l, tb_h, tb_l, (int)M, (int)N, (int)A.ldk, epi, sk, use_sk ? 1 : 0, skip, h->d_status);
        ct_note_launch();
    } else {
        dim3 grid((unsigned)ct_cdiv(N, BN), (unsigned)ct_cdiv(M, TC_BM));
        if (grid.y > 65535) return CT_ERR_UNSUPPORTED;
        tc_gemm_kernel<BN, STAGES><<<grid, TC_THREADS, L::TOTAL, h->stream>>>(
            ta_h, ta_l, tb_h, tb_l, (int)M, (int)N, (int)A.ldk, epi, skip, h->d_status); ct_note_launch();
    }
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

// The launcher's choices for an M x N product over ldk (a multiple of 32): the tile width and
// whether to compute the transposed product C^T = B A^T (B's rows as the tile rows) when its
// tiles fill the waves better -- 4096 x 1024 x 5120 takes 128 tiles of 128 x 256 on 152 SMs,
// its transpose 1024 x 4096 takes 152 tiles of 128 x 224.  single_level: C's rows have one
// stride (the transposed epilogue's condition).
struct TcChoice {
    int bn = 128;
    bool trans = false;
    bool chunked = false;
};
TcChoice tc_choose(int num_sms, bool no_alloc, int64_t M, int64_t N, int64_t ldk, bool single_level) {
    TcChoice c;
    c.chunked = tc_use_persistent() && tc_kchunk() > 0 && !tc_use_stream_k();
    const int hkc = c.chunked && !no_alloc ? tc_kchunk() : 0;
    double cost = 0.0;
    c.bn = tc_pick_bn(M, N, ldk, num_sms, c.chunked, hkc, &cost);
    const int tmode = tc_trans_mode();
    if (c.chunked && single_level && (tmode == 1 || (tmode < 0 && !tc_bn_mode()))) {
        double cost_t = 0.0;
        const int bt = tc_pick_bn(N, M, ldk, num_sms, c.chunked, hkc, &cost_t);
        if (tmode == 1 || cost_t < 0.97 * cost) {
            c.bn = bt;
            c.trans = true;
        }
    }
    return c;
}

int tc_gemm_launch(ct_handle* h, const SplitOperand& A, const SplitOperand& B, int64_t M, int64_t N,
                   const TcEpi& epi, const int* skip) {
    if (A.ldk != B.ldk) return CT_ERR_SHAPE;
    if (M <= 0 || N <= 0) return CT_OK;
    if (M > (1ll << 31) || N > (1ll << 31)) return CT_ERR_UNSUPPORTED;
    TcEpi e = epi;
    {
        const int64_t per16 = e.out_fp64 ? 2 : 4;   // elements per 16 bytes
        e.vec = ((uintptr_t)e.C % 16 == 0) && e.sCm0 % per16 == 0 && (e.M0 >= M || e.sCm1 % per16 == 0);
    }
    int slot = -1;
    CT_TRY(ct_ktime_begin(h, KT_TC_GEMM, 2.0 * (double)M * (double)N * (double)A.ldk, &slot));
    const TcChoice ch = tc_choose(h->num_sms, h->no_alloc, M, N, A.ldk, e.M0 >= M);
    const int bn = ch.bn;
    const SplitOperand* opA = &A;
    const SplitOperand* opB = &B;
    int64_t Mr = M, Nr = N;
    if (ch.trans) {
        // the epilogue stores C^T's rows as C's columns
        e.trans = 1;
        e.vec = 0;
        opA = &B;
        opB = &A;
        Mr = N;
        Nr = M;
    }
    const int rc = bn == 256 ? tc_gemm_run<256, GEMM_STAGES_W>(h, *opA, *opB, Mr, Nr, e, skip)
                 : bn == 224 ? tc_gemm_run<224, GEMM_STAGES_W>(h, *opA, *opB, Mr, Nr, e, skip)
                 : bn == 192 ? tc_gemm_run<192, GEMM_STAGES_W>(h, *opA, *opB, Mr, Nr, e, skip)
                             : tc_gemm_run<128, GEMM_STAGES_N>(h, *opA, *opB, Mr, Nr, e, skip);
    CT_TRY(rc);
    CT_TRY(ct_ktime_end(h, slot));
    return CT_OK;
}

int pack_launch(ct_handle* h, const PackDesc& p, bool k_fast, const int* skip) {
    if (p.rows <= 0 || p.ldk <= 0) return CT_OK;
    dim3 grid((unsigned)ct_cdiv(p.ldk, 32), (unsigned)ct_cdiv(p.rows, 32));
    if (grid.y > 65535) return CT_ERR_UNSUPPORTED;
    dim3 block(32, 8);
    if (k_fast) { pack_split_kernel<true><<<grid, block, 0, h->stream>>>(p, skip); ct_note_launch(); }
    else { pack_split_kernel<false><<<grid, block, 0, h->stream>>>(p, skip); ct_note_launch(); }
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

// Plain 2-level-row, 1-level-k pack helper.
PackDesc pack_desc(const double* src, int64_t rows, int64_t R0, int64_t s_r1, int64_t s_r0, int64_t K, int64_t s_k,
                   const SplitOperand& dst) {
    PackDesc p{};
    p.src = src;
    p.rows = rows; p.R0 = R0; p.s_r1 = s_r1; p.s_r0 = s_r0;
    p.K1 = 1; p.K0 = K; p.K0p = dst.ldk; p.s_k1 = 0; p.s_k0 = s_k;
    p.hi = dst.hi; p.lo = dst.lo; p.ldk = dst.ldk;
    p.scale = 1.0; p.scale_ptr = nullptr;
    return p;
}

template <int JT>
int mpo_tc2_launch(ct_handle* h, const MpoTcDesc& m) {
    const size_t smem = (size_t)((m.K * JT + 3) & ~(int64_t)3) * sizeof(float) + JT * sizeof(int64_t);
    static int attr_dev = -1;
    if (attr_dev != h->device) {
        CT_CUDA(h, cudaFuncSetAttribute(mpo_tc2_kernel<JT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        96 * 1024));
        attr_dev = h->device;
    }
    dim3 grid((unsigned)ct_cdiv(m.I / 2, MPOT_NT), (unsigned)m.O, (unsigned)ct_cdiv(m.J, JT));
    mpo_tc2_kernel<JT><<<grid, MPOT_NT, smem, h->stream>>>(m); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

int mpo_tc_launch(ct_handle* h, const MpoTcDesc& m) {
    if (m.O <= 0 || m.I <= 0 || m.J <= 0) return CT_OK;
    // paired-column kernel when the layout allows float2 access and the weight
    // chunk fits (K x 32 floats within 96 KB)
    const bool even = m.sIi == 1 && m.sOi == 1 && (m.I % 2) == 0 && (m.sIo % 2) == 0 && (m.sIk % 2) == 0 &&
                      (m.sOo % 2) == 0 && (m.sOj1 % 2) == 0 && (m.sOj0 % 2) == 0 &&
                      (((uintptr_t)m.in | (uintptr_t)m.hi | (uintptr_t)m.lo) & 7) == 0;
    if (even && m.O <= 65535 && (size_t)m.K * 32 * sizeof(float) + 256 <= 96 * 1024) {
        if (m.J <= 8) return mpo_tc2_launch<8>(h, m);
        if (m.J <= 12) return mpo_tc2_launch<12>(h, m);
        if (m.J <= 16) return mpo_tc2_launch<16>(h, m);
        if (m.J <= 20) return mpo_tc2_launch<20>(h, m);
        if (m.J <= 24) return mpo_tc2_launch<24>(h, m);
        return mpo_tc2_launch<32>(h, m);
    }
    // the whole of Wt in shared memory when it fits in 96 KB, else chunks of rows
    constexpr size_t kBudget = 96 * 1024;
    const size_t per_row = (size_t)m.K * sizeof(float) + sizeof(int64_t);
    int64_t jch = m.J;
    if ((size_t)m.J * per_row + 8 > kBudget) {
        jch = (int64_t)((kBudget - 8) / per_row);
        if (jch >= MPOT_JC) jch -= jch % MPOT_JC;
        if (jch < 1) return CT_ERR_UNSUPPORTED;
    }
    const size_t smem = (size_t)((jch * m.K + 1) & ~(int64_t)1) * sizeof(float) + (size_t)jch * sizeof(int64_t);
    const int64_t nz = ct_cdiv(m.J, jch);
    if (m.O > 65535 || nz > 65535) return CT_ERR_UNSUPPORTED;
    static int attr_dev = -1;
    if (attr_dev != h->device) {
        CT_CUDA(h, cudaFuncSetAttribute(mpo_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBudget));
        attr_dev = h->device;
    }
    dim3 grid((unsigned)ct_cdiv(m.I, MPOT_NT), (unsigned)m.O, (unsigned)nz);
    mpo_tc_kernel<<<grid, MPOT_NT, smem, h->stream>>>(m, jch); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

SplitOperand take_split(Arena& ar, int64_t rows, int64_t ldk) {
    SplitOperand s;
    s.rows = rows;
    s.ldk = ldk;
    s.hi = ar.take<float>((size_t)(rows * ldk));
    s.lo = ar.take<float>((size_t)(rows * ldk));
    return s;
}
size_t split_bytes(int64_t rows, int64_t ldk) { return 2 * ct_bytes((size_t)(rows * ldk), 4); }

struct TcHeff {
    SplitOperand Lp;   // [wL*Dl][Dl_pad]
    SplitOperand R4;   // [Dr][wR*Dr_pad]
    SplitOperand th;   // [d*d*Dr][Dl_pad]
    SplitOperand A4;   // [Dl*d*d][wR*Dr_pad]
    float* T1 = nullptr;
    double* W12 = nullptr;
    int64_t Dl_pad = 0, Dr_pad = 0;
};

}  // namespace

// ---------------------------------------------------------------------------
// entry points used by ct_ops.cu / ct_api.cu
// ---------------------------------------------------------------------------
int ct_tc_available(ct_handle* h) {
    if (!h->tc_checked) {
        h->tc_checked = true;
        int major = 0, minor = 0;
        cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, h->device);
        cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, h->device);
        h->tc_ok = (major == 10 && minor == 3) && get_encoder();
    }
    return h->tc_ok ? 1 : 0;
}

size_t ct_tc_heff_ws_bytes(int64_t Dl, int64_t d, int64_t Dr, int64_t wL, int64_t wM, int64_t wR) {
    (void)wM;
    const int64_t Dlp = ct_round_up(Dl, TC_BK), Drp = ct_round_up(Dr, TC_BK);
    return split_bytes(wL * Dl, Dlp) + split_bytes(Dr, wR * Drp) + split_bytes(d * d * Dr, Dlp) +
           split_bytes(Dl * d * d, wR * Drp) + ct_bytes((size_t)(Dl * wL * d * d * Dr), 4) +
           ct_bytes((size_t)((d * d * wR) * (wL * d * d)), 8) + 256;
}

int ct_tc_heff_prepare(ct_handle* h, Arena& ar, HeffPlan& p) {
    static_assert(sizeof(TcHeff) <= sizeof(p.tc_store), "HeffPlan::tc_store too small");
    TcHeff& q = *new (p.tc_store) TcHeff();
    const int64_t Dl = p.Dl, d = p.d, Dr = p.Dr, wL = p.wL, wM = p.wM, wR = p.wR;
    q.Dl_pad = ct_round_up(Dl, TC_BK);
    q.Dr_pad = ct_round_up(Dr, TC_BK);
    q.Lp = take_split(ar, wL * Dl, q.Dl_pad);
    q.R4 = take_split(ar, Dr, wR * q.Dr_pad);
    q.th = take_split(ar, d * d * Dr, q.Dl_pad);
    q.A4 = take_split(ar, Dl * d * d, wR * q.Dr_pad);
    q.T1 = ar.take<float>((size_t)(Dl * wL * d * d * Dr));
    q.W12 = ar.take<double>((size_t)((d * d * wR) * (wL * d * d)));
    if (!q.Lp.lo || !q.R4.lo || !q.th.lo || !q.A4.lo || !q.T1 || !q.W12) return CT_ERR_OOM;
    CT_TRY(ct_build_w12(h, p.W1, p.W2, q.W12, wL, d, wM, wR));
    // L[wL, Dl, Dl'] -> Lp[(wL, Dl')][Dl]
    CT_TRY(pack_launch(h, pack_desc(p.L, wL * Dl, Dl, Dl * Dl, 1, Dl, Dl, q.Lp), false, nullptr));
    // R[wR, Dr, Dr'] -> R4[Dr'][(wR, Dr)] with per-wR padding
    {
        PackDesc pd{};
        pd.src = p.R;
        pd.rows = Dr; pd.R0 = Dr; pd.s_r1 = 0; pd.s_r0 = 1;
        pd.K1 = wR; pd.K0 = Dr; pd.K0p = q.Dr_pad; pd.s_k1 = Dr * Dr; pd.s_k0 = Dr;
        pd.hi = q.R4.hi; pd.lo = q.R4.lo; pd.ldk = wR * q.Dr_pad;
        pd.scale = 1.0;
        CT_TRY(pack_launch(h, pd, false, nullptr));
    }
    // padding columns of A4 are never written by the MPO leg: zero them once
    CT_CUDA(h, cudaMemsetAsync(q.A4.hi, 0, (size_t)(q.A4.rows * q.A4.ldk) * 4, h->stream));
    CT_CUDA(h, cudaMemsetAsync(q.A4.lo, 0, (size_t)(q.A4.rows * q.A4.ldk) * 4, h->stream));
    p.tc = &q;
    return CT_OK;
}

int ct_tc_heff_run(ct_handle* h, const HeffPlan& p, const double* theta, double* out, const int* skip) {
    const TcHeff& q = *(const TcHeff*)p.tc;
    const int64_t Dl = p.Dl, d = p.d, Dr = p.Dr, wL = p.wL, wR = p.wR;
    const int64_t n1 = d * d * Dr;
    // theta[Dl, n1] -> th[n1][Dl]
    CT_TRY(pack_launch(h, pack_desc(theta, n1, n1, 0, 1, Dl, n1, q.th), false, skip));
    {   // T1[Dl'][wL][n1] (fp32) = Lp . th^T
        TcEpi e{};
        e.C = q.T1; e.out_fp64 = 0; e.M0 = Dl; e.sCm1 = n1; e.sCm0 = wL * n1; e.alpha = 1.0; e.beta = 0.0;
        CT_TRY(tc_gemm_launch(h, q.Lp, q.th, wL * Dl, n1, e, skip));
    }
    {   // A4[(Dl' t1 t2)][(wR, Dr)] = W12 . T1
        MpoTcDesc m{};
        m.O = Dl; m.K = wL * d * d; m.J = d * d * wR; m.I = Dr;
        m.in = q.T1; m.sIo = wL * d * d * Dr; m.sIk = Dr; m.sIi = 1;
        const int64_t K4 = wR * q.Dr_pad;
        m.hi = q.A4.hi; m.lo = q.A4.lo; m.sOo = d * d * K4; m.sOi = 1; m.J0 = wR; m.sOj1 = K4; m.sOj0 = q.Dr_pad;
        m.Wt = q.W12; m.skip = skip;
        CT_TRY(mpo_tc_launch(h, m));
    }
    {   // out[(Dl' t1 t2)][Dr'] = A4 . R4^T  (fp64)
        TcEpi e{};
        e.C = out; e.out_fp64 = 1; e.M0 = Dl * d * d; e.sCm1 = 0; e.sCm0 = Dr; e.alpha = 1.0; e.beta = 0.0;
        CT_TRY(tc_gemm_launch(h, q.A4, q.R4, Dl * d * d, Dr, e, skip));
    }
    return CT_OK;
}

// One-site effective Hamiltonian (the local adjoint of the environment chain):
//   out[(Dl' s'), Dr'] = sum L[wl,Dl,Dl'] A[Dl,s,Dr] W[wl,s,s',wr] R[wr,Dr,Dr']
// the two-site apply's chain with one physical leg: L . A on the tensor cores,
// the MPO leg into split planes with per-wr padding, then . R.
size_t ct_tc_heff1_ws_bytes(int64_t Dl, int64_t d, int64_t Dr, int64_t wl, int64_t wr) {
    const int64_t Dlp = ct_round_up(Dl, TC_BK), Drp = ct_round_up(Dr, TC_BK);
    return split_bytes(wl * Dl, Dlp) + split_bytes(Dr, wr * Drp) + split_bytes(d * Dr, Dlp) +
           split_bytes(Dl * d, wr * Drp) + ct_bytes((size_t)(Dl * wl * d * Dr), 4) +
           ct_bytes((size_t)((d * wr) * (wl * d)), 8) + 1024;
}

int ct_tc_heff1_run(ct_handle* h, Arena& ar, const double* L, const double* A, const double* W, const double* R,
                    double* out, int64_t Dl, int64_t d, int64_t Dr, int64_t wl, int64_t wr) {
    const int64_t Dlp = ct_round_up(Dl, TC_BK), Drp = ct_round_up(Dr, TC_BK);
    const int64_t n1 = d * Dr, K4 = wr * Drp;
    SplitOperand Lp = take_split(ar, wl * Dl, Dlp);
    SplitOperand R4 = take_split(ar, Dr, K4);
    SplitOperand th = take_split(ar, n1, Dlp);
    SplitOperand A4 = take_split(ar, Dl * d, K4);
    float* T1 = ar.take<float>((size_t)(Dl * wl * n1));
    double* Wt = ar.take<double>((size_t)((d * wr) * (wl * d)));
    if (!Lp.lo || !R4.lo || !th.lo || !A4.lo || !T1 || !Wt) return CT_ERR_OOM;
    CT_TRY(ct_build_wt_left(h, W, Wt, wl, d, wr));
    // L[wl, Dl, Dl'] -> Lp[(wl, Dl')][Dl]
    CT_TRY(pack_launch(h, pack_desc(L, wl * Dl, Dl, Dl * Dl, 1, Dl, Dl, Lp), false, nullptr));
    {   // R[wr, Dr, Dr'] -> R4[Dr'][(wr, Dr)] with per-wr padding
        PackDesc pd{};
        pd.src = R;
        pd.rows = Dr; pd.R0 = Dr; pd.s_r1 = 0; pd.s_r0 = 1;
        pd.K1 = wr; pd.K0 = Dr; pd.K0p = Drp; pd.s_k1 = Dr * Dr; pd.s_k0 = Dr;
        pd.hi = R4.hi; pd.lo = R4.lo; pd.ldk = K4;
        pd.scale = 1.0;
        CT_TRY(pack_launch(h, pd, false, nullptr));
    }
    // A[Dl, (s Dr)] -> th[(s Dr)][Dl]
    CT_TRY(pack_launch(h, pack_desc(A, n1, n1, 0, 1, Dl, n1, th), false, nullptr));
    {   // T1[Dl'][wl][(s Dr)] (fp32) = Lp . th^T
        TcEpi e{};
        e.C = T1; e.out_fp64 = 0; e.M0 = Dl; e.sCm1 = n1; e.sCm0 = wl * n1; e.alpha = 1.0; e.beta = 0.0;
        CT_TRY(tc_gemm_launch(h, Lp, th, wl * Dl, n1, e, nullptr));
    }
    CT_CUDA(h, cudaMemsetAsync(A4.hi, 0, (size_t)(A4.rows * A4.ldk) * 4, h->stream));
    CT_CUDA(h, cudaMemsetAsync(A4.lo, 0, (size_t)(A4.rows * A4.ldk) * 4, h->stream));
    {   // A4[(Dl' s')][(wr, Dr)] = Wt . T1
        MpoTcDesc m{};
        m.O = Dl; m.K = wl * d; m.J = d * wr; m.I = Dr;
        m.in = T1; m.sIo = wl * d * Dr; m.sIk = Dr; m.sIi = 1;
        m.hi = A4.hi; m.lo = A4.lo; m.sOo = d * K4; m.sOi = 1; m.J0 = wr; m.sOj1 = K4; m.sOj0 = Drp;
        m.Wt = Wt;
        CT_TRY(mpo_tc_launch(h, m));
    }
    TcEpi e{};   // out[(Dl' s')][Dr'] = A4 . R4^T (fp64)
    e.C = out; e.out_fp64 = 1; e.M0 = Dl * d; e.sCm1 = 0; e.sCm0 = Dr; e.alpha = 1.0; e.beta = 0.0;
    return tc_gemm_launch(h, A4, R4, Dl * d, Dr, e, nullptr);
}

size_t ct_tc_env_ws_bytes(int64_t Dl, int64_t d, int64_t Dr, int64_t wL, int64_t wR) {
    const int64_t Dlp = ct_round_up(Dl, TC_BK), Drp = ct_round_up(Dr, TC_BK);
    const int64_t K3l = ct_round_up(Dl * d, TC_BK), K3r = ct_round_up(d * Dr, TC_BK);
    const size_t wt = ct_bytes((size_t)((wL * d) * (wR * d)), 8);
    const size_t left = split_bytes(wL * Dl, Dlp) + split_bytes(d * Dr, Dlp) +
                        ct_bytes((size_t)(Dl * wL * d * Dr), 4) + split_bytes(wR * Dr, K3l) + split_bytes(Dr, K3l) +
                        wt;
    const size_t right = split_bytes(wR * Dr, Drp) + split_bytes(d * Dl, Drp) +
                         ct_bytes((size_t)(Dr * wR * d * Dl), 4) + split_bytes(wL * Dl, K3r) +
                         split_bytes(Dl, K3r) + wt;
    return std::max(left, right) + 1024;
}

int ct_tc_env_left_run(ct_handle* h, Arena& ar, const double* Lp, const double* A, const double* W, double* Ln,
                       int64_t Dl, int64_t d, int64_t Dr, int64_t wL, int64_t wR) {
    const int64_t Dlp = ct_round_up(Dl, TC_BK);
    const int64_t K3 = ct_round_up(Dl * d, TC_BK);
    const int64_t n1 = d * Dr;
    SplitOperand La = take_split(ar, wL * Dl, Dlp);
    SplitOperand Ab = take_split(ar, n1, Dlp);
    float* T1 = ar.take<float>((size_t)(Dl * wL * n1));
    SplitOperand A3 = take_split(ar, wR * Dr, K3);
    SplitOperand B3 = take_split(ar, Dr, K3);
    double* Wt = ar.take<double>((size_t)((d * wR) * (wL * d)));
    if (!La.lo || !Ab.lo || !T1 || !A3.lo || !B3.lo || !Wt) return CT_ERR_OOM;
    CT_TRY(ct_build_wt_left(h, W, Wt, wL, d, wR));
    CT_TRY(pack_launch(h, pack_desc(Lp, wL * Dl, Dl, Dl * Dl, 1, Dl, Dl, La), false, nullptr));
    CT_TRY(pack_launch(h, pack_desc(A, n1, n1, 0, 1, Dl, n1, Ab), false, nullptr));
    {   // T1[Dl'][wL][(s Dr)]
        TcEpi e{};
        e.C = T1; e.out_fp64 = 0; e.M0 = Dl; e.sCm1 = n1; e.sCm0 = wL * n1; e.alpha = 1.0;
        CT_TRY(tc_gemm_launch(h, La, Ab, wL * Dl, n1, e, nullptr));
    }
    CT_CUDA(h, cudaMemsetAsync(A3.hi, 0, (size_t)(A3.rows * A3.ldk) * 4, h->stream));
    CT_CUDA(h, cudaMemsetAsync(A3.lo, 0, (size_t)(A3.rows * A3.ldk) * 4, h->stream));
    {   // A3[(wR Dr)][(Dl' s')] = Wt . T1
        MpoTcDesc m{};
        m.O = Dl; m.K = wL * d; m.J = d * wR; m.I = Dr;
        m.in = T1; m.sIo = wL * d * Dr; m.sIk = Dr; m.sIi = 1;
        m.hi = A3.hi; m.lo = A3.lo; m.sOo = d; m.sOi = K3; m.J0 = wR; m.sOj1 = 1; m.sOj0 = Dr * K3;
        m.Wt = Wt;
        CT_TRY(mpo_tc_launch(h, m));
    }
    // B3[Dr'][(Dl' s')] = A[Dl', s', Dr']
    CT_TRY(pack_launch(h, pack_desc(A, Dr, Dr, 0, 1, Dl * d, Dr, B3), false, nullptr));
    TcEpi e{};
    e.C = Ln; e.out_fp64 = 1; e.M0 = wR * Dr; e.sCm1 = 0; e.sCm0 = Dr; e.alpha = 1.0;
    return tc_gemm_launch(h, A3, B3, wR * Dr, Dr, e, nullptr);
}

int ct_tc_env_right_run(ct_handle* h, Arena& ar, const double* Rn, const double* A, const double* W, double* Rp,
                        int64_t Dl, int64_t d, int64_t Dr, int64_t wL, int64_t wR) {
    const int64_t Drp = ct_round_up(Dr, TC_BK);
    const int64_t K3 = ct_round_up(d * Dr, TC_BK);
    SplitOperand Ra = take_split(ar, wR * Dr, Drp);
    SplitOperand Ab = take_split(ar, d * Dl, Drp);
    float* T1 = ar.take<float>((size_t)(Dr * wR * d * Dl));
    SplitOperand A3 = take_split(ar, wL * Dl, K3);
    SplitOperand B3 = take_split(ar, Dl, K3);
    double* Wt = ar.take<double>((size_t)((wL * d) * (wR * d)));
    if (!Ra.lo || !Ab.lo || !T1 || !A3.lo || !B3.lo || !Wt) return CT_ERR_OOM;
    CT_TRY(ct_build_wt_right(h, W, Wt, wL, d, wR));
    // R[wR, Dr, Dr'] -> Ra[(wR, Dr')][Dr]
    CT_TRY(pack_launch(h, pack_desc(Rn, wR * Dr, Dr, Dr * Dr, 1, Dr, Dr, Ra), false, nullptr));
    // A[Dl, s, Dr] -> Ab[(s, Dl)][Dr]   (row n' = s*Dl + Dl_idx)
    CT_TRY(pack_launch(h, pack_desc(A, d * Dl, Dl, Dr, d * Dr, Dr, 1, Ab), true, nullptr));
    {   // T1[Dr'][wR][s][Dl]
        TcEpi e{};
        e.C = T1; e.out_fp64 = 0; e.M0 = Dr; e.sCm1 = d * Dl; e.sCm0 = wR * d * Dl; e.alpha = 1.0;
        CT_TRY(tc_gemm_launch(h, Ra, Ab, wR * Dr, d * Dl, e, nullptr));
    }
    CT_CUDA(h, cudaMemsetAsync(A3.hi, 0, (size_t)(A3.rows * A3.ldk) * 4, h->stream));
    CT_CUDA(h, cudaMemsetAsync(A3.lo, 0, (size_t)(A3.rows * A3.ldk) * 4, h->stream));
    {   // A3[(wL Dl)][(s' Dr')] = Wt . T1
        MpoTcDesc m{};
        m.O = Dr; m.K = wR * d; m.J = wL * d; m.I = Dl;
        m.in = T1; m.sIo = wR * d * Dl; m.sIk = Dl; m.sIi = 1;
        m.hi = A3.hi; m.lo = A3.lo; m.sOo = 1; m.sOi = K3; m.J0 = d; m.sOj1 = Dl * K3; m.sOj0 = Dr;
        m.Wt = Wt;
        CT_TRY(mpo_tc_launch(h, m));
    }
    // B3[Dl'][(s' Dr')] = A natural layout
    CT_TRY(pack_launch(h, pack_desc(A, Dl, Dl, 0, d * Dr, d * Dr, 1, B3), true, nullptr));
    TcEpi e{};
    e.C = Rp; e.out_fp64 = 1; e.M0 = wL * Dl; e.sCm1 = 0; e.sCm0 = Dl; e.alpha = 1.0;
    return tc_gemm_launch(h, A3, B3, wL * Dl, Dl, e, nullptr);
}

size_t ct_tc_gemm_ws_bytes(int64_t m, int64_t n, int64_t k) {
    const int64_t kp = ct_round_up(k, TC_BK);
    return split_bytes(m, kp) + split_bytes(n, kp) + 512;
}

int ct_tc_gemm(ct_handle* h, Arena& ar, int trans_a, int trans_b, int64_t m, int64_t n, int64_t k, double alpha,
               const double* A, int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc) {
    return ct_tc_gemm_ex(h, ar, trans_a, trans_b, m, n, k, alpha, A, lda, B, ldb, beta, C, 1, ldc);
}

int ct_tc_gemm_ex(ct_handle* h, Arena& ar, int trans_a, int trans_b, int64_t m, int64_t n, int64_t k, double alpha,
                  const double* A, int64_t lda, const double* B, int64_t ldb, double beta, void* C, int out_fp64,
                  int64_t ldc) {
    const int64_t kp = ct_round_up(k, TC_BK);
    SplitOperand a = take_split(ar, m, kp);
    SplitOperand b = take_split(ar, n, kp);
    if (!a.lo || !b.lo) return CT_ERR_OOM;
    // op(A)[i, p]: trans_a=0 -> A[i*lda + p] (k contiguous), 1 -> A[p*lda + i]
    CT_TRY(pack_launch(h, trans_a ? pack_desc(A, m, m, 0, 1, k, lda, a) : pack_desc(A, m, m, 0, lda, k, 1, a),
                       !trans_a, nullptr));
    // op(B)[p, j]: trans_b=0 -> B[p*ldb + j] -> rows j, k stride ldb; 1 -> B[j*ldb + p]
    CT_TRY(pack_launch(h, trans_b ? pack_desc(B, n, n, 0, ldb, k, 1, b) : pack_desc(B, n, n, 0, 1, k, ldb, b),
                       trans_b != 0, nullptr));
    TcEpi e{};
    e.C = C; e.out_fp64 = out_fp64; e.M0 = m; e.sCm1 = 0; e.sCm0 = ldc; e.alpha = alpha; e.beta = beta;
    return tc_gemm_launch(h, a, b, m, n, e, nullptr);
}

// The launcher's plan for a plain m x n x k TF32x3 product on num_sms SMs, host only (no
// device, no handle): out[0] tile width, [1] 1 when the transposed product runs, [2] tiles,
// [3] whole tiles of the hybrid schedule, [4] CTAs sharing the stream-K units (0: none),
// [5] stream-K units (k-blocks), [6] most pieces of a stream-K tile, [7] k-blocks per tile.
extern "C" CT_API int ct_tc_gemm_plan(int64_t m, int64_t n, int64_t k, int num_sms, int64_t* out) {
    if (!out || m <= 0 || n <= 0 || k <= 0 || num_sms <= 0) return CT_ERR_INVALID;
    const int64_t ldk = ct_round_up(k, TC_BK);
    const TcChoice c = tc_choose(num_sms, false, m, n, ldk, true);
    const int64_t Mr = c.trans ? n : m, Nr = c.trans ? m : n;
    const int64_t tiles = ct_cdiv(Nr, c.bn) * ct_cdiv(Mr, TC_BM);
    TcHybrid hy;
    if (!(c.chunked && tc_plan_hybrid(tiles, num_sms, ldk / TC_BK, tc_kchunk(), hy))) {
        hy = TcHybrid{};
        hy.tiles_dp = (int)tiles;
        hy.maxp = 1;
    }
    out[0] = c.bn;
    out[1] = c.trans ? 1 : 0;
    out[2] = tiles;
    out[3] = hy.tiles_dp;
    out[4] = hy.gsk;
    out[5] = hy.units;
    out[6] = hy.maxp;
    out[7] = ldk / TC_BK;
    return CT_OK;
}

// Times launches of the raw TF32x3 GEMM kernel (operands already split and
// resident) with CUDA events on the handle's stream.
extern "C" CT_API int ct_tc_gemm_time(ct_handle* h, int64_t m, int64_t n, int64_t k, int reps, double* ms_per_launch) {
    if (!h || !ms_per_launch || m <= 0 || n <= 0 || k <= 0 || reps <= 0) return CT_ERR_INVALID;
    if (!ct_tc_available(h)) return CT_ERR_UNSUPPORTED;
    const int64_t kp = ct_round_up(k, TC_BK);
    float* C = nullptr;
    CT_TRY(ct_reserve(h, split_bytes(m, kp) + split_bytes(n, kp) + ct_bytes((size_t)(m * n), 4) + 1024));
    Arena ar(h);
    SplitOperand a = take_split(ar, m, kp);
    SplitOperand b = take_split(ar, n, kp);
    C = ar.take<float>((size_t)(m * n));
    if (!a.lo || !b.lo || !C) return CT_ERR_OOM;
    CT_CUDA(h, cudaMemsetAsync(a.hi, 0, (size_t)(m * kp) * 4, h->stream));
    CT_CUDA(h, cudaMemsetAsync(a.lo, 0, (size_t)(m * kp) * 4, h->stream));
    CT_CUDA(h, cudaMemsetAsync(b.hi, 0, (size_t)(n * kp) * 4, h->stream));
    CT_CUDA(h, cudaMemsetAsync(b.lo, 0, (size_t)(n * kp) * 4, h->stream));
    TcEpi e{};
    e.C = C; e.out_fp64 = 0; e.M0 = m; e.sCm1 = 0; e.sCm0 = n; e.alpha = 1.0;
    for (int i = 0; i < 2; ++i) CT_TRY(tc_gemm_launch(h, a, b, m, n, e, nullptr));
    cudaEvent_t e0, e1;
    CT_CUDA(h, cudaEventCreate(&e0));
    CT_CUDA(h, cudaEventCreate(&e1));
    CT_CUDA(h, cudaEventRecord(e0, h->stream));
    for (int i = 0; i < reps; ++i) CT_TRY(tc_gemm_launch(h, a, b, m, n, e, nullptr));
    CT_CUDA(h, cudaEventRecord(e1, h->stream));
    CT_CUDA(h, cudaEventSynchronize(e1));
    float ms = 0.f;
    CT_CUDA(h, cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms_per_launch = (double)ms / reps;
    return CT_OK;
}

