// FP64 GEMM emulated on the BF16 tensor cores (error-free slicing).
//
// C[M,N] = alpha * sum_k A[m,k] B[n,k] + beta * C with FP64 A, B and C.  The
// scheme is Ozaki's error-free transformation of a matrix product into sums
// of products that low-precision units compute exactly (K. Ozaki, T. Ogita,
// S. Oishi, S. M. Rump, Numer. Algorithms 59:95-118, 2012), here on tcgen05
// kind::f16 with BF16 operands and FP32 accumulation in TMEM:
//
//   * every row of A and of B is scaled by a power of two 2^e so that its
//     entries satisfy |x| < 1, and cut into S = 8 slices of 7 bits with
//     round-to-nearest digits:  x = sum_s a_s 2^{-7s} + r,  a_1 in [-128, 128],
//     a_s in [-64, 64] for s > 1,  |r| <= 2^{-57}.  a_s 2^{-7s} is exact in
//     BF16 (8 significant bits, FP32's exponent range);
//   * a product of slices s and t is an integer times 2^{-7(s+t)}.  Summed over
//     512 of K, the products of one level l = s + t stay below 2^24 for l <= 6
//     (level 2: 2^14 per term; level 6: five pairs, at most 7 * 2^12 per term),
//     so an FP32 accumulator holds them exactly and the tensor core's truncating
//     adds lose nothing;
//   * levels 2..6 get one exact accumulator each; levels 7..9, at 2^{-35} and
//     below relative to level 2, share a sixth whose rounding stays below 2^{-53}
//     of the result; pairs with s + t > 9 (below 2^{-56}) are not formed.  36
//     BF16 products per FP64 product;
//   * per 512 of K the epilogue combines the six accumulators with error-free
//     FP32 two-sums into hi + lo and adds both to FP64 registers; the result is
//     scaled back by 2^{e_m + e_n} once per tile.  (7-bit slices and 512-wide
//     chunks, not 8-bit and 128: the epilogue's FP64 adds and conversions, at
//     1/64 of the FP32 rate, bound an 8-bit version -- FP64 pipe 59%, tensor pipe
//     22% in an ncu capture of a 1024 x 2048 x 1024 product.)
//
// Accuracy (NumPy model of exactly this arithmetic): |C - AB| <= 2.6e-15 |A||B|
// elementwise on graded data with entries spanning 1e-18 of the row maximum
// (2.5e-15 for a plain FP64 GEMM of the same data), 1.7e-16 on Gaussian data
// (1.1e-16); the largest level sum met was 8.1e5 against the 2^24 limit.
//
// Kernel: one CTA per SM walks 128 x 64 tiles (consecutive CTAs share the A
// rows, which stay in L2); warp 0 issues TMA loads (64-byte swizzle, 32 BF16
// of K per row, all 8 slices of A and of B per stage, 2 stages), one thread of
// warp 1 issues the 72 MMAs (M128 N64 K16) of a K-block, and 8 epilogue warps
// (two per TMEM lane quadrant, 32 columns each) read the six accumulators of a
// 512-wide chunk (384 TMEM columns, one buffer: the MMAs of the next chunk wait
// only for the reads, ~1 us against ~20 us of MMAs) and add them in FP64.
// (128 x 32 tiles with two TMEM buffers kept the tensor pipe at 24%: an N = 32
// MMA is too short to fill it, ncu showing its issue pipe 87% busy.)  Every
// wait is bounded (2 s), after which the kernel sets the status word, releases
// TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>

#include "ct_ops.cuh"
#include "ct_tc_ptx.cuh"

PFN_cuTensorMapEncodeTiled_v12000 ct_tma_encoder();

namespace {

constexpr int OZ_S = 8;                                  // slices per operand
constexpr int OZ_BITS = 7;                               // bits per slice
constexpr int OZ_MAXLEV = OZ_S + 1;                      // pairs s + t <= OZ_MAXLEV are formed
constexpr int OZ_EXACT = 6;                              // levels 2..OZ_EXACT accumulate exactly
constexpr int OZ_BM = 128;
constexpr int OZ_BN = 64;
constexpr int OZ_BK = 32;                                // BF16 of K per 64-byte row
constexpr int OZ_STAGES = 2;
constexpr int OZ_KCH = 16;                               // k-blocks per exact chunk (512 of K)
constexpr int OZ_G = OZ_EXACT;                           // groups: levels 2..6 and one for 7..9
constexpr int OZ_EPW = 2;                                // epilogue warps per lane quadrant
constexpr int OZ_HC = OZ_BN / OZ_EPW;                    // columns per epilogue thread
constexpr int OZ_HH = OZ_HC / 2;                         // ... handled in two halves
constexpr int OZ_THREADS = 32 * (2 + 4 * OZ_EPW);
constexpr int OZ_A_SLICE = OZ_BM * OZ_BK * 2;            // 8 KB
constexpr int OZ_B_SLICE = OZ_BN * OZ_BK * 2;            // 4 KB
constexpr int OZ_STAGE = OZ_S * (OZ_A_SLICE + OZ_B_SLICE);
constexpr int OZ_TILE_BYTES = OZ_STAGES * OZ_STAGE;
constexpr int OZ_SMEM = OZ_TILE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
constexpr int OZ_ACC_COLS = OZ_G * OZ_BN;                // TMEM columns per buffer
constexpr int OZ_NBUF = 1;                               // 6 groups x 64 columns fill 384 of 512
constexpr int OZ_TMEM_COLS = 512;                        // power of two >= OZ_NBUF * OZ_ACC_COLS
static_assert(OZ_NBUF * OZ_ACC_COLS <= OZ_TMEM_COLS, "TMEM budget");
static_assert(OZ_SMEM <= 227 * 1024, "shared memory budget");
static_assert(OZ_HH % 8 == 0, "epilogue loads 8 columns at a time");

// K-major operand, 64-byte swizzle: rows of 64 B, 8-row groups 512 B apart.
__device__ __forceinline__ uint64_t sw64_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;               // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(512 >> 4) << 32;      // stride byte offset: 8 rows x 64 B
    d |= (uint64_t)1 << 46;               // descriptor version
    d |= (uint64_t)4 << 61;               // SWIZZLE_64B
    return d;
}

// kind::f16 instruction descriptor: D f32, A and B bf16, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t dtm, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
        ::"r"(dtm), "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
        : "memory");
}

// s + e = a + b exactly (Knuth's two-sum, round-to-nearest FP32)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

struct OzEpi {
    double* C;       // row m at (m / M0) * s1 + (m % M0) * s0, columns contiguous
    int64_t M0, s1, s0;
    double alpha, beta;
    const int* ea;   // row exponents of A (M)
    const int* eb;   // row exponents of B (N)
};

__global__ void __launch_bounds__(OZ_THREADS, 1)
    oz_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int M, int N,
                   int Mp, int Np, int Kpad, int lower, OzEpi epi, int* status) {
    extern __shared__ uint8_t oz_smem_raw[];
    uint8_t* smem = oz_smem_raw + ((1024u - (smem_u32(oz_smem_raw) & 1023u)) & 1023u);
    uint64_t* full = (uint64_t*)(smem + OZ_TILE_BYTES);
    uint64_t* empty = full + OZ_STAGES;
    uint64_t* acc_full = empty + OZ_STAGES;
    uint64_t* acc_empty = acc_full + OZ_NBUF;
    uint32_t* tmem_slot = (uint32_t*)(acc_empty + OZ_NBUF);
    volatile int* abort_flag = (volatile int*)(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tiles_n = (N + OZ_BN - 1) / OZ_BN;
    const int tiles = tiles_n * ((M + OZ_BM - 1) / OZ_BM);
    const int nkb = Kpad / OZ_BK;
    const int c = blockIdx.x, G = gridDim.x;

    if (threadIdx.x == 0) {
        for (int s = 0; s < OZ_STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < OZ_NBUF; ++b) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], 4 * OZ_EPW);
        }
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"((uint32_t)OZ_TMEM_COLS)
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
            for (int t = c; t < tiles && ok; t += G) {
                const int m0 = (t / tiles_n) * OZ_BM, n0 = (t % tiles_n) * OZ_BN;
                if (lower && n0 >= m0 + OZ_BM) continue;
                for (int kb = 0; kb < nkb; ++kb, ++g) {
                    const int s = g % OZ_STAGES;
                    const uint32_t ph = (uint32_t)(g / OZ_STAGES) & 1u;
                    if (g >= OZ_STAGES && !mbar_wait(&empty[s], ph ^ 1u, abort_flag)) {
                        *abort_flag = 1;
                        ct_set_status(status, CT_ERR_CUDA);
                        ok = false;
                        break;
                    }
                    uint8_t* st = smem + s * OZ_STAGE;
                    mbar_expect_tx(&full[s], OZ_STAGE);
                    const int x = kb * OZ_BK;
#pragma unroll
                    for (int sl = 0; sl < OZ_S; ++sl) {
                        tma_load_2d(st + sl * OZ_A_SLICE, &tmA, x, sl * Mp + m0, &full[s]);
                        tma_load_2d(st + OZ_S * OZ_A_SLICE + sl * OZ_B_SLICE, &tmB, x, sl * Np + n0, &full[s]);
                    }
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = idesc_bf16(OZ_BM, OZ_BN);
            int g = 0, gc = 0;
            bool ok = true;
            for (int t = c; t < tiles && ok; t += G) {
                if (lower && (t % tiles_n) * OZ_BN >= (t / tiles_n) * OZ_BM + OZ_BM) continue;
                for (int kb0 = 0; kb0 < nkb && ok; kb0 += OZ_KCH, ++gc) {
                    const int b = gc % OZ_NBUF, u = gc / OZ_NBUF;
                    if (u > 0 && !mbar_wait(&acc_empty[b], (uint32_t)((u - 1) & 1), abort_flag)) {
                        *abort_flag = 1;
                        ct_set_status(status, CT_ERR_CUDA);
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t dt = tmem + (uint32_t)(b * OZ_ACC_COLS);
                    const int kb1 = kb0 + OZ_KCH < nkb ? kb0 + OZ_KCH : nkb;
                    for (int kb = kb0; kb < kb1; ++kb, ++g) {
                        const int s = g % OZ_STAGES;
                        const uint32_t ph = (uint32_t)(g / OZ_STAGES) & 1u;
                        if (!mbar_wait(&full[s], ph, abort_flag)) {
                            *abort_flag = 1;
                            ct_set_status(status, CT_ERR_CUDA);
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                        // descriptors built once per stage; every MMA adds a compile-time
                        // offset (in 16-byte units) to the start-address field
                        const uint32_t a0 = smem_u32(smem + s * OZ_STAGE);
                        const uint64_t da = sw64_desc(a0), db = sw64_desc(a0 + OZ_S * OZ_A_SLICE);
                        const uint32_t first = (kb == kb0) ? 1u : 0u;
#pragma unroll
                        for (int l = 2; l <= OZ_MAXLEV; ++l) {
                            const int grp = l <= OZ_EXACT ? l - 2 : OZ_G - 1;
                            const uint32_t d = dt + (uint32_t)(grp * OZ_BN);
                            // the group's first product in a chunk overwrites the accumulator
                            const int l0 = l <= OZ_EXACT ? l : OZ_EXACT + 1;
                            const int s_first = l0 - OZ_S > 1 ? l0 - OZ_S : 1;
#pragma unroll
                            for (int sa = 1; sa <= OZ_S; ++sa) {
                                const int tb = l - sa;
                                if (tb < 1 || tb > OZ_S) continue;
#pragma unroll
                                for (int kk = 0; kk < 2; ++kk) {
                                    const bool fresh = (l == l0 && sa == s_first && kk == 0);
                                    const uint32_t acc = fresh ? (first ^ 1u) : 1u;
                                    mma_bf16(d, da + (uint64_t)((((sa - 1) * OZ_A_SLICE) + kk * 32) >> 4),
                                             db + (uint64_t)((((tb - 1) * OZ_B_SLICE) + kk * 32) >> 4), idesc, acc);
                                }
                            }
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
        double acc[OZ_HC];
        int gc = 0;
        bool ok = true;
        for (int t = c; t < tiles && ok; t += G) {
            if (lower && (t % tiles_n) * OZ_BN >= (t / tiles_n) * OZ_BM + OZ_BM) continue;
#pragma unroll
            for (int j = 0; j < OZ_HC; ++j) acc[j] = 0.0;
            for (int kb0 = 0; kb0 < nkb; kb0 += OZ_KCH, ++gc) {
                const int b = gc % OZ_NBUF, u = gc / OZ_NBUF;
                if (!mbar_wait(&acc_full[b], (uint32_t)(u & 1), abort_flag)) {
                    *abort_flag = 1;
                    ct_set_status(status, CT_ERR_CUDA);
                    ok = false;
                    break;
                }
                __syncwarp();
                tc_fence_after();
                const uint32_t tq = tmem + (uint32_t)(b * OZ_ACC_COLS + hf * OZ_HC) + ((uint32_t)(q * 32) << 16);
                // this thread's OZ_HC columns in two halves; per half the six groups are
                // folded into hi + lo by two-sums, largest level first
#pragma unroll
                for (int half = 0; half < 2; ++half) {
                    float hi[OZ_HH], lo[OZ_HH];
#pragma unroll
                    for (int grp = 0; grp < OZ_G; ++grp) {
                        uint32_t v[OZ_HH];
#pragma unroll
                        for (int q8 = 0; q8 < OZ_HH; q8 += 8)
                            tmem_ld8_nowait(tq + (uint32_t)(grp * OZ_BN + half * OZ_HH + q8),
                                            *reinterpret_cast<uint32_t(*)[8]>(&v[q8]));
                        tmem_wait_ld();
#pragma unroll
                        for (int j = 0; j < OZ_HH; ++j) {
                            const float x = __uint_as_float(v[j]);
                            if (grp == 0) {
                                hi[j] = x;
                                lo[j] = 0.f;
                            } else {
                                float sm, e;
                                two_sum(hi[j], x, sm, e);
                                hi[j] = sm;
                                lo[j] = __fadd_rn(lo[j], e);
                            }
                        }
                    }
                    if (half == 1) {   // every column read: the MMAs may overwrite the buffer
                        tc_fence_before();
                        __syncwarp();
                        if (lane == 0) mbar_arrive(&acc_empty[b]);
                    }
#pragma unroll
                    for (int j = 0; j < OZ_HH; ++j) {
                        acc[half * OZ_HH + j] += (double)hi[j];
                        acc[half * OZ_HH + j] += (double)lo[j];
                    }
                }
            }
            if (!ok) break;
            const int m0 = (t / tiles_n) * OZ_BM;
            const int n0 = (t % tiles_n) * OZ_BN + hf * OZ_HC;
            const int64_t m = (int64_t)m0 + row;
            if (m >= M) continue;
            const int em = epi.ea[m];
            double* Cr = epi.C + (m / epi.M0) * epi.s1 + (m % epi.M0) * epi.s0;
#pragma unroll
            for (int j = 0; j < OZ_HC; ++j) {
                const int64_t n = (int64_t)n0 + j;
                if (n >= N) break;
                double r = epi.alpha * scalbn(acc[j], em + epi.eb[n]);
                if (epi.beta != 0.0) r = fma(epi.beta, Cr[n], r);
                Cr[n] = r;
            }
        }
    }
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)OZ_TMEM_COLS)
                     : "memory");
    }
}

// ---- operand slicing ------------------------------------------------------------
// Row r of an operand is x[r][k] = src[(r / R0) * s1 + (r % R0) * s0 + k * sk] for r < R,
// k < K; the slices are stored [S][Rp][ldk] as BF16 (rows R..Rp-1, columns K..ldk-1 zero).
struct OzSrc {
    const double* p;
    int64_t R, K, R0, s1, s0, sk;
    __host__ __device__ int64_t row(int64_t r) const { return (r / R0) * s1 + (r % R0) * s0; }
};

// ex[r]: 2^ex[r] > max_k |x[r][k]| >= 2^(ex[r] - 1); 0 for a zero row (and rows >= R).
// One warp per row; lanes stride over k.
__global__ void oz_rowexp_kernel(OzSrc a, int64_t Rp, int* ex) {
    const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x & 31;
    if (r >= Rp) return;
    double m = 0.0;
    if (r < a.R) {
        const double* x = a.p + a.row(r);
        for (int64_t k = lane; k < a.K; k += 32) m = fmax(m, fabs(x[k * a.sk]));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) {
        int e = 0;
        if (m > 0.0) frexp(m, &e);
        ex[r] = e;
    }
}

// 32 x 32 tiles through shared memory, the 32 row offsets of a tile computed once;
// K_FAST: source contiguous along k (read with threads along k), else along rows.
template <bool K_FAST>
__global__ void __launch_bounds__(256) oz_slice_kernel(OzSrc a, int64_t Rp, int64_t ldk, const int* ex,
                                                       __nv_bfloat16* out) {
    __shared__ double tile[32][33];
    __shared__ int64_t rbase[32];
    const int64_t r0 = (int64_t)blockIdx.y * 32, k0 = (int64_t)blockIdx.x * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    if (ty == 0) rbase[tx] = (r0 + tx < a.R) ? a.row(r0 + tx) : 0;
    __syncthreads();
    for (int dy = ty; dy < 32; dy += 8) {
        if (K_FAST) {
            const int64_t r = r0 + dy, k = k0 + tx;
            tile[dy][tx] = (r < a.R && k < a.K) ? a.p[rbase[dy] + k * a.sk] : 0.0;
        } else {
            const int64_t r = r0 + tx, k = k0 + dy;
            tile[tx][dy] = (r < a.R && k < a.K) ? a.p[rbase[tx] + k * a.sk] : 0.0;
        }
    }
    __syncthreads();
    // Digits from the bit pattern with integer arithmetic (FP64 issues at 1/64 of the
    // FP32 rate here): X = round(x * 2^56) with x = v 2^-e, |X| < 2^56, then balanced
    // base-2^7 digits, most significant first, d = round(Y / 2^k), Y -= d 2^k:
    // X = sum_s d_s 2^(56 - 7s) exactly, |d_1| <= 128, |d_s| <= 64 for s > 1.
    constexpr int FRAC = OZ_S * OZ_BITS;   // 56 fractional bits
    for (int dy = ty; dy < 32; dy += 8) {
        const int64_t r = r0 + dy, k = k0 + tx;
        if (r >= Rp || k >= ldk) continue;
        long long X = 0;
        const double v = (r < a.R) ? tile[dy][tx] : 0.0;
        if (v != 0.0) {
            const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
            int ev = (int)((bits >> 52) & 0x7FF);
            unsigned long long m = bits & ((1ull << 52) - 1);
            if (ev == 0) ev = 1;           // subnormal
            else m |= 1ull << 52;
            // v = m 2^(ev - 1075), so x 2^56 = m 2^sh with sh <= 3 (|x| < 1)
            const int sh = ev - 1075 - ex[r] + FRAC;
            unsigned long long u = 0;
            if (sh >= 0) u = m << sh;
            else if (sh > -63) u = (m + (1ull << (-sh - 1))) >> (-sh);
            X = (bits >> 63) ? -(long long)u : (long long)u;
        }
#pragma unroll
        for (int s = 0; s < OZ_S; ++s) {
            const int sh = FRAC - OZ_BITS * (s + 1);
            long long d;
            if (sh > 0) {
                d = (X + (1ll << (sh - 1))) >> sh;
                X -= d << sh;
            } else {
                d = X;
            }
            // d 2^(-7(s+1)) is exact in FP32 and in BF16
            out[((int64_t)s * Rp + r) * ldk + k] = __float2bfloat16_rn(__int2float_rn((int)d) *
                                                                       __int_as_float((127 - OZ_BITS * (s + 1)) << 23));
        }
    }
}

struct OzOperand {
    __nv_bfloat16* sl = nullptr;
    int* ex = nullptr;
    int64_t rows = 0, rows_p = 0, ldk = 0;
};

int oz_pack(ct_handle* h, const OzSrc& a, const OzOperand& op) {
    {
        const int64_t thr = op.rows_p * 32;
        oz_rowexp_kernel<<<(unsigned)ct_cdiv(thr, 256), 256, 0, h->stream>>>(a, op.rows_p, op.ex);
        ct_note_launch();
    }
    dim3 grid((unsigned)ct_cdiv(op.ldk, 32), (unsigned)ct_cdiv(op.rows_p, 32));
    if (grid.y > 65535) return CT_ERR_UNSUPPORTED;
    if (a.sk == 1) oz_slice_kernel<true><<<grid, dim3(32, 8), 0, h->stream>>>(a, op.rows_p, op.ldk, op.ex, op.sl);
    else oz_slice_kernel<false><<<grid, dim3(32, 8), 0, h->stream>>>(a, op.rows_p, op.ldk, op.ex, op.sl);
    ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

int oz_map(ct_handle* h, CUtensorMap* m, const OzOperand& op, int box_rows) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = ct_tma_encoder();
    if (!enc) {
        ct_seterr(h, "cuTensorMapEncodeTiled unavailable");
        return CT_ERR_UNSUPPORTED;
    }
    if (((uintptr_t)op.sl & 15) || (op.ldk % OZ_BK)) {
        ct_seterr(h, "TMA operand misaligned (base %p, ldk %lld)", (const void*)op.sl, (long long)op.ldk);
        return CT_ERR_INVALID;
    }
    cuuint64_t dims[2] = {(cuuint64_t)op.ldk, (cuuint64_t)(OZ_S * op.rows_p)};
    cuuint64_t strides[1] = {(cuuint64_t)(op.ldk * 2)};
    cuuint32_t box[2] = {(cuuint32_t)OZ_BK, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)op.sl, dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        ct_seterr(h, "cuTensorMapEncodeTiled failed (%d)", (int)r);
        return CT_ERR_CUDA;
    }
    return CT_OK;
}

void oz_dims(int64_t M, int64_t N, int64_t K, int64_t& Mp, int64_t& Np, int64_t& ldk) {
    Mp = ct_round_up(M, OZ_BM);
    Np = ct_round_up(N, OZ_BN);
    ldk = ct_round_up(K, OZ_BK);
}

}  // namespace

size_t ct_oz_gemm_ws_bytes(int64_t M, int64_t N, int64_t K) {
    int64_t Mp, Np, ldk;
    oz_dims(M, N, K, Mp, Np, ldk);
    return ct_bytes(OZ_S * Mp * ldk, 2) + ct_bytes(OZ_S * Np * ldk, 2) + ct_bytes(Mp, 4) + ct_bytes(Np, 4);
}

// The slices live in a handle-owned buffer (the callers inside the factorisation
// have no arena at hand); it grows, after a stream synchronisation, when a larger
// product appears, so steady-state calls allocate nothing.
static int oz_workspace(ct_handle* h, size_t bytes, void** ws) {
    if (h->oz_ws_bytes < bytes) {
        if (h->no_alloc) {
            ct_seterr(h, "FP64 tensor-core GEMM: workspace of %zu bytes not available without allocation", bytes);
            return CT_ERR_TOO_LARGE;
        }
        CT_CUDA(h, cudaStreamSynchronize(h->stream));
        if (h->oz_ws) cudaFree(h->oz_ws);
        h->oz_ws = nullptr;
        h->oz_ws_bytes = 0;
        CT_CUDA(h, cudaMalloc(&h->oz_ws, bytes));
        h->oz_ws_bytes = bytes;
    }
    *ws = h->oz_ws;
    return CT_OK;
}

// C(m,n) = alpha * sum_k A(m,k) B(n,k) + beta * C(m,n), FP64 in and out, products on the
// BF16 tensor cores; operands and C with two-level row indexing (OzMat, OzOut in
// ct_ops.cuh).  A Gram product (B the same matrix as A) slices its operand once.
// lower != 0 skips the 128 x 32 tiles strictly above the diagonal (their C is left
// untouched).
int ct_oz_gemm_ex(ct_handle* h, int64_t M, int64_t N, int64_t K, const OzMat& A, const OzMat& B, double alpha,
                  double beta, const OzOut& Cout, int lower) {
    if (M <= 0 || N <= 0) return CT_OK;
    if (!ct_tc_available(h)) {
        ct_seterr(h, "the FP64 tensor-core GEMM needs an sm_103 device");
        return CT_ERR_UNSUPPORTED;
    }
    int64_t Mp, Np, ldk;
    oz_dims(M, N, K > 0 ? K : 1, Mp, Np, ldk);
    const bool gram = (A.p == B.p && A.R0 == B.R0 && A.s1 == B.s1 && A.s0 == B.s0 && A.sk == B.sk && M == N);
    if (gram) Np = Mp;
    if (OZ_S * Mp > (1ll << 31) || OZ_S * Np > (1ll << 31) || ldk > (1ll << 31)) return CT_ERR_UNSUPPORTED;
    const size_t bytes = gram ? ct_bytes(OZ_S * Mp * ldk, 2) + ct_bytes(Mp, 4)
                              : ct_oz_gemm_ws_bytes(M, N, K > 0 ? K : 1);
    void* ws = nullptr;
    CT_TRY(oz_workspace(h, bytes, &ws));
    OzOperand a, b;
    a.rows = M; a.rows_p = Mp; a.ldk = ldk;
    uint8_t* p = (uint8_t*)ws;
    a.sl = (__nv_bfloat16*)p;
    p += ct_bytes(OZ_S * Mp * ldk, 2);
    if (gram) {
        a.ex = (int*)p;
        b = a;
    } else {
        b.rows = N; b.rows_p = Np; b.ldk = ldk;
        b.sl = (__nv_bfloat16*)p;
        p += ct_bytes(OZ_S * Np * ldk, 2);
        a.ex = (int*)p;
        p += ct_bytes(Mp, 4);
        b.ex = (int*)p;
    }
    OzSrc sa{A.p, M, K, A.R0 > 0 ? A.R0 : M, A.s1, A.s0, A.sk};
    CT_TRY(oz_pack(h, sa, a));
    if (!gram) {
        OzSrc sb{B.p, N, K, B.R0 > 0 ? B.R0 : N, B.s1, B.s0, B.sk};
        CT_TRY(oz_pack(h, sb, b));
    }
    CUtensorMap ta, tb;
    CT_TRY(oz_map(h, &ta, a, OZ_BM));
    CT_TRY(oz_map(h, &tb, b, OZ_BN));
    static int attr_dev = -1;
    if (attr_dev != h->device) {
        CT_CUDA(h, cudaFuncSetAttribute(oz_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, OZ_SMEM));
        attr_dev = h->device;
    }
    OzEpi e;
    e.C = Cout.p;
    e.M0 = Cout.M0 > 0 ? Cout.M0 : M;
    e.s1 = Cout.s1;
    e.s0 = Cout.s0;
    e.alpha = alpha;
    e.beta = beta;
    e.ea = a.ex;
    e.eb = b.ex;
    const int64_t tiles = ct_cdiv(N, OZ_BN) * ct_cdiv(M, OZ_BM);
    const int64_t grid = tiles < h->num_sms ? tiles : h->num_sms;
    int slot = -1;
    CT_TRY(ct_ktime_begin(h, KT_OZ_GEMM, 2.0 * (double)M * (double)N * (double)K, &slot));
    oz_gemm_kernel<<<(unsigned)grid, OZ_THREADS, OZ_SMEM, h->stream>>>(ta, tb, (int)M, (int)N, (int)Mp, (int)Np,
                                                                       (int)ldk, lower ? 1 : 0, e, h->d_status);
    ct_note_launch();
    CT_LAUNCH_CHECK(h);
    CT_TRY(ct_ktime_end(h, slot));
    return CT_OK;
}

int ct_oz_gemm(ct_handle* h, int64_t M, int64_t N, int64_t K, const double* A, int64_t a_sr, int64_t a_sk,
               const double* B, int64_t b_sr, int64_t b_sk, double alpha, double beta, double* C, int64_t ldc,
               int lower) {
    const OzMat a{A, M, 0, a_sr, a_sk};
    const OzMat b{B, N, 0, b_sr, b_sk};
    const OzOut c{C, M, 0, ldc};
    return ct_oz_gemm_ex(h, M, N, K, a, b, alpha, beta, c, lower);
}
