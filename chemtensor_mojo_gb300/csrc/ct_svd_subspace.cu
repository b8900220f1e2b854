// Warm-started subspace split for the mixed form (large bonds, chi_max binding).
//
// When chi_max < min(m, n) and the discarded weight at chi_max exceeds
// eps_trunc, the reference rule keeps exactly chi_max states
// (dense_tensor.mojo:1528-1548), and the two-site split only needs an
// orthonormal basis of theta's dominant chi_max-dimensional singular subspace:
// any basis of that subspace gives the same MPS up to a gauge transformation
// on the new bond, and the reference's own SVD basis is one of them.
//
// Warm start.  The split at bond i alternates direction from one half-sweep to
// the next, and the basis that stays valid between two visits is the one on
// the far side of the bond just split:
//   * a left-to-right split of bond i keeps Q (c x m, rows over (a_{i-1}, s_i));
//     bond i-1's gauge does not change before the right-to-left visit of bond i;
//   * a right-to-left split keeps V (c x n, rows over (s_{i+1}, a_{i+1}));
//     bond i+1's gauge does not change before the next left-to-right visit.
// The next split of bond i starts from that basis X:
//   left-to-right:  Q = orth(X theta^T),  A = Q^T,  B = Q theta
//   right-to-left:  V = orth(X theta),    A = theta V^T,  B = V
// (optionally after power steps X <- orth(orth(X theta^T) theta)).
//
// orth() is CholeskyQR2 on row-normalised rows: G = Z Z^T, G = L L^T,
// Z <- L^{-1} Z in FP64, then a second pass on the nearly orthonormal rows Q.
// The second pass computes E = Q Q^T - I in FP64 and, when |E| <= 1e-4, applies
// the first-order inverse Cholesky factor of I + E instead of factorising it:
//   L = I + Phi(E) + O(E^2),  Phi(E) = strict_lower(E) + diag(E) / 2,
//   Q <- (I - Phi(E)) Q   (a TF32x3 GEMM: the correction is ~|E| small, so its
//                          rounding is ~1e-7 |E|; repeated once if |E| > 1e-7)
// which leaves |Q Q^T - I| = O(E^2) and keeps the triangular order.  Larger E
// takes the full Cholesky pass.  It is triangular (Gram-Schmidt order), so
// rows that start close to singular vectors ordered by weight stay ordered and
// close to them; a symmetric orthogonalisation would keep any rotation between
// the basis and the singular vectors and the next product X theta^T would
// become ill-conditioned.  The first pass must be FP64: a basis found by the
// FP32 Jacobi carries strong directions into its weak rows at the FP32 level,
// so rows of X theta^T for states near the cut are nearly parallel to the
// strong ones (first-pass pivots ~1e-6 measured at chi = 128); Gram-Schmidt
// in FP64 removes that, a TF32x3 Gram matrix cannot resolve it.
//
// The discarded weight is measured from the residual theta - A B (a
// tensor-core GEMM; the residual is orthogonal to the kept part, so the
// products' rounding enters only at second order).
//
// Rank completion (first visits only).  When theta's numerical rank is below
// c -- the first visit of a bond at a larger chi_max, where theta still
// carries the old bond's rank up to small Lanczos corrections -- rows of
// X theta^T have no direction left outside the rows before them.  With
// completion enabled, a first-pass pivot below MIN_PIVOT marks its row instead
// of failing (the row's factor entry becomes 1), the marked rows of the pass-1
// output are replaced by fresh Gaussian rows, and the second pass runs the full
// Cholesky.  The replacements stand in for directions that carry less than
// MIN_PIVOT of the row's weight; the discarded weight is still measured from
// the residual.
//
// The split is refused (the caller retries or falls back to the Jacobi SVD)
// when the Cholesky factorisation breaks down, when the discarded weight
// exceeds stale_mult x that of the previous visit of the bond plus stale_abs
// (the cached basis no longer tracks the dominant subspace), or when it is
// <= eps_trunc (then the rule may keep fewer states and needs the spectrum).
#include <stdlib.h>

#include "ct_ops.cuh"

namespace {

// Cholesky block.  A leaf factors and inverts one CH_NB x CH_NB block in one CTA
// (chol_diag_kernel).  32 x 32 leaves were measured slower overall (7.4 vs 6.4 ms
// per chi=1024 warm split, with the earlier three-barrier leaf): the extra
// recursion level's small products cost more than the leaves saved.
constexpr int CH_NB = 64;
constexpr int CH_THREADS = 288;      // leaf: 8 row warps and the pivot warp
constexpr int FL_CHOL_FAIL = 100;    // d_flags slot: non-positive pivot seen
constexpr int FL_DEF_COUNT = 101;    // d_flags slot: rows marked for replacement in a first pass
// smallest accepted Cholesky pivot of a first pass (the squared share of a
// normalised row outside the span of the rows before it)
constexpr double MIN_PIVOT = 1e-12;

// counter-based N(0,1) values: splitmix64 of (seed, index), Box-Muller
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ double randn_at(uint64_t seed, uint64_t t) {
    const uint64_t a = mix64(seed ^ mix64(t * 2)), b = mix64(seed ^ mix64(t * 2 + 1));
    const double u1 = ((double)(a >> 11) + 1.0) * (1.0 / 9007199254740993.0);   // (0, 1]
    const double u2 = (double)(b >> 11) * (1.0 / 9007199254740992.0);
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

// rows[k] (k < count) of Y (rows x len) <- Gaussian rows; one block per listed row
__global__ void replace_rows_kernel(double* Y, int64_t len, const int* rows, const int* count, int cap,
                                    uint64_t seed) {
    const int n = min(*count, cap);
    for (int k = blockIdx.x; k < n; k += gridDim.x) {
        const int64_t r = rows[k];
        for (int64_t i = threadIdx.x; i < len; i += blockDim.x)
            Y[r * len + i] = randn_at(seed, (uint64_t)(r * len + i));
    }
}

__global__ void row_normalize_kernel(double* Y, int64_t rows, int64_t len) {
    const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x & 31;
    if (r >= rows) return;
    double* y = Y + r * len;
    double a = 0.0;
    for (int64_t i = lane; i < len; i += 32) a = fma(y[i], y[i], a);
    a = ct_warp_sum(a);
    const double inv = (a > 0.0) ? 1.0 / sqrt(a) : 0.0;
    for (int64_t i = lane; i < len; i += 32) y[i] *= inv;
}

__global__ void transpose_copy_kernel(const double* src, int64_t rows, int64_t cols, double* dst) {
    // dst[c][r] = src[r][c]
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < rows * cols;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = t / cols, c = t % cols;
        dst[c * rows + r] = src[t];
    }
}

// G (cp x cp): the padding rows/columns >= c become the identity; Linv is cleared.
__global__ void chol_prepare_kernel(double* G, double* Linv, int64_t c, int64_t cp) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < cp * cp;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / cp, j = t % cp;
        if (i >= c || j >= c) G[t] = (i == j) ? 1.0 : 0.0;
        Linv[t] = 0.0;
    }
}

// 1/sqrt(p) in FP64 for finite p > 0, by Newton-Raphson on the reciprocal square root:
// p = m 2^(2k) with m in [1, 4), an FP32 estimate r of m^(-1/2) (~23 correct bits), then
// twice r <- r + (r/2) (1 - m r^2), each step doubling the correct bits (~46, then FP64
// rounding), and the result r 2^(-k).  The scalings by powers of two, the halving and the
// FP32 <-> FP64 conversions are exact operations on the exponent and mantissa fields,
// done with integer instructions: on this part FP64 issues at ~1/64 of the FP32 rate, the
// pivot is on the leaf's critical path, and it keeps 8 FP64 operations (the Newton steps
// and r^2, p r at the end).
__device__ __forceinline__ double chol_rsqrt(double p) {
    constexpr long long ONE_EXP = 1ll << 52;   // one unit of the FP64 exponent field
    int adj = 0;
    long long bits = __double_as_longlong(p);
    if ((bits >> 52) == 0) {   // subnormal: into the normal range, exactly
        p *= 18446744073709551616.0;   // 2^64
        adj = 32;
        bits = __double_as_longlong(p);
    }
    const int e = (int)((bits >> 52) & 0x7ff) - 1023;
    const int k = e >> 1;   // floor(e / 2)
    const long long mb = bits - (long long)(2 * k) * ONE_EXP;   // m = p 2^(-2k)
    const double m = __longlong_as_double(mb);
    const int em = (int)((mb >> 52) & 0x7ff) - 1023;            // 0 or 1
    const float mf = __int_as_float(((em + 127) << 23) | (int)((mb >> 29) & 0x7fffff));   // m, truncated
    const int rb = __float_as_int(rsqrtf(mf));
    double r = __longlong_as_double((long long)((rb >> 23) - 127 + 1023) * ONE_EXP +
                                    ((long long)(rb & 0x7fffff) << 29));
#pragma unroll
    for (int it = 0; it < 2; ++it) {
        const double h = __longlong_as_double(__double_as_longlong(r) - ONE_EXP);   // r / 2
        r = fma(h, fma(-(m * r), r, 1.0), r);
    }
    return __longlong_as_double(__double_as_longlong(r) + (long long)(adj - k) * ONE_EXP);
}

// Pivot j of the leaf (by one lane): the replacement rules, the running minimum (as
// the bit pattern: pivots are >= 0 when recorded, so the integer order is the order),
// then 1/p, sqrt(p) and 1/sqrt(p) for the step into pv[0..2].  The tests run on the
// bit pattern too (integer instructions instead of FP64 ones).
__device__ __forceinline__ void chol_pivot(double p, int j, double* pv, long long* mp, int* fail, int* defrows,
                                           int* defcount, int64_t row0, long long floor_bits) {
    const long long pb = __double_as_longlong(p);
    const bool finite = (pb & 0x7fffffffffffffffll) < 0x7ff0000000000000ll;
    // with floor > 0, a finite p is below it exactly when its bit pattern is (a negative
    // p or -0 reads as a negative integer)
    if (floor_bits > 0 && finite && pb < floor_bits) {
        // no direction left outside the rows before: mark the row for replacement
        const int k = atomicAdd(defcount, 1);
        defrows[k] = (int)(row0 + j);
        p = 1.0;
    } else if (!(finite && pb > 0)) {
        *fail = 1;
        p = 1.0;
        *mp = min(*mp, __double_as_longlong(1.0));
    } else {
        *mp = min(*mp, pb);
    }
    const double r = chol_rsqrt(p);
    pv[0] = r * r;
    pv[1] = p * r;
    pv[2] = r;
}

// Cholesky of the CH_NB x CH_NB block at G (lower triangle, trailing updates
// already applied) and the inverse of that factor, in FP64.  L goes back into
// G's block (zeros above the diagonal), L^{-1} into Linv's block.  A pivot that
// is not positive and finite is replaced by 1 and flagged; the smallest pivot
// goes to *minpiv (bit pattern, atomicMin; pivots are >= 0 when recorded).
//
// One elimination sweep builds both factors, one barrier per column.  Working
// row i holds, at step j, the inverse's row (unscaled: X = I eliminated) at
// positions k <= j and the trailing matrix's row at positions j < l <= i, so its
// update at step j is exactly i + 1 multiply-adds with f = a_ij / p_j:
//     R[i][k] -= f R[j][k]   (k < j)        R[i][j] = -f
//     R[i][l] -= f a_lj      (j < l <= i)
// where a_lj is column j of the trailing matrix, snapshotted when the step before
// finished it (col[], double-buffered).  Column j of L is a_ij / sqrt(p_j) (stored
// unscaled during the sweep, scaled once at the end), row j of L^{-1} is
// R[j][k] / sqrt(p_j) (R[j][j] = 1).  A ninth warp forms the next pivot at the start
// of each step, p_{j+1} = a_{j+1,j+1} - a_{j+1,j}^2 / p_j (the same arithmetic as the
// row update, whose owner leaves that element unwritten: nothing reads it again), and
// its 1/p, sqrt(p), 1/sqrt(p) (double-buffered), while warps 0..7 run the step's
// multiply-adds: the pivot chain is no longer behind any row's.  Warp w < 8 owns the
// rows i = w (mod 8), up to 8 per step, lane l the positions l and l + 32 of each; a
// warp loads all its rows before its multiply-adds, so their latencies overlap.
// On this part FP64 issues at ~1/64 of the FP32 rate: the sweep's cost is its FP64
// instruction count (about 2.8k warp-instructions of multiply-adds) and one barrier
// per column.
__global__ void __launch_bounds__(CH_THREADS) chol_diag_kernel(double* G, double* Linv, int64_t ld,
                                                        unsigned long long* minpiv, int* fail, int* defrows,
                                                        int* defcount, int64_t row0, double floor) {
    extern __shared__ __align__(16) unsigned char chol_smem_raw[];   // three CH_NB x (CH_NB + 1) tiles
    double(*R)[CH_NB + 1] = reinterpret_cast<double(*)[CH_NB + 1]>(chol_smem_raw);
    double(*Ls)[CH_NB + 1] = R + CH_NB;
    double(*Xs)[CH_NB + 1] = Ls + CH_NB;
    __shared__ double col[2][CH_NB];
    __shared__ double piv[2][3];
    __shared__ double dinv[CH_NB];
    __shared__ long long mp;
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const long long floor_bits = floor > 0.0 ? __double_as_longlong(floor) : 0ll;
    for (int e = t; e < CH_NB * CH_NB; e += blockDim.x) {
        const int i = e / CH_NB, j = e % CH_NB;
        const double g = (j <= i) ? G[i * ld + j] : 0.0;
        R[i][j] = g;
        Ls[i][j] = 0.0;
        Xs[i][j] = 0.0;
        if (j == 0) col[0][i] = g;
    }
    if (t == 0) {
        mp = __double_as_longlong(1.0e300);
        chol_pivot(G[0], 0, piv[0], &mp, fail, defrows, defcount, row0, floor_bits);
    }
    __syncthreads();
    const int k0 = lane, k1 = lane + 32;
    for (int j = 0; j < CH_NB; ++j) {
        const int b = j & 1;
        const double inv_p = piv[b][0];
        if (warp == 8) {
            // the pivot of step j + 1 from a_{j+1,j} and a_{j+1,j+1}, both final since step j - 1
            if (lane == 0 && j + 1 < CH_NB) {
                const double a = col[b][j + 1];
                const double v = fma(-(a * inv_p), a, R[j + 1][j + 1]);
                chol_pivot(v, j + 1, piv[b ^ 1], &mp, fail, defrows, defcount, row0, floor_bits);
            }
            __syncthreads();
            continue;
        }
        // this warp's rows i > j, i = warp (mod 8); lane q < 8 forms row q's multiplier and
        // keeps its entry of L's column j (unscaled)
        const int i0 = j + 1 + ((warp - (j + 1)) & 7);
        double fq = 0.0;
        {
            const int iq = i0 + 8 * lane;
            if (lane < 8 && iq < CH_NB) {
                const double a = col[b][iq];
                fq = a * inv_p;
                Ls[iq][j] = a;
            }
        }
        if (warp == (j & 7)) {
            // row j is final: its row of L^{-1} and the diagonal of L
            const double inv_d = piv[b][2];
            for (int k = lane; k <= j; k += 32) Xs[j][k] = (k == j ? 1.0 : R[j][k]) * inv_d;
            if (lane == 0) {
                Ls[j][j] = piv[b][1];
                dinv[j] = inv_d;
            }
        }
        // the sources of positions k0, k1 are the same for every row
        const double s0 = k0 == j ? 1.0 : (k0 < j ? R[j][k0] : col[b][k0]);
        const double s1 = k1 == j ? 1.0 : (k1 < j ? R[j][k1] : col[b][k1]);
        double base0[8], base1[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int i = i0 + 8 * q;
            base0[q] = (i < CH_NB && k0 <= i && k0 != j) ? R[i][k0] : 0.0;
            base1[q] = (i < CH_NB && k1 <= i && k1 != j) ? R[i][k1] : 0.0;
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int i = i0 + 8 * q;
            if (i >= CH_NB) break;   // warp-uniform
            const double f = __shfl_sync(0xffffffffu, fq, q);
            // (the next pivot's element, i == k == j + 1, is warp 8's)
            if (k0 <= i && !(i == j + 1 && k0 == j + 1)) {
                const double v = fma(-f, s0, base0[q]);
                R[i][k0] = v;
                if (k0 == j + 1) col[b ^ 1][i] = v;
            }
            if (i >= 32 && k1 <= i && !(i == j + 1 && k1 == j + 1)) {
                const double v = fma(-f, s1, base1[q]);
                R[i][k1] = v;
                if (k1 == j + 1) col[b ^ 1][i] = v;
            }
        }
        __syncthreads();
    }
    if (t == 0) atomicMin(minpiv, (unsigned long long)mp);
    for (int e = t; e < CH_NB * CH_NB; e += blockDim.x) {
        const int i = e / CH_NB, j = e % CH_NB;
        G[i * ld + j] = i > j ? Ls[i][j] * dinv[j] : Ls[i][j];
        Linv[i * ld + j] = Xs[i][j];
    }
}

__global__ void split_piv_set_kernel(unsigned long long* piv, double p) {
    if (threadIdx.x == 0) atomicMin(piv, (unsigned long long)__double_as_longlong(p < 0.0 ? 0.0 : p));
}

// running minima of the two passes' pivots start at 1e300; the failure flag at 0
__global__ void split_flags_init_kernel(unsigned long long* piv, int* fail) {
    if (threadIdx.x < 2) piv[threadIdx.x] = (unsigned long long)__double_as_longlong(1.0e300);
    if (threadIdx.x == 0) *fail = 0;
}

int grid_n(ct_handle* h, int64_t n) {
    int64_t g = ct_cdiv(n, 256);
    if (g > h->num_sms * 16) g = h->num_sms * 16;
    if (g < 1) g = 1;
    return (int)g;
}

GemmDesc gemm2d(int64_t M, int64_t N, int64_t K, const double* A, int64_t sAm, int64_t sAk, const double* B,
                int64_t sBk, int64_t sBn, double* C, int64_t sCm, double alpha, double beta) {
    GemmDesc g{};
    g.M = M; g.N = N; g.K = K;
    g.A = A; g.sAm = sAm; g.sAk = sAk;
    g.B = B; g.sBk = sBk; g.sBn = sBn;
    g.C = C; g.sCm = sCm; g.sCn = 1;
    g.alpha = alpha; g.beta = beta;
    g.nb1 = 1; g.nb0 = 1;
    return g;
}

// C = alpha A op(B) + beta C in FP64 for the factorisation (tri as in GemmDesc).  On the
// tensor cores, tri == 1 skips the tiles above the diagonal block and tri == 2 (lower-
// triangular A) runs over the whole K: the zeros of A's upper triangle add nothing.
int fac_gemm(ct_handle* h, int64_t M, int64_t N, int64_t K, const double* A, int64_t lda, const double* B,
             int64_t ldb, int trans_b, double* C, int64_t ldc, double alpha, double beta, int tri) {
    if (ct_fp64_tc_enabled(h, M, N, K))
        return ct_oz_gemm(h, M, N, K, A, lda, 1, B, trans_b ? ldb : 1, trans_b ? 1 : ldb, alpha, beta, C, ldc,
                          tri == 1);
    GemmDesc g = trans_b ? gemm2d(M, N, K, A, lda, 1, B, 1, ldb, C, ldc, alpha, beta)
                         : gemm2d(M, N, K, A, lda, 1, B, ldb, 1, C, ldc, alpha, beta);
    g.tri = tri;
    return ct_gemm_f64_launch(h, g);
}

// Recursive Cholesky G = L L^T of the n x n block at G (leading dimension ld,
// n a multiple of CH_NB; the upper triangle is not read) and the inverse of
// the factor into Linv (its upper triangle must be zero):
//   L11 = chol(G11);  L21 = G21 L11^{-T};  L22 = chol(G22 - L21 L21^T)
//   inv(L) = [inv(L11) 0; -inv(L22) L21 inv(L11)  inv(L22)]
// The large products run as whole FP64 GEMMs, the 64 x 64 leaves in one CTA.
// S is scratch of (n/2)^2 doubles; it is free again whenever a recursive
// call runs.
// Rows whose pivot falls below `floor` (> 0) are recorded in defrows (row0 is
// the global index of the block's first row) instead of failing.
struct CholMarks {
    int* rows = nullptr;
    int* count = nullptr;
    double floor = 0.0;
};

int chol_inv(ct_handle* h, double* G, double* Linv, int64_t ld, int64_t n, double* S,
             unsigned long long* d_minpiv, int* d_fail, const CholMarks& mk, int64_t row0) {
    if (n <= CH_NB) {
        constexpr int smem = 3 * CH_NB * (CH_NB + 1) * (int)sizeof(double);
        static int attr_dev = -1;
        if (attr_dev != h->device) {
            CT_CUDA(h, cudaFuncSetAttribute(chol_diag_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
            attr_dev = h->device;
        }
        chol_diag_kernel<<<1, CH_THREADS, smem, h->stream>>>(G, Linv, ld, d_minpiv, d_fail, mk.rows, mk.count, row0,
                                                      mk.rows ? mk.floor : 0.0);
        ct_note_launch();
        CT_LAUNCH_CHECK(h);
        return CT_OK;
    }
    const int64_t n1 = ct_round_up(n / 2, CH_NB), n2 = n - n1;
    double* G21 = G + n1 * ld;
    double* G22 = G21 + n1;
    double* I21 = Linv + n1 * ld;
    double* I22 = I21 + n1;
    CT_TRY(chol_inv(h, G, Linv, ld, n1, S, d_minpiv, d_fail, mk, row0));
    // L21 = G21 inv(L11)^T -> S -> G21
    CT_TRY(fac_gemm(h, n2, n1, n1, G21, ld, Linv, ld, 1, S, n1, 1.0, 0.0, 0));
    CT_CUDA(h, cudaMemcpy2DAsync(G21, (size_t)ld * 8, S, (size_t)n1 * 8, (size_t)n1 * 8, (size_t)n2,
                                 cudaMemcpyDeviceToDevice, h->stream));
    // G22 -= L21 L21^T (lower tiles only)
    CT_TRY(fac_gemm(h, n2, n2, n1, G21, ld, G21, ld, 1, G22, ld, -1.0, 1.0, 1));
    CT_TRY(chol_inv(h, G22, I22, ld, n2, S, d_minpiv, d_fail, mk, row0 + n1));
    // inv(L)21 = -inv(L22) (L21 inv(L11))
    CT_TRY(fac_gemm(h, n2, n1, n1, G21, ld, Linv, ld, 0, S, n1, 1.0, 0.0, 0));
    CT_TRY(fac_gemm(h, n2, n1, n2, I22, ld, S, n1, 0, I21, ld, -1.0, 0.0, 2));
    return CT_OK;
}

// F = -Phi(G - I) (see the header) from G's lower triangle, F c x c with leading
// dimension c; the largest |G - I| of the lower triangle -> *emax (bit pattern of
// a non-negative double, atomicMax; a NaN counts as 1e300).
__global__ void orth_correction_kernel(const double* G, int64_t ldg, int64_t c, double* F,
                                       unsigned long long* emax) {
    double m = 0.0;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < c * c;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / c, j = t % c;
        double f = 0.0;
        if (j <= i) {
            const double e = G[i * ldg + j] - (i == j ? 1.0 : 0.0);
            const double a = fabs(e);
            if (!(a <= m)) m = (a == a) ? a : 1.0e300;
            f = (i == j) ? -0.5 * e : -e;
        }
        F[t] = f;
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(emax, (unsigned long long)__double_as_longlong(m));
}

struct OrthBufs {
    double* G;      // cp x cp
    double* Linv;   // cp x cp
    double* S;      // (cp / 2)^2 + CH_NB^2
    int64_t cp;
    int* defrows;   // cp: rows marked by a first pass with completion
};

constexpr double ORTH_CORR_MAX = 1e-4;    // largest |Q Q^T - I| the first-order step takes
constexpr double ORTH_CORR_DONE = 1e-7;   // one step suffices below this (leaves ~E^2)

// Second pass by first-order correction: rows Q (c x len, nearly orthonormal)
// -> out.  *done is false (out untouched beyond scratch use) when |E| exceeds
// ORTH_CORR_MAX and the caller runs the Cholesky pass.  1 - |E| of the first
// step goes to *piv (the smallest pivot of a Cholesky pass is ~ 1 - |E|).
int orth_correct(ct_handle* h, Arena& ar, const double* Q, double* out, int64_t c, int64_t len, const OrthBufs& ob,
                 unsigned long long* piv, bool* done) {
    *done = false;
    const size_t mark = ar.off;
    unsigned long long* d_emax = (unsigned long long*)(h->d_scalars + SC_ORTH_EMAX);
    const double* cur = Q;
    for (int step = 0; step < 2; ++step) {
        CT_CUDA(h, cudaMemsetAsync(d_emax, 0, sizeof(unsigned long long), h->stream));
        CT_TRY(fac_gemm(h, c, c, len, cur, len, cur, len, 1, ob.G, ob.cp, 1.0, 0.0, 1));   // lower tiles of Q Q^T
        orth_correction_kernel<<<grid_n(h, c * c), 256, 0, h->stream>>>(ob.G, ob.cp, c, ob.Linv, d_emax);
        ct_note_launch();
        CT_LAUNCH_CHECK(h);
        unsigned long long bits = 0;
        CT_CUDA(h, cudaMemcpyAsync(&bits, d_emax, sizeof(bits), cudaMemcpyDeviceToHost, h->stream));
        CT_CUDA(h, cudaStreamSynchronize(h->stream));
        double emax;
        memcpy(&emax, &bits, sizeof(emax));
        if (step == 0) {
            if (!(emax <= ORTH_CORR_MAX)) return CT_OK;
            const double p = 1.0 - emax;
            split_piv_set_kernel<<<1, 32, 0, h->stream>>>(piv, p);
            ct_note_launch();
            CT_LAUNCH_CHECK(h);
        } else if (!(emax <= ORTH_CORR_MAX)) {
            return CT_OK;   // the step did not converge: Cholesky pass from Q
        }
        // out = cur + F cur   (out may alias cur only through the copy below)
        if (out != cur)
            CT_CUDA(h, cudaMemcpyAsync(out, cur, (size_t)(c * len) * sizeof(double), cudaMemcpyDeviceToDevice,
                                       h->stream));
        CT_TRY(ct_tc_gemm(h, ar, 0, 0, c, len, c, 1.0, ob.Linv, c, cur, len, 1.0, out, len));
        ar.off = mark;
        cur = out;
        if (emax <= ORTH_CORR_DONE) break;
    }
    *done = true;
    return CT_OK;
}

// Orthonormalise the c rows of Z (c x len) by CholeskyQR in FP64; the result
// goes to W (c x len) and Z is scratch.  The optional second pass makes the rows
// orthonormal to FP64 rounding.  Pivots of pass 1 go to d_minpiv[0], of pass 2
// to d_minpiv[1].
int orth_rows(ct_handle* h, Arena& ar, double* Z, double* W, int64_t c, int64_t len, const OrthBufs& ob,
              bool two_pass, unsigned long long* d_minpiv, int* d_fail, bool complete, uint64_t seed,
              int* replaced) {
    const int64_t cp = ob.cp;
    row_normalize_kernel<<<(unsigned)ct_cdiv(c * 32, 256), 256, 0, h->stream>>>(Z, c, len); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    double* src = Z;
    double* dst = W;
    int* d_count = h->d_flags + FL_DEF_COUNT;
    int nrep = 0;
    for (int pass = 0; pass < (two_pass ? 2 : 1); ++pass) {
        if (pass == 1 && nrep == 0) {
            bool done = false;
            CT_TRY(orth_correct(h, ar, src, dst, c, len, ob, d_minpiv + 1, &done));
            if (done) {
                src = dst;   // the corrected rows
                break;
            }
        }
        chol_prepare_kernel<<<grid_n(h, cp * cp), 256, 0, h->stream>>>(ob.G, ob.Linv, c, cp); ct_note_launch();
        CT_LAUNCH_CHECK(h);
        CT_TRY(fac_gemm(h, c, c, len, src, len, src, len, 1, ob.G, cp, 1.0, 0.0, 1));
        CholMarks mk;
        if (pass == 0 && complete) {
            CT_CUDA(h, cudaMemsetAsync(d_count, 0, sizeof(int), h->stream));
            mk.rows = ob.defrows;
            mk.count = d_count;
            mk.floor = MIN_PIVOT;
        }
        CT_TRY(chol_inv(h, ob.G, ob.Linv, cp, cp, ob.S, d_minpiv + pass, d_fail, mk, 0));
        CT_TRY(fac_gemm(h, c, len, c, ob.Linv, cp, src, len, 0, dst, len, 1.0, 0.0, 2));
        if (pass == 0 && complete) {
            CT_CUDA(h, cudaMemcpyAsync(&nrep, d_count, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
            CT_CUDA(h, cudaStreamSynchronize(h->stream));
            if (nrep > 0) {
                const unsigned g = (unsigned)std::min<int64_t>(nrep, (int64_t)h->num_sms * 4);
                replace_rows_kernel<<<g, 256, 0, h->stream>>>(dst, len, ob.defrows, d_count, (int)cp, seed);
                ct_note_launch();
                CT_LAUNCH_CHECK(h);
                row_normalize_kernel<<<(unsigned)ct_cdiv(c * 32, 256), 256, 0, h->stream>>>(dst, c, len);
                ct_note_launch();
                CT_LAUNCH_CHECK(h);
            }
        }
        double* t = src;
        src = dst;
        dst = t;
    }
    // the result is in src: W after one pass, Z after two
    if (src != W)
        CT_CUDA(h, cudaMemcpyAsync(W, src, (size_t)(c * len) * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    if (replaced) *replaced += nrep;
    (void)ar;
    return CT_OK;
}

}  // namespace

size_t ct_split_subspace_ws_bytes(int64_t m, int64_t n, int64_t c) {
    const int64_t big = m > n ? m : n;
    const int64_t cp = ct_round_up(c, CH_NB);
    size_t b = 2 * ct_bytes(c * big, 8) + 2 * ct_bytes(cp * cp, 8) + ct_bytes(cp * cp / 4 + CH_NB * CH_NB, 8) +
               ct_bytes(m * n, 8) + ct_bytes(cp, 4) + 4096;
    size_t g = ct_tc_gemm_ws_bytes(c, big, big);
    const size_t more[] = {ct_tc_gemm_ws_bytes(c, c, big), ct_tc_gemm_ws_bytes(big, c, big),
                           ct_tc_gemm_ws_bytes(c, big, c), ct_tc_gemm_ws_bytes(m, n, c),
                           ct_tc_gemm_ws_bytes(cp, cp, cp)};
    for (size_t x : more)
        if (x > g) g = x;
    return b + g;
}

namespace {

enum SplitVerdict { SPLIT_OK, SPLIT_BREAKDOWN, SPLIT_STALE, SPLIT_EPS };

struct SplitBufs {
    double* Z;
    double* W;
    double* R;
    OrthBufs ob;
};

// The warm split (products with theta on the tensor cores, orthonormalisation in FP64).
int split_attempt(ct_handle* h, Arena& ar, const SplitBufs& sb, const double* M, int64_t m, int64_t n, int64_t c,
                  int mode, const double* basis_in, double* basis_out, double* Aout, double* Bout,
                  const double* d_total, double eps_trunc, double disc_ref, double stale_mult, double stale_abs,
                  int power_steps, bool complete, uint64_t seed, SvdOut* out, SplitVerdict* verdict) {
    const size_t mark = ar.off;
    unsigned long long* d_piv = (unsigned long long*)(h->d_scalars + SC_SPLIT_PIV);   // [0] pass 1, [1] pass 2
    int* d_fail = h->d_flags + FL_CHOL_FAIL;
    double* Z = sb.Z;
    double* W = sb.W;
    const OrthBufs& ob = sb.ob;
    int replaced = 0;
    uint64_t call = 0;
    auto orth = [&](double* Zr, double* Wr, int64_t len, bool two) {
        return orth_rows(h, ar, Zr, Wr, c, len, ob, two, d_piv, d_fail, complete, seed + 0x9E37ull * ++call,
                         &replaced);
    };
    split_flags_init_kernel<<<1, 32, 0, h->stream>>>(d_piv, d_fail); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    // X: c rows over n (left-to-right) or over m (right-to-left).  The power
    // steps' intermediate bases need no second pass.
    const double* X = basis_in;
    for (int it = 0; it < power_steps; ++it) {
        if (mode == 0) {
            CT_TRY(ct_tc_gemm(h, ar, 0, 1, c, m, n, 1.0, X, n, M, n, 0.0, Z, m));   // X theta^T
            ar.off = mark;
            CT_TRY(orth(Z, W, m, false));
            CT_TRY(ct_tc_gemm(h, ar, 0, 0, c, n, m, 1.0, W, m, M, n, 0.0, Z, n));   // . theta
            ar.off = mark;
            CT_TRY(orth(Z, W, n, false));
        } else {
            CT_TRY(ct_tc_gemm(h, ar, 0, 0, c, n, m, 1.0, X, m, M, n, 0.0, Z, n));   // X theta
            ar.off = mark;
            CT_TRY(orth(Z, W, n, false));
            CT_TRY(ct_tc_gemm(h, ar, 0, 1, c, m, n, 1.0, W, n, M, n, 0.0, Z, m));   // . theta^T
            ar.off = mark;
            CT_TRY(orth(Z, W, m, false));
        }
        X = W;
    }
    if (mode == 0) {
        // Q = orth(X theta^T) -> basis_out; A = Q^T; B = Q theta
        CT_TRY(ct_tc_gemm(h, ar, 0, 1, c, m, n, 1.0, X, n, M, n, 0.0, Z, m));
        ar.off = mark;
        CT_TRY(orth(Z, basis_out, m, true));
        CT_TRY(ct_tc_gemm(h, ar, 0, 0, c, n, m, 1.0, basis_out, m, M, n, 0.0, Bout, n));
        ar.off = mark;
        transpose_copy_kernel<<<grid_n(h, c * m), 256, 0, h->stream>>>(basis_out, c, m, Aout); ct_note_launch();
        CT_LAUNCH_CHECK(h);
    } else {
        // V = orth(X theta) -> B and basis_out; A = theta V^T
        CT_TRY(ct_tc_gemm(h, ar, 0, 0, c, n, m, 1.0, X, m, M, n, 0.0, Z, n));
        ar.off = mark;
        CT_TRY(orth(Z, Bout, n, true));
        CT_CUDA(h, cudaMemcpyAsync(basis_out, Bout, (size_t)(c * n) * sizeof(double), cudaMemcpyDeviceToDevice,
                                   h->stream));
        CT_TRY(ct_tc_gemm(h, ar, 0, 1, m, c, n, 1.0, M, n, Bout, n, 0.0, Aout, c));
        ar.off = mark;
    }
    // discarded weight |theta - A B|^2
    CT_CUDA(h, cudaMemcpyAsync(sb.R, M, (size_t)(m * n) * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    CT_TRY(ct_tc_gemm(h, ar, 0, 0, m, n, c, -1.0, Aout, c, Bout, n, 1.0, sb.R, n));
    ar.off = mark;
    CT_TRY(ct_reduce_nrm2sq(h, m * n, sb.R, h->d_scalars + SC_TMP1, nullptr));
    double host[2];
    unsigned long long piv[2];
    int fail = 0;
    CT_CUDA(h, cudaMemcpyAsync(host, d_total, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CT_CUDA(h, cudaMemcpyAsync(host + 1, h->d_scalars + SC_TMP1, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CT_CUDA(h, cudaMemcpyAsync(piv, d_piv, sizeof(piv), cudaMemcpyDeviceToHost, h->stream));
    CT_CUDA(h, cudaMemcpyAsync(&fail, d_fail, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CT_CUDA(h, cudaStreamSynchronize(h->stream));
    double piv1, piv2;
    memcpy(&piv1, &piv[0], 8);
    memcpy(&piv2, &piv[1], 8);
    const double total = host[0], resid = host[1];
    const double disc = (total > 0.0) ? resid / total : 0.0;
    out->chi = c;
    out->sum_s2_all = total;
    out->sum_s2_kept = total - resid;
    out->min_pivot = piv1;
    out->min_pivot2 = piv2;
    out->chol_fail = fail;
    out->replaced = replaced;
    // a second pass over nearly orthonormal rows has pivots near 1; completed
    // rows are random and keep (len - c) / len of their weight outside the rest
    if (fail || !(piv1 >= MIN_PIVOT) || !(piv2 > (replaced ? 1e-3 : 0.5))) {
        *verdict = SPLIT_BREAKDOWN;
    } else if (disc_ref >= 0.0 && disc > stale_mult * disc_ref + stale_abs) {
        *verdict = SPLIT_STALE;   // more weight lost than at the previous visit of the bond allows
        out->stale = 1;
    } else if (eps_trunc > 0.0 && disc <= eps_trunc) {
        *verdict = SPLIT_EPS;     // eps binds: the rule may keep fewer states
    } else {
        *verdict = SPLIT_OK;
    }
    return CT_OK;
}

}  // namespace

int ct_split_subspace(ct_handle* h, Arena& ar, const double* M, int64_t m, int64_t n, int64_t c, int mode,
                      const double* basis_in, double* basis_out, double* Aout, double* Bout,
                      const double* d_total, double eps_trunc, double disc_ref, double stale_mult,
                      double stale_abs, int power_steps, bool complete, uint64_t seed, SvdOut* out,
                      bool* accepted) {
    *accepted = false;
    const int64_t big = m > n ? m : n;
    SplitBufs sb{};
    sb.ob.cp = ct_round_up(c, CH_NB);
    sb.Z = ar.take<double>(c * big);
    sb.W = ar.take<double>(c * big);
    sb.ob.G = ar.take<double>(sb.ob.cp * sb.ob.cp);
    sb.ob.Linv = ar.take<double>(sb.ob.cp * sb.ob.cp);
    sb.ob.S = ar.take<double>(sb.ob.cp * sb.ob.cp / 4 + CH_NB * CH_NB);
    sb.R = ar.take<double>(m * n);
    sb.ob.defrows = ar.take<int>(sb.ob.cp);
    if (!sb.Z || !sb.W || !sb.ob.G || !sb.ob.Linv || !sb.ob.S || !sb.R || !sb.ob.defrows) return CT_ERR_OOM;
    SplitVerdict v = SPLIT_BREAKDOWN;
    out->stale = 0;
    CT_TRY(split_attempt(h, ar, sb, M, m, n, c, mode, basis_in, basis_out, Aout, Bout, d_total, eps_trunc,
                         disc_ref, stale_mult, stale_abs, power_steps, complete, seed, out, &v));
    *accepted = (v == SPLIT_OK);
    return CT_OK;
}

// ---------------------------------------------------------------------------
// Thin QR on the device (dense_tensor_qr, dense_tensor.mojo:1333-1433): A[m,n]
// = Q[m,k] R[k,n], k = min(m,n), Q with orthonormal columns, R upper
// triangular (trapezoidal when n > m) with a non-negative diagonal -- LAPACK's
// Householder QR returns the same factors up to the signs of Q's columns and
// R's rows.  The first k columns of A, as rows, go through the FP64
// CholeskyQR of the subspace split with rank completion; R = Q^T A in FP64.
// A column whose part outside the columns before it is below 1e-6 of its
// norm (a first-pass pivot below 1e-12) gets a completed Q column inside the
// same Gram-Schmidt order, so the spans stay nested and R triangular: exactly
// dependent columns (zero, repeated, linear combinations) are reproduced to
// FP64 rounding, a nearly dependent one to its part below that threshold.
// ---------------------------------------------------------------------------
namespace {
// Z[j][i] = A[i][j], j < k  (the first k columns of A[m,n] as rows)
__global__ void cols_to_rows_kernel(const double* A, int64_t m, int64_t n, int64_t k, double* Z) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < k * m; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = t / m, i = t % m;
        Z[t] = A[i * n + j];
    }
}
// R[i][j] = 0 for j < i
__global__ void zero_strict_lower_kernel(double* R, int64_t k, int64_t n) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < k * n; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / n, j = t % n;
        if (j < i) R[t] = 0.0;
    }
}
}  // namespace

size_t ct_qr_ws_bytes(int64_t m, int64_t n) {
    const int64_t k = std::min(m, n), cp = ct_round_up(k, CH_NB);
    return 2 * ct_bytes(k * m, 8) + 2 * ct_bytes(cp * cp, 8) +
           ct_bytes(cp * cp / 4 + CH_NB * CH_NB, 8) + ct_bytes(cp, 4) + ct_tc_gemm_ws_bytes(k, m, k) + 4096;
}

int ct_qr_run(ct_handle* h, Arena& ar, const double* A, int64_t m, int64_t n, double* Q, double* R,
              int* completed) {
    const int64_t k = std::min(m, n);
    OrthBufs ob;
    ob.cp = ct_round_up(k, CH_NB);
    double* Z = ar.take<double>(k * m);
    double* W = ar.take<double>(k * m);
    ob.G = ar.take<double>(ob.cp * ob.cp);
    ob.Linv = ar.take<double>(ob.cp * ob.cp);
    ob.S = ar.take<double>(ob.cp * ob.cp / 4 + CH_NB * CH_NB);
    ob.defrows = ar.take<int>(ob.cp);
    if (!Z || !W || !ob.G || !ob.Linv || !ob.S || !ob.defrows) return CT_ERR_OOM;
    unsigned long long* d_piv = (unsigned long long*)(h->d_scalars + SC_SPLIT_PIV);
    int* d_fail = h->d_flags + FL_CHOL_FAIL;
    split_flags_init_kernel<<<1, 32, 0, h->stream>>>(d_piv, d_fail); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    cols_to_rows_kernel<<<grid_n(h, k * m), 256, 0, h->stream>>>(A, m, n, k, Z); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    int nrep = 0;
    CT_TRY(orth_rows(h, ar, Z, W, k, m, ob, true, d_piv, d_fail, true, 0x51ED270B0ull, &nrep));
    CT_TRY(fac_gemm(h, k, n, m, W, m, A, n, 0, R, n, 1.0, 0.0, 0));   // R = Q^T A
    transpose_copy_kernel<<<grid_n(h, k * m), 256, 0, h->stream>>>(W, k, m, Q); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    zero_strict_lower_kernel<<<grid_n(h, k * n), 256, 0, h->stream>>>(R, k, n); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    int fail = 0;
    CT_CUDA(h, cudaMemcpyAsync(&fail, d_fail, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CT_CUDA(h, cudaStreamSynchronize(h->stream));
    if (completed) *completed = nrep;
    if (fail) {
        ct_seterr(h, "ct_qr: the Cholesky factorisation met a non-finite pivot");
        return CT_ERR_NONFINITE;
    }
    return CT_OK;
}

namespace {
__global__ void randn_fill_kernel(double* X, int64_t n, uint64_t seed) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
        X[t] = randn_at(seed, (uint64_t)t);
}
}  // namespace

// Start basis for a first visit: the rows kept at a smaller chi (prev, c_prev
// rows of length len, may be null) followed by random Gaussian rows.
int ct_cold_basis(ct_handle* h, const double* prev, int64_t c_prev, int64_t c, int64_t len, uint64_t seed,
                  double* X) {
    if (c_prev > c) c_prev = c;
    if (prev && c_prev > 0)
        CT_CUDA(h, cudaMemcpyAsync(X, prev, (size_t)(c_prev * len) * sizeof(double), cudaMemcpyDeviceToDevice,
                                   h->stream));
    else
        c_prev = 0;
    const int64_t nr = (c - c_prev) * len;
    if (nr > 0) {
        randn_fill_kernel<<<grid_n(h, nr), 256, 0, h->stream>>>(X + c_prev * len, nr, seed); ct_note_launch();
        CT_LAUNCH_CHECK(h);
    }
    return CT_OK;
}

// Refresh a basis cache (c rows) from an exact split's outputs: the rows of
// A^T after a left-to-right split, the rows of B after a right-to-left one.
int ct_basis_from_split(ct_handle* h, int mode, const double* Aout, const double* Bout, int64_t m, int64_t n,
                        int64_t c, double* basis) {
    if (mode == 0) {
        transpose_copy_kernel<<<grid_n(h, m * c), 256, 0, h->stream>>>(Aout, m, c, basis); ct_note_launch();
        CT_LAUNCH_CHECK(h);
    } else {
        CT_CUDA(h, cudaMemcpyAsync(basis, Bout, (size_t)(c * n) * sizeof(double), cudaMemcpyDeviceToDevice,
                                   h->stream));
    }
    return CT_OK;
}
