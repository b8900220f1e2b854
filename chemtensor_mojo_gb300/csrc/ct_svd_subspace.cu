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
// Z <- L^{-1} Z, twice.  It is triangular (Gram-Schmidt order), so rows that
// start close to singular vectors ordered by weight stay ordered and close to
// them; a symmetric orthogonalisation would keep any rotation between the
// basis and the singular vectors and the next product X theta^T would become
// ill-conditioned.  The first pass takes its Gram matrix and applies L^{-1} on
// the tensor cores; the second pass is FP64 throughout, so the canonical factor
// is orthonormal to FP64 rounding.
//
// The split is refused (the caller falls back to the Jacobi SVD) when a
// Cholesky pivot of the first pass is small (a row of X theta^T nearly in the
// span of the rows before it: the cached basis no longer tracks the subspace)
// or when the discarded weight at chi_max is <= eps_trunc (then the rule may
// keep fewer states and needs the spectrum).
#include "ct_ops.cuh"

namespace {

constexpr int CH_NB = 64;            // Cholesky block
constexpr int FL_CHOL_FAIL = 100;    // d_flags slot: non-positive pivot seen
constexpr double MIN_PIVOT = 0.25;   // squared share of a row outside the span of the rows before it

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

// Cholesky of the diagonal block [k0, k0 + CH_NB) of G (lower triangle, trailing
// updates already applied) and the inverse of that factor.  L goes back into
// G's block (zeros above the diagonal), L^{-1} into Linv's block.  A pivot that
// is not positive and finite is replaced by 1 and flagged; the smallest pivot
// goes to *minpiv (bit pattern, atomicMin; pivots are >= 0 when recorded).
__global__ void __launch_bounds__(256) chol_diag_kernel(double* G, double* Linv, int64_t ld, int64_t k0,
                                                        unsigned long long* minpiv, int* fail) {
    extern __shared__ double chol_smem[];   // two CH_NB x (CH_NB + 1) tiles
    double(*A)[CH_NB + 1] = reinterpret_cast<double(*)[CH_NB + 1]>(chol_smem);
    double(*X)[CH_NB + 1] = reinterpret_cast<double(*)[CH_NB + 1]>(chol_smem + CH_NB * (CH_NB + 1));
    __shared__ double dj;
    const int t = threadIdx.x;
    for (int e = t; e < CH_NB * CH_NB; e += blockDim.x) {
        const int i = e / CH_NB, j = e % CH_NB;
        A[i][j] = (j <= i) ? G[(k0 + i) * ld + k0 + j] : 0.0;
    }
    __syncthreads();
    double mp = 1.0e300;
    for (int j = 0; j < CH_NB; ++j) {
        if (t == 0) {
            double p = A[j][j];
            if (!(p > 0.0) || !isfinite(p)) {
                *fail = 1;
                p = 1.0;
            }
            mp = fmin(mp, p);
            dj = sqrt(p);
            A[j][j] = dj;
        }
        __syncthreads();
        for (int i = j + 1 + t; i < CH_NB; i += blockDim.x) A[i][j] /= dj;
        __syncthreads();
        const int r = CH_NB - j - 1;
        for (int e = t; e < r * r; e += blockDim.x) {
            const int i = j + 1 + e / r, l = j + 1 + e % r;
            if (l <= i) A[i][l] = fma(-A[i][j], A[l][j], A[i][l]);
        }
        __syncthreads();
    }
    if (t == 0) atomicMin(minpiv, (unsigned long long)__double_as_longlong(mp));
    // column t of L^{-1} by forward substitution
    if (t < CH_NB) {
        for (int i = 0; i < CH_NB; ++i) X[i][t] = 0.0;
        for (int i = t; i < CH_NB; ++i) {
            double s = (i == t) ? 1.0 : 0.0;
            for (int l = t; l < i; ++l) s = fma(-A[i][l], X[l][t], s);
            X[i][t] = s / A[i][i];
        }
    }
    __syncthreads();
    for (int e = t; e < CH_NB * CH_NB; e += blockDim.x) {
        const int i = e / CH_NB, j = e % CH_NB;
        G[(k0 + i) * ld + k0 + j] = A[i][j];
        Linv[(k0 + i) * ld + k0 + j] = X[i][j];
    }
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

// Blocked right-looking Cholesky of G (cp x cp, cp a multiple of CH_NB, lower
// triangle meaningful) followed by the full inverse of the factor into Linv
// by recursive doubling: inv([A 0; B C]) = [A^-1 0; -C^-1 B A^-1  C^-1].
// P is scratch of cp * CH_NB doubles, T of cp * cp / 2 doubles.
int chol_and_inverse(ct_handle* h, double* G, double* Linv, int64_t cp, double* P, double* T,
                     unsigned long long* d_minpiv, int* d_fail) {
    constexpr int smem = 2 * CH_NB * (CH_NB + 1) * (int)sizeof(double);
    static int attr_dev = -1;
    if (attr_dev != h->device) {
        CT_CUDA(h, cudaFuncSetAttribute(chol_diag_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        attr_dev = h->device;
    }
    for (int64_t k0 = 0; k0 < cp; k0 += CH_NB) {
        chol_diag_kernel<<<1, 256, smem, h->stream>>>(G, Linv, cp, k0, d_minpiv, d_fail); ct_note_launch();
        CT_LAUNCH_CHECK(h);
        const int64_t r0 = k0 + CH_NB, rem = cp - r0;
        if (rem <= 0) break;
        // panel: L21 = G21 L11^{-T}
        CT_TRY(ct_gemm_f64_launch(h, gemm2d(rem, CH_NB, CH_NB, G + r0 * cp + k0, cp, 1, Linv + k0 * cp + k0, 1, cp,
                                            P, CH_NB, 1.0, 0.0)));
        CT_CUDA(h, cudaMemcpy2DAsync(G + r0 * cp + k0, (size_t)cp * 8, P, (size_t)CH_NB * 8, (size_t)CH_NB * 8,
                                     (size_t)rem, cudaMemcpyDeviceToDevice, h->stream));
        // trailing: G22 -= L21 L21^T (lower tiles only; the upper triangle is never read)
        GemmDesc gt = gemm2d(rem, rem, CH_NB, P, CH_NB, 1, P, 1, CH_NB, G + r0 * cp + r0, cp, -1.0, 1.0);
        gt.tri = 1;
        CT_TRY(ct_gemm_f64_launch(h, gt));
    }
    for (int64_t s = CH_NB; s < cp; s *= 2) {
        // pairs (A at r0, C at r0 + s); full pairs are batched, a short last pair runs alone
        const int64_t full = cp / (2 * s);
        const int64_t tail_r0 = full * 2 * s;
        const int64_t tail_b = (tail_r0 + s < cp) ? cp - tail_r0 - s : 0;
        for (int part = 0; part < 2; ++part) {
            const int64_t npairs = part == 0 ? full : (tail_b > 0 ? 1 : 0);
            if (npairs == 0) continue;
            const int64_t b = part == 0 ? s : tail_b;
            const int64_t r0 = part == 0 ? 0 : tail_r0;
            const int64_t step = 2 * s * (cp + 1);   // down the diagonal by 2s
            // T = L[r0+s.., r0..] * Linv[r0.., r0..]     (b x s x s)
            GemmDesc g1 = gemm2d(b, s, s, G + (r0 + s) * cp + r0, cp, 1, Linv + r0 * cp + r0, cp, 1, T, s, 1.0, 0.0);
            g1.nb0 = npairs; g1.sA0 = step; g1.sB0 = step; g1.sC0 = b * s;
            CT_TRY(ct_gemm_f64_launch(h, g1));
            // Linv[r0+s.., r0..] = -Linv[r0+s.., r0+s..] * T   (b x s x b)
            GemmDesc g2 = gemm2d(b, s, b, Linv + (r0 + s) * cp + r0 + s, cp, 1, T, s, 1, Linv + (r0 + s) * cp + r0,
                                 cp, -1.0, 0.0);
            g2.nb0 = npairs; g2.sA0 = step; g2.sB0 = b * s; g2.sC0 = step;
            g2.tri = 2;
            CT_TRY(ct_gemm_f64_launch(h, g2));
        }
    }
    return CT_OK;
}

struct OrthBufs {
    double* G;      // cp x cp
    double* Linv;   // cp x cp
    double* P;      // cp x CH_NB
    double* T;      // cp x cp / 2
    int64_t cp;
};

// Orthonormalise the c rows of Z (c x len) by CholeskyQR2; the result is
// written to W (c x len); Z is left row-normalised.  Pivots of the first pass
// go to d_minpiv[0], of the second to d_minpiv[1].
int orth_rows(ct_handle* h, Arena& ar, double* Z, double* W, int64_t c, int64_t len, const OrthBufs& ob,
              unsigned long long* d_minpiv, int* d_fail) {
    const size_t mark = ar.off;
    const int64_t cp = ob.cp;
    row_normalize_kernel<<<(unsigned)ct_cdiv(c * 32, 256), 256, 0, h->stream>>>(Z, c, len); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    // pass 1: Gram and L^{-1} Z on the tensor cores, factorisation in FP64
    chol_prepare_kernel<<<grid_n(h, cp * cp), 256, 0, h->stream>>>(ob.G, ob.Linv, c, cp); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    CT_TRY(ct_tc_gemm(h, ar, 0, 1, c, c, len, 1.0, Z, len, Z, len, 0.0, ob.G, cp));
    ar.off = mark;
    CT_TRY(chol_and_inverse(h, ob.G, ob.Linv, cp, ob.P, ob.T, d_minpiv, d_fail));
    CT_TRY(ct_tc_gemm(h, ar, 0, 0, c, len, c, 1.0, ob.Linv, cp, Z, len, 0.0, W, len));
    ar.off = mark;
    // pass 2: FP64 throughout
    chol_prepare_kernel<<<grid_n(h, cp * cp), 256, 0, h->stream>>>(ob.G, ob.Linv, c, cp); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    GemmDesc gg = gemm2d(c, c, len, W, len, 1, W, 1, len, ob.G, cp, 1.0, 0.0);
    gg.tri = 1;   // Cholesky reads the lower triangle only
    CT_TRY(ct_gemm_f64_launch(h, gg));
    CT_TRY(chol_and_inverse(h, ob.G, ob.Linv, cp, ob.P, ob.T, d_minpiv + 1, d_fail));
    GemmDesc ga = gemm2d(c, len, c, ob.Linv, cp, 1, W, len, 1, Z, len, 1.0, 0.0);
    ga.tri = 2;   // L^{-1} is lower triangular
    CT_TRY(ct_gemm_f64_launch(h, ga));
    CT_CUDA(h, cudaMemcpyAsync(W, Z, (size_t)(c * len) * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    return CT_OK;
}

}  // namespace

size_t ct_split_subspace_ws_bytes(int64_t m, int64_t n, int64_t c) {
    const int64_t big = m > n ? m : n;
    const int64_t cp = ct_round_up(c, CH_NB);
    size_t b = 2 * ct_bytes(c * big, 8) + 2 * ct_bytes(cp * cp, 8) + ct_bytes(cp * CH_NB, 8) +
               ct_bytes(cp * cp / 2 + CH_NB * CH_NB, 8) + 4096;
    size_t g = ct_tc_gemm_ws_bytes(c, big, big);
    const size_t g2 = ct_tc_gemm_ws_bytes(c, c, big);
    const size_t g3 = ct_tc_gemm_ws_bytes(big, c, big);
    const size_t g4 = ct_tc_gemm_ws_bytes(c, big, c);
    if (g2 > g) g = g2;
    if (g3 > g) g = g3;
    if (g4 > g) g = g4;
    return b + g;
}

int ct_split_subspace(ct_handle* h, Arena& ar, const double* M, int64_t m, int64_t n, int64_t c, int mode,
                      const double* basis_in, double* basis_out, double* Aout, double* Bout, const double* d_total,
                      double eps_trunc, int power_steps, SvdOut* out, bool* accepted) {
    *accepted = false;
    const int64_t big = m > n ? m : n;
    OrthBufs ob{};
    ob.cp = ct_round_up(c, CH_NB);
    double* Z = ar.take<double>(c * big);
    double* W = ar.take<double>(c * big);
    ob.G = ar.take<double>(ob.cp * ob.cp);
    ob.Linv = ar.take<double>(ob.cp * ob.cp);
    ob.P = ar.take<double>(ob.cp * CH_NB);
    ob.T = ar.take<double>(ob.cp * ob.cp / 2 + CH_NB * CH_NB);
    if (!Z || !W || !ob.G || !ob.Linv || !ob.P || !ob.T) return CT_ERR_OOM;
    const size_t mark = ar.off;
    unsigned long long* d_piv = (unsigned long long*)(h->d_scalars + SC_SPLIT_PIV);   // [0] pass 1, [1] pass 2
    int* d_fail = h->d_flags + FL_CHOL_FAIL;
    split_flags_init_kernel<<<1, 32, 0, h->stream>>>(d_piv, d_fail); ct_note_launch();
    CT_LAUNCH_CHECK(h);

    // X: c rows over n (left-to-right) or over m (right-to-left)
    const double* X = basis_in;
    for (int it = 0; it < power_steps; ++it) {
        if (mode == 0) {
            CT_TRY(ct_tc_gemm(h, ar, 0, 1, c, m, n, 1.0, X, n, M, n, 0.0, Z, m));   // X theta^T
            ar.off = mark;
            CT_TRY(orth_rows(h, ar, Z, W, c, m, ob, d_piv, d_fail));
            CT_TRY(ct_tc_gemm(h, ar, 0, 0, c, n, m, 1.0, W, m, M, n, 0.0, Z, n));   // . theta
            ar.off = mark;
            CT_TRY(orth_rows(h, ar, Z, W, c, n, ob, d_piv, d_fail));
        } else {
            CT_TRY(ct_tc_gemm(h, ar, 0, 0, c, n, m, 1.0, X, m, M, n, 0.0, Z, n));   // X theta
            ar.off = mark;
            CT_TRY(orth_rows(h, ar, Z, W, c, n, ob, d_piv, d_fail));
            CT_TRY(ct_tc_gemm(h, ar, 0, 1, c, m, n, 1.0, W, n, M, n, 0.0, Z, m));   // . theta^T
            ar.off = mark;
            CT_TRY(orth_rows(h, ar, Z, W, c, m, ob, d_piv, d_fail));
        }
        X = W;
    }
    if (mode == 0) {
        // Q = orth(X theta^T) -> basis_out; A = Q^T; B = Q theta
        CT_TRY(ct_tc_gemm(h, ar, 0, 1, c, m, n, 1.0, X, n, M, n, 0.0, Z, m));
        ar.off = mark;
        CT_TRY(orth_rows(h, ar, Z, basis_out, c, m, ob, d_piv, d_fail));
        CT_TRY(ct_tc_gemm(h, ar, 0, 0, c, n, m, 1.0, basis_out, m, M, n, 0.0, Bout, n));
        ar.off = mark;
        transpose_copy_kernel<<<grid_n(h, c * m), 256, 0, h->stream>>>(basis_out, c, m, Aout); ct_note_launch();
        CT_LAUNCH_CHECK(h);
        CT_TRY(ct_reduce_nrm2sq(h, c * n, Bout, h->d_scalars + SC_TMP1, nullptr));
    } else {
        // V = orth(X theta) -> B and basis_out; A = theta V^T
        CT_TRY(ct_tc_gemm(h, ar, 0, 0, c, n, m, 1.0, X, m, M, n, 0.0, Z, n));
        ar.off = mark;
        CT_TRY(orth_rows(h, ar, Z, Bout, c, n, ob, d_piv, d_fail));
        CT_CUDA(h, cudaMemcpyAsync(basis_out, Bout, (size_t)(c * n) * sizeof(double), cudaMemcpyDeviceToDevice,
                                   h->stream));
        CT_TRY(ct_tc_gemm(h, ar, 0, 1, m, c, n, 1.0, M, n, Bout, n, 0.0, Aout, c));
        ar.off = mark;
        CT_TRY(ct_reduce_nrm2sq(h, m * c, Aout, h->d_scalars + SC_TMP1, nullptr));
    }
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
    const double total = host[0], kept = host[1];
    const double disc = (total > 0.0) ? (total - kept) / total : 0.0;
    out->chi = c;
    out->sum_s2_all = total;
    out->sum_s2_kept = kept;
    out->min_pivot = piv1;
    out->min_pivot2 = piv2;
    out->chol_fail = fail;
    if (fail || !(piv1 >= MIN_PIVOT) || !(piv2 > 0.5)) return CT_OK;
    // eps binds: the rule may keep fewer than chi_max states
    if (eps_trunc > 0.0 && disc <= eps_trunc) return CT_OK;
    *accepted = true;
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
