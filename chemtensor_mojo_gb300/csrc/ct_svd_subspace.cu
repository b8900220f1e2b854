// Warm-started subspace split for the mixed form (large bonds, chi_max binding).
//
// When chi_max < min(m, n) and the discarded weight at chi_max exceeds
// eps_trunc, the reference rule keeps exactly chi_max states
// (dense_tensor.mojo:1528-1548), and the two-site split only needs an
// orthonormal basis of theta's dominant chi_max-dimensional singular subspace:
// any basis of that subspace gives the same MPS up to a gauge transformation.
// From one sweep to the next that subspace moves little, so the basis kept at
// the same bond in the previous sweep is refined by power steps
//     U <- orth(theta theta^T U)          (left-to-right; theta^T theta for
//                                          right-to-left)
// on the tensor cores.  orth() normalises the rows of the power step, then
// runs Newton-Schulz steps Q <- Q - 1/2 (Q Q^T - I) Q.  Mixing between
// singular directions across the chi_max cut changes the truncation error
// only through (s_c^2 - s_{c+1}^2), which is why no separate eigensolve of
// the subspace is needed.  The last Newton-Schulz step takes its Gram matrix
// in FP64, so the canonical factor is orthonormal to FP64 accuracy.
//
// The split is refused (the caller falls back to the Jacobi SVD) when the
// cached basis is stale (normalised power step not close to orthogonal), or
// when the discarded weight at chi_max is <= eps_trunc (then the rule may keep
// fewer states and needs the spectrum).
#include "ct_ops.cuh"

namespace {

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

// G <- G - I, and max |G - I| into *maxdev (atomicMax on the bit pattern; values >= 0)
__global__ void gram_dev_kernel(double* G, int64_t c, unsigned long long* maxdev) {
    double mx = 0.0;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < c * c; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / c, j = t % c;
        double v = G[t];
        if (i == j) v -= 1.0;
        G[t] = v;
        mx = fmax(mx, fabs(v));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) atomicMax(maxdev, (unsigned long long)__double_as_longlong(mx));
}

__global__ void transpose_copy_kernel(const double* src, int64_t rows, int64_t cols, double* dst) {
    // dst[c][r] = src[r][c]
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < rows * cols;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = t / cols, c = t % cols;
        dst[c * rows + r] = src[t];
    }
}

int grid_n(ct_handle* h, int64_t n) {
    int64_t g = ct_cdiv(n, 256);
    if (g > h->num_sms * 16) g = h->num_sms * 16;
    if (g < 1) g = 1;
    return (int)g;
}

// One Newton-Schulz step on the rows of Q (c x len); Gram on the tensor cores or in FP64.
int ns_step(ct_handle* h, Arena& ar, double* Q, int64_t c, int64_t len, double* G, bool fp64_gram,
            unsigned long long* d_maxdev) {
    const size_t mark = ar.off;
    if (fp64_gram) {
        GemmDesc g{};
        g.M = c; g.N = c; g.K = len;
        g.A = Q; g.sAm = len; g.sAk = 1;
        g.B = Q; g.sBk = 1; g.sBn = len;
        g.C = G; g.sCm = c; g.sCn = 1;
        g.alpha = 1.0; g.beta = 0.0; g.nb1 = 1; g.nb0 = 1;
        CT_TRY(ct_gemm_f64_launch(h, g));
    } else {
        CT_TRY(ct_tc_gemm(h, ar, 0, 1, c, c, len, 1.0, Q, len, Q, len, 0.0, G, c));
        ar.off = mark;
    }
    gram_dev_kernel<<<grid_n(h, c * c), 256, 0, h->stream>>>(G, c, d_maxdev); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    CT_TRY(ct_tc_gemm(h, ar, 0, 0, c, len, c, -0.5, G, c, Q, len, 1.0, Q, len));
    ar.off = mark;
    return CT_OK;
}

}  // namespace

size_t ct_split_subspace_ws_bytes(int64_t m, int64_t n, int64_t c) {
    const int64_t big = m > n ? m : n;
    size_t b = 2 * ct_bytes(c * big, 8) + ct_bytes(c * c, 8) + 4096;
    size_t g = ct_tc_gemm_ws_bytes(c, big, big);
    const size_t g2 = ct_tc_gemm_ws_bytes(c, big, c);
    const size_t g3 = ct_tc_gemm_ws_bytes(big, c, big);
    if (g2 > g) g = g2;
    if (g3 > g) g = g3;
    return b + g;
}

int ct_split_subspace(ct_handle* h, Arena& ar, const double* M, int64_t m, int64_t n, int64_t c, int mode,
                      double* basis, double* Aout, double* Bout, const double* d_total, double eps_trunc,
                      int power_steps, SvdOut* out, bool* accepted) {
    *accepted = false;
    const int64_t nvec = mode ? n : m;
    double* Z = ar.take<double>(c * (m > n ? m : n));
    double* Y = ar.take<double>(c * (m > n ? m : n));
    double* G = ar.take<double>(c * c);
    if (!Z || !Y || !G) return CT_ERR_OOM;
    const size_t mark = ar.off;
    unsigned long long* d_dev = (unsigned long long*)(h->d_scalars + SC_MISC + 300);
    unsigned long long* d_dev_final = (unsigned long long*)(h->d_scalars + SC_MISC + 301);
    CT_CUDA(h, cudaMemsetAsync(d_dev, 0, 2 * sizeof(double), h->stream));
    double* Q = basis;
    for (int it = 0; it < power_steps; ++it) {
        double* src = (it == 0) ? Q : Y;
        if (mode == 0) {
            // Z = src . M (c x n);  Y = Z . M^T (c x m)
            CT_TRY(ct_tc_gemm(h, ar, 0, 0, c, n, m, 1.0, src, m, M, n, 0.0, Z, n));
            ar.off = mark;
            CT_TRY(ct_tc_gemm(h, ar, 0, 1, c, m, n, 1.0, Z, n, M, n, 0.0, Y, m));
        } else {
            // Z = src . M^T (c x m);  Y = Z . M (c x n)
            CT_TRY(ct_tc_gemm(h, ar, 0, 1, c, m, n, 1.0, src, n, M, n, 0.0, Z, m));
            ar.off = mark;
            CT_TRY(ct_tc_gemm(h, ar, 0, 0, c, n, m, 1.0, Z, m, M, n, 0.0, Y, n));
        }
        ar.off = mark;
        row_normalize_kernel<<<(unsigned)ct_cdiv(c * 32, 256), 256, 0, h->stream>>>(Y, c, nvec); ct_note_launch();
        CT_LAUNCH_CHECK(h);
        // the first Gram decides whether the cached basis was close to converged
        CT_TRY(ns_step(h, ar, Y, c, nvec, G, false, it == 0 ? d_dev : d_dev_final + 1));
        CT_TRY(ns_step(h, ar, Y, c, nvec, G, false, d_dev_final + 1));
    }
    // two steps with FP64 Gram matrices: 1e-6 -> 1e-12 -> FP64 rounding
    CT_TRY(ns_step(h, ar, Y, c, nvec, G, true, d_dev_final));
    CT_TRY(ns_step(h, ar, Y, c, nvec, G, true, d_dev_final + 1));
    CT_CUDA(h, cudaMemcpyAsync(basis, Y, (size_t)(c * nvec) * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    // outputs and the kept weight
    if (mode == 0) {
        CT_TRY(ct_tc_gemm(h, ar, 0, 0, c, n, m, 1.0, basis, m, M, n, 0.0, Bout, n));   // B = U^T theta
        ar.off = mark;
        transpose_copy_kernel<<<grid_n(h, c * m), 256, 0, h->stream>>>(basis, c, m, Aout); ct_note_launch();
        CT_LAUNCH_CHECK(h);
        CT_TRY(ct_reduce_nrm2sq(h, c * n, Bout, h->d_scalars + SC_TMP1, nullptr));
    } else {
        CT_TRY(ct_tc_gemm(h, ar, 0, 1, m, c, n, 1.0, M, n, basis, n, 0.0, Aout, c));   // A = theta V
        ar.off = mark;
        CT_CUDA(h, cudaMemcpyAsync(Bout, basis, (size_t)(c * n) * sizeof(double), cudaMemcpyDeviceToDevice,
                                   h->stream));
        CT_TRY(ct_reduce_nrm2sq(h, m * c, Aout, h->d_scalars + SC_TMP1, nullptr));
    }
    double host[3];
    unsigned long long devs[2];
    CT_CUDA(h, cudaMemcpyAsync(host, d_total, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CT_CUDA(h, cudaMemcpyAsync(host + 1, h->d_scalars + SC_TMP1, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CT_CUDA(h, cudaMemcpyAsync(devs, d_dev, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, h->stream));
    CT_CUDA(h, cudaStreamSynchronize(h->stream));
    double first_dev, final_dev;
    memcpy(&first_dev, &devs[0], 8);
    memcpy(&final_dev, &devs[1], 8);
    const double total = host[0], kept = host[1];
    const double disc = (total > 0.0) ? (total - kept) / total : 0.0;
    out->chi = c;
    out->sum_s2_all = total;
    out->sum_s2_kept = kept;
    // stale basis: the normalised power step was far from orthogonal, or the
    // final FP64 correction was not small
    if (!(first_dev < 0.5) || !(final_dev < 1e-3)) return CT_OK;
    // eps binds: the rule may keep fewer than chi_max states
    if (eps_trunc > 0.0 && disc <= eps_trunc) return CT_OK;
    *accepted = true;
    return CT_OK;
}

// Refresh a basis cache (c x nvec rows) from an exact split's outputs.
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
