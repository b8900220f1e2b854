// SVD split of the mixed-precision form.
//
// FP64 on GB300 issues at ~1/60 of the FP32 rate, and a one-sided Jacobi SVD
// of a 2048 x 2048 theta costs ~9 n^3 flops per sweep, so the FP64 Jacobi of
// ct_svd.cu is the bottleneck of a chi=1024 sweep.  The mixed form splits the
// work by what each quantity needs:
//
//   1. one-sided Jacobi in FP32 (rows for left-to-right, columns for
//      right-to-left), same round-robin schedule as ct_svd.cu: it finds the
//      dominant subspace to ~1e-6;
//   2. the kept candidates (top min(k, chi_max) by FP32 norm) of the
//      accumulated rotations are lifted to FP64 and re-orthonormalised by two
//      Newton-Schulz steps  Q <- Q - 1/2 (Q Q^T - I) Q  with the Gram matrix in
//      FP64 (the canonical factor must be orthonormal to FP64 accuracy: its
//      defect enters the next H_eff as a metric error, first order in energy);
//   3. the centre factor (S Vt or U S) is the projection of theta on that basis,
//      on the tensor cores (TF32x3) when chi = min(k, chi_max) is fixed -- an
//      error there only perturbs the next Lanczos start vector -- and in FP64
//      when eps_trunc can decide chi or the spectrum is returned;
//   4. singular values = FP64 norms of the projected rows/columns, descending;
//      chi by the reference rule with the total weight |theta|^2 in FP64.
//
// The projected weights are exact to second order in the FP32 Jacobi's angles
// (~1e-12 of |theta|^2 measured), which decides chi exactly only when the cut is
// far from eps_trunc.  So the split is handed to the FP64 Jacobi of ct_svd.cu
// (QR-preconditioned, ~11 sweeps) when the caller wants the spectrum, and when
// eps_trunc > 0 and the projected tail at chi = min(k, chi_max) is below
// 2 eps_trunc + 1e-9 of |theta|^2: then eps_trunc may decide chi, and the FP64
// split gives the reference's chi, spectrum and discarded weight.  Otherwise
// the exact tail exceeds eps_trunc as well, chi = min(k, chi_max) is the
// reference's, and the reported weights are those of the split returned.
#include "ct_ops.cuh"
#include "ct_jacobi_coop.cuh"

namespace {

constexpr int NT = 256;

__global__ void to_f32_kernel(const double* M, int64_t m, int64_t n, int cols, float* X, float* Q, int64_t nvec) {
    const int64_t len = cols ? m : n;
    const int64_t tot = nvec * len;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = t / len, e = t % len;
        X[t] = (float)(cols ? M[e * n + v] : M[v * n + e]);
    }
    const int64_t tq = nvec * nvec;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < tq; t += (int64_t)gridDim.x * blockDim.x)
        Q[t] = ((t / nvec) == (t % nvec)) ? 1.f : 0.f;
}

__global__ void norms32_kernel(const float* X, int64_t len, int64_t nvec, double* sig) {
    const int64_t v = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x & 31;
    if (v >= nvec) return;
    double a = 0.0;
    for (int64_t i = lane; i < len; i += 32) {
        const double u = X[v * len + i];
        a = fma(u, u, a);
    }
    a = ct_warp_sum(a);
    if (lane == 0) sig[v] = sqrt(a);
}

__global__ void rank_desc_kernel(const double* sig, int64_t n, int* perm) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const double sj = ct_rank_key(sig[j]);
    int64_t rank = 0;
    for (int64_t i = 0; i < n; ++i) {
        const double si = ct_rank_key(sig[i]);
        if (si > sj || (si == sj && i < j)) ++rank;
    }
    perm[rank] = (int)j;
}

// Qt[i][x] = (double) Q32[perm[i]][x]
__global__ void lift_kernel(const float* Q, int64_t nvec, const int* perm, int64_t c, double* Qt) {
    const int64_t tot = c * nvec;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / nvec, x = t % nvec;
        Qt[t] = (double)Q[(int64_t)perm[i] * nvec + x];
    }
}

__global__ void f32_to_f64_kernel(const float* a, double* b, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (double)a[i];
}

__global__ void sub_identity_kernel(double* G, int64_t c) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < c; i += (int64_t)gridDim.x * blockDim.x)
        G[i * c + i] -= 1.0;
}

// FP64 norms of the c projected vectors: rows of P[c][ld] (rows=1) or columns of P[len][c] (rows=0)
__global__ void proj_norms_kernel(const double* P, int64_t c, int64_t len, int rows, double* sig) {
    const int64_t v = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x & 31;
    if (v >= c) return;
    double a = 0.0;
    for (int64_t i = lane; i < len; i += 32) {
        const double u = rows ? P[v * len + i] : P[i * c + v];
        a = fma(u, u, a);
    }
    a = ct_warp_sum(a);
    if (lane == 0) sig[v] = sqrt(a);
}

// chi rule with the total weight |theta|^2 (dense_tensor.mojo:1528-1548)
__global__ void trunc_kernel(const double* sig, const int* perm, int64_t limit, int64_t k, double eps,
                             const double* total_p, double* scalars, int* flags) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const double total = *total_p;
    int64_t chi = limit;
    if (eps > 0.0 && k > 0) {
        if (total <= 0.0) {
            chi = 0;
        } else {
            double kept = 0.0;
            for (int64_t t = 1; t <= limit; ++t) {
                const double s = sig[perm[t - 1]];
                kept += s * s;
                if ((total - kept) / total <= eps) {
                    chi = t;
                    break;
                }
            }
        }
    }
    double kept_at = 0.0;
    for (int64_t i = 0; i < chi; ++i) {
        const double s = sig[perm[i]];
        kept_at += s * s;
    }
    flags[FL_CHI] = (int)chi;
    scalars[SC_TMP0] = total;
    scalars[SC_TMP1] = kept_at;
}

// mode 0: A = U = Qt^T cols, B = P rows ; mode 1: A = P cols (U S), B = Qt rows (Vt)
__global__ void gather_kernel(const double* Qt, int64_t nvec, const double* P, int64_t c, const int* perm,
                              const int* flags, const double* sig, int64_t m, int64_t n, int mode, double* A,
                              double* B, double* S) {
    const int64_t chi = flags[FL_CHI];
    const int64_t totA = m * chi;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < totA; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = t / chi, j = t % chi;
        const int64_t v = perm[j];
        A[t] = (mode == 0) ? Qt[v * nvec + r] : P[r * c + v];
    }
    const int64_t totB = chi * n;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < totB; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = t / n, x = t % n;
        const int64_t v = perm[j];
        B[t] = (mode == 0) ? P[v * n + x] : Qt[v * nvec + x];
    }
    if (S)
        for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < chi; t += (int64_t)gridDim.x * blockDim.x)
            S[t] = sig[perm[t]];
}

int grid_elems(ct_handle* h, int64_t n) {
    int64_t g = ct_cdiv(n, 256);
    if (g > h->num_sms * 16) g = h->num_sms * 16;
    if (g < 1) g = 1;
    return (int)g;
}

}  // namespace

size_t ct_svd_mixed_ws_bytes(int64_t m, int64_t n, int64_t chi_max, int mode) {
    const int cols = mode ? 1 : 0;
    const int64_t nvec = cols ? n : m, len = cols ? m : n;
    const int64_t k = m < n ? m : n;
    const int64_t c = k < chi_max ? k : chi_max;
    size_t b = ct_bytes(nvec * len, 4) + ct_bytes(nvec * nvec, 4) + ct_bytes(nvec, 8) + ct_bytes(nvec, 4);
    b += ct_bytes(c * nvec, 8) + ct_bytes(c * c, 8) + ct_bytes(c * (m > n ? m : n), 8) + ct_bytes(c, 8) +
         ct_bytes(c, 4) + ct_bytes(nvec * nvec, 8) + 4096;
    // tensor-core operand planes: Newton-Schulz (c x c by c x nvec) and projection
    const size_t ns = ct_tc_gemm_ws_bytes(c, nvec, c);
    const size_t pj = (mode == 0) ? ct_tc_gemm_ws_bytes(c, n, m) : ct_tc_gemm_ws_bytes(m, c, n);
    const size_t wm = (mode == 0) ? ct_tc_gemm_ws_bytes(nvec, n, m) : ct_tc_gemm_ws_bytes(nvec, m, n);
    size_t mx = ns > pj ? ns : pj;
    mx = mx > wm ? mx : wm;
    return b + mx;
}

int ct_svd_mixed_run(ct_handle* h, Arena& ar, const double* M, int64_t m, int64_t n, int64_t chi_max,
                     double eps_trunc, int mode, double* Aout, double* Bout, double* Sout, const double* d_total,
                     SvdOut* out, float* qcache, int warm) {
    const int cols = mode ? 1 : 0;
    const int64_t nvec = cols ? n : m, len = cols ? m : n;
    const int64_t k = m < n ? m : n;
    const int64_t c = k < chi_max ? k : chi_max;
    if (c <= 0) {
        out->chi = 0;
        return CT_OK;
    }
    if (Sout) return ct_svd_run(h, ar, M, m, n, chi_max, eps_trunc, mode, Aout, Bout, Sout, out);
    const size_t entry = ar.off;
    float* X = ar.take<float>(nvec * len);
    float* Q = ar.take<float>(nvec * nvec);
    double* sig32 = ar.take<double>(nvec);
    int* perm32 = ar.take<int>(nvec);
    double* Qt = ar.take<double>(c * nvec);
    double* G = ar.take<double>(c * c);
    double* Pj = ar.take<double>(c * (m > n ? m : n));
    double* sig = ar.take<double>(c);
    int* perm = ar.take<int>(c);
    if (!X || !Q || !sig32 || !perm32 || !Qt || !G || !Pj || !sig || !perm) return CT_ERR_OOM;
    const size_t mark = ar.off;

    if (warm && qcache) {
        // X0 = Qprev . M (rows) or Qprev . M^T (columns); Q0 = Qprev
        double* Qp64 = ar.take<double>(nvec * nvec);
        if (!Qp64) return CT_ERR_OOM;
        const size_t mark2 = ar.off;
        f32_to_f64_kernel<<<grid_elems(h, nvec * nvec), 256, 0, h->stream>>>(qcache, Qp64, nvec * nvec); ct_note_launch();
        CT_LAUNCH_CHECK(h);
        if (!cols) CT_TRY(ct_tc_gemm_ex(h, ar, 0, 0, nvec, n, m, 1.0, Qp64, nvec, M, n, 0.0, X, 0, n));
        else CT_TRY(ct_tc_gemm_ex(h, ar, 0, 1, nvec, m, n, 1.0, Qp64, nvec, M, n, 0.0, X, 0, m));
        ar.off = mark2;
        CT_CUDA(h, cudaMemcpyAsync(Q, qcache, (size_t)(nvec * nvec) * sizeof(float), cudaMemcpyDeviceToDevice,
                                   h->stream));
    } else {
        to_f32_kernel<<<grid_elems(h, nvec * (len > nvec ? len : nvec)), 256, 0, h->stream>>>(M, m, n, cols, X, Q, nvec); ct_note_launch();
        CT_LAUNCH_CHECK(h);
    }
    // 1. FP32 one-sided Jacobi
    if (nvec >= 2) {
        double* d_f2 = h->d_scalars + SC_SVD_FROB2;
        CT_TRY(ct_reduce_nrm2sq(h, m * n, M, d_f2, nullptr));
        CT_TRY(ct_jacobi::run<float>(h, X, len, Q, nvec, 1e-6, 1.4210854715202004e-14, d_f2, nullptr));
    }
    if (qcache)
        CT_CUDA(h, cudaMemcpyAsync(qcache, Q, (size_t)(nvec * nvec) * sizeof(float), cudaMemcpyDeviceToDevice,
                                   h->stream));
    norms32_kernel<<<(unsigned)ct_cdiv(nvec * 32, 256), 256, 0, h->stream>>>(X, len, nvec, sig32); ct_note_launch();
    rank_desc_kernel<<<(unsigned)ct_cdiv(nvec, 256), 256, 0, h->stream>>>(sig32, nvec, perm32); ct_note_launch();
    lift_kernel<<<grid_elems(h, c * nvec), 256, 0, h->stream>>>(Q, nvec, perm32, c, Qt); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    // 2. Newton-Schulz: Qt <- Qt - 1/2 (Qt Qt^T - I) Qt, Gram matrix in FP64
    for (int it = 0; it < 2; ++it) {
        GemmDesc g{};
        g.M = c; g.N = c; g.K = nvec;
        g.A = Qt; g.sAm = nvec; g.sAk = 1;
        g.B = Qt; g.sBk = 1; g.sBn = nvec;
        g.C = G; g.sCm = c; g.sCn = 1;
        g.alpha = 1.0; g.beta = 0.0; g.nb1 = 1; g.nb0 = 1;
        CT_TRY(ct_gemm_f64_launch(h, g));
        sub_identity_kernel<<<grid_elems(h, c), 256, 0, h->stream>>>(G, c); ct_note_launch();
        CT_LAUNCH_CHECK(h);
        ar.off = mark;
        CT_TRY(ct_tc_gemm(h, ar, 0, 0, c, nvec, c, -0.5, G, c, Qt, nvec, 1.0, Qt, nvec));
    }
    // 3. centre factor: on the tensor cores when only the kept subspace matters
    // (eps_trunc = 0: chi = min(k, chi_max)); in FP64 when eps_trunc > 0, where
    // the tail sums decide whether the FP64 split takes over.  The basis is
    // FP64-orthonormal and within ~1e-6 (angle) of the singular subspace, so the
    // weights it captures are exact to second order in that angle.
    ar.off = mark;
    const bool fp64_proj = eps_trunc > 0.0;
    if (mode == 0) {
        // Pj[c][n] = Qt[c][m] . M[m][n]
        if (fp64_proj) {
            GemmDesc g{};
            g.M = c; g.N = n; g.K = m;
            g.A = Qt; g.sAm = nvec; g.sAk = 1;
            g.B = M; g.sBk = n; g.sBn = 1;
            g.C = Pj; g.sCm = n; g.sCn = 1;
            g.alpha = 1.0; g.beta = 0.0; g.nb1 = 1; g.nb0 = 1;
            CT_TRY(ct_gemm_f64_launch(h, g));
        } else {
            CT_TRY(ct_tc_gemm(h, ar, 0, 0, c, n, m, 1.0, Qt, nvec, M, n, 0.0, Pj, n));
        }
        proj_norms_kernel<<<(unsigned)ct_cdiv(c * 32, 256), 256, 0, h->stream>>>(Pj, c, n, 1, sig); ct_note_launch();
    } else {
        // Pj[m][c] = M[m][n] . Qt[c][n]^T
        if (fp64_proj) {
            GemmDesc g{};
            g.M = m; g.N = c; g.K = n;
            g.A = M; g.sAm = n; g.sAk = 1;
            g.B = Qt; g.sBk = 1; g.sBn = nvec;
            g.C = Pj; g.sCm = c; g.sCn = 1;
            g.alpha = 1.0; g.beta = 0.0; g.nb1 = 1; g.nb0 = 1;
            CT_TRY(ct_gemm_f64_launch(h, g));
        } else {
            CT_TRY(ct_tc_gemm(h, ar, 0, 1, m, c, n, 1.0, M, n, Qt, nvec, 0.0, Pj, c));
        }
        proj_norms_kernel<<<(unsigned)ct_cdiv(c * 32, 256), 256, 0, h->stream>>>(Pj, c, m, 0, sig); ct_note_launch();
    }
    rank_desc_kernel<<<(unsigned)ct_cdiv(c, 256), 256, 0, h->stream>>>(sig, c, perm); ct_note_launch();
    trunc_kernel<<<1, 32, 0, h->stream>>>(sig, perm, c, k, eps_trunc, d_total, h->d_scalars, h->d_flags); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    int chi = 0;
    double sums[2];
    CT_CUDA(h, cudaMemcpyAsync(&chi, h->d_flags + FL_CHI, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CT_CUDA(h, cudaMemcpyAsync(sums, h->d_scalars + SC_TMP0, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CT_CUDA(h, cudaStreamSynchronize(h->stream));
    if (eps_trunc > 0.0 && sums[0] > 0.0 &&
        (chi < c || (sums[0] - sums[1]) / sums[0] <= 2.0 * eps_trunc + 1e-9)) {
        ar.off = entry;
        h->mixed_fp64_splits++;
        return ct_svd_run(h, ar, M, m, n, chi_max, eps_trunc, mode, Aout, Bout, Sout, out);
    }
    out->chi = chi;
    out->sum_s2_all = sums[0];
    out->sum_s2_kept = sums[1];
    if (chi > 0) {
        gather_kernel<<<grid_elems(h, (m > n ? m : n) * (int64_t)chi), 256, 0, h->stream>>>(
            Qt, nvec, Pj, c, perm, h->d_flags, sig, m, n, mode, Aout, Bout, Sout); ct_note_launch();
        CT_LAUNCH_CHECK(h);
    }
    return CT_OK;
}

size_t ct_split_ws_bytes(int prec, int64_t m, int64_t n, int64_t chi_max, int mode) {
    const size_t exact = ct_svd_ws_bytes(m, n, mode);
    if (prec == CT_PREC_TF32X3 && !ct_svd_is_small(m, n, mode)) {
        // the mixed split may hand over to the FP64 one (same arena, from its start)
        const size_t mixed = ct_svd_mixed_ws_bytes(m, n, chi_max, mode);
        return mixed > exact ? mixed : exact;
    }
    return exact;
}

int ct_split_run(ct_handle* h, Arena& ar, int prec, const double* M, int64_t m, int64_t n, int64_t chi_max,
                 double eps_trunc, int mode, double* A, double* B, double* S, const double* d_total, SvdOut* out,
                 float* qcache, int warm) {
    if (prec == CT_PREC_TF32X3 && !ct_svd_is_small(m, n, mode))
        return ct_svd_mixed_run(h, ar, M, m, n, chi_max, eps_trunc, mode, A, B, S, d_total, out, qcache, warm);
    return ct_svd_run(h, ar, M, m, n, chi_max, eps_trunc, mode, A, B, S, out);
}
