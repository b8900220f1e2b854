// C ABI of libctdmrg (include/ctdmrg.h): handle lifecycle, scratch arena,
// argument validation, and the entry points that replace the reference's
// DenseTensor / environment / DMRG functions on the two-site DMRG path.
#include <stdarg.h>
#include <math.h>
#include <chrono>
#include <algorithm>

#include "ct_ops.cuh"

// ---------------------------------------------------------------------------
// errors, handle, arena
// ---------------------------------------------------------------------------
std::atomic<long long> g_ct_launches{0};

void ct_seterr(ct_handle* h, const char* fmt, ...) {
    if (!h) return;
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    h->err = buf;
}

int ct_reserve(ct_handle* h, size_t bytes) {
    if (bytes <= h->ws_cap) return CT_OK;
    size_t want = bytes + bytes / 4 + (1u << 20);
    if (h->ws_limit && want > h->ws_limit) want = bytes;
    if (h->ws_limit && want > h->ws_limit) {
        ct_seterr(h, "workspace of %zu bytes exceeds the limit of %zu bytes", bytes, h->ws_limit);
        return CT_ERR_OOM;
    }
    if (h->ws) {
        CT_CUDA(h, cudaStreamSynchronize(h->stream));
        CT_CUDA(h, cudaFree(h->ws));
        h->ws = nullptr;
        h->ws_cap = 0;
    }
    cudaError_t e = cudaMalloc((void**)&h->ws, want);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        h->ws = nullptr;
        ct_seterr(h, "cudaMalloc(%zu) failed: %s", want, cudaGetErrorString(e));
        return CT_ERR_OOM;
    }
    h->ws_cap = want;
    return CT_OK;
}

static int check_status(ct_handle* h) {
    int st = 0;
    CT_CUDA(h, cudaMemcpyAsync(&st, h->d_status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CT_CUDA(h, cudaStreamSynchronize(h->stream));
    if (st != 0) {
        CT_CUDA(h, cudaMemsetAsync(h->d_status, 0, sizeof(int), h->stream));
        if (h->err.empty()) ct_seterr(h, "device status %d", st);
        return st;
    }
    return CT_OK;
}

#define CT_NULLCHK(h, p)                                                   \
    do {                                                                   \
        if (!(p)) {                                                        \
            ct_seterr((h), "%s: null pointer argument '%s'", __func__, #p); \
            return CT_ERR_INVALID;                                         \
        }                                                                  \
    } while (0)

#define CT_POSCHK(h, v)                                                          \
    do {                                                                         \
        if ((v) <= 0) {                                                          \
            ct_seterr((h), "%s: dimension %s=%lld must be > 0", __func__, #v, (long long)(v)); \
            return CT_ERR_SHAPE;                                                 \
        }                                                                        \
    } while (0)

static int check_prec(ct_handle* h, int prec) {
    if (prec == CT_PREC_FP64) return CT_OK;
    if (prec == CT_PREC_TF32X3) {
        if (ct_tc_available(h)) return CT_OK;
        ct_seterr(h, "TF32x3 tensor-core path needs an sm_103 device");
        return CT_ERR_UNSUPPORTED;
    }
    ct_seterr(h, "unknown precision %d", prec);
    return CT_ERR_INVALID;
}

extern "C" {

int ct_version(void) { return CTDMRG_VERSION; }

int64_t ct_launch_count(void) { return (int64_t)g_ct_launches.load(); }

const char* ct_error_string(int s) {
    switch (s) {
        case CT_OK: return "ok";
        case CT_ERR_INVALID: return "invalid argument";
        case CT_ERR_CUDA: return "CUDA error";
        case CT_ERR_OOM: return "out of device memory";
        case CT_ERR_NOCONV: return "iterative solver did not converge";
        case CT_ERR_ZERO_NORM: return "initial vector has zero norm";
        case CT_ERR_SHAPE: return "shape mismatch";
        case CT_ERR_UNSUPPORTED: return "unsupported";
        case CT_ERR_NONFINITE: return "non-finite value";
        case CT_ERR_EMPTY: return "truncation kept no singular values";
        case CT_ERR_TOO_LARGE: return "problem exceeds the static scratch of the no-alloc entry point";
        default: return "unknown status";
    }
}

const char* ct_last_error(ct_handle* h) { return h ? h->err.c_str() : "null handle"; }

int ct_create(int device, void* stream, ct_handle** out) {
    if (!out) return CT_ERR_INVALID;
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        (void)cudaGetLastError();
        return CT_ERR_CUDA;
    }
    if (device < 0 || device >= ndev) return CT_ERR_INVALID;
    ct_handle* h = new ct_handle();
    h->device = device;
    if (cudaSetDevice(device) != cudaSuccess) {
        delete h;
        return CT_ERR_CUDA;
    }
    cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (stream) {
        h->stream = (cudaStream_t)stream;
    } else {
        if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete h;
            return CT_ERR_CUDA;
        }
        h->own_stream = true;
    }
    bool ok = cudaMalloc((void**)&h->d_status, sizeof(int)) == cudaSuccess &&
              cudaMalloc((void**)&h->d_scalars, CT_NSCALARS * sizeof(double)) == cudaSuccess &&
              cudaMalloc((void**)&h->d_partials, CT_NPARTIALS * sizeof(double)) == cudaSuccess &&
              cudaMalloc((void**)&h->d_flags, CT_NFLAGS * sizeof(int)) == cudaSuccess;
    if (ok) ok = cudaMemset(h->d_status, 0, sizeof(int)) == cudaSuccess &&
                 cudaMemset(h->d_flags, 0, CT_NFLAGS * sizeof(int)) == cudaSuccess &&
                 cudaMemset(h->d_scalars, 0, CT_NSCALARS * sizeof(double)) == cudaSuccess;
    if (!ok) {
        ct_destroy(h);
        return CT_ERR_OOM;
    }
    *out = h;
    return CT_OK;
}

int ct_destroy(ct_handle* h) {
    if (!h) return CT_ERR_INVALID;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    cudaFree(h->ws);
    for (auto& b : h->basis_cache) cudaFree(b.p);
    for (auto e : h->ktime_ev) cudaEventDestroy(e);
    cudaFree(h->splitk);
    cudaFree(h->oz_ws);
    cudaFree(h->tc_sk_part);
    cudaFree(h->tc_sk_flag);
    cudaFree(h->tc_hy_part);
    cudaFree(h->tc_hy_cnt);
    cudaFree(h->d_status);
    cudaFree(h->d_scalars);
    cudaFree(h->d_partials);
    cudaFree(h->d_flags);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return CT_OK;
}

int ct_set_stream(ct_handle* h, void* stream) {
    CT_NULLCHK(h, h);
    if (h->own_stream && h->stream) {
        cudaStreamSynchronize(h->stream);
        cudaStreamDestroy(h->stream);
        h->own_stream = false;
    }
    if (stream) {
        h->stream = (cudaStream_t)stream;
    } else {
        CT_CUDA(h, cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        h->own_stream = true;
    }
    return CT_OK;
}

int ct_synchronize(ct_handle* h) {
    CT_NULLCHK(h, h);
    CT_CUDA(h, cudaStreamSynchronize(h->stream));
    return CT_OK;
}

int ct_get_status(ct_handle* h, int* status_out) {
    CT_NULLCHK(h, h);
    CT_NULLCHK(h, status_out);
    int st = 0;
    CT_CUDA(h, cudaMemcpyAsync(&st, h->d_status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CT_CUDA(h, cudaStreamSynchronize(h->stream));
    CT_CUDA(h, cudaMemsetAsync(h->d_status, 0, sizeof(int), h->stream));
    *status_out = st;
    return CT_OK;
}

int ct_workspace_bytes(ct_handle* h, int64_t* bytes_out) {
    CT_NULLCHK(h, h);
    CT_NULLCHK(h, bytes_out);
    *bytes_out = (int64_t)h->ws_cap;
    return CT_OK;
}

int ct_svd_sweeps(ct_handle* h, int* last_host, int64_t* total_host) {
    CT_NULLCHK(h, h);
    if (last_host) *last_host = h->last_svd_sweeps;
    if (total_host) *total_host = h->total_svd_sweeps;
    return CT_OK;
}

int ct_set_workspace_limit(ct_handle* h, int64_t bytes) {
    CT_NULLCHK(h, h);
    if (bytes < 0) return CT_ERR_INVALID;
    h->ws_limit = (size_t)bytes;
    return CT_OK;
}

int ct_set_svd_max_sweeps(ct_handle* h, int max_sweeps) {
    CT_NULLCHK(h, h);
    if (max_sweeps < 0) return CT_ERR_INVALID;
    h->svd_max_sweeps = max_sweeps;
    return CT_OK;
}

// ---------------------------------------------------------------------------
// dense tensor core
// ---------------------------------------------------------------------------
int ct_gemm(ct_handle* h, int prec, int trans_a, int trans_b, int64_t m, int64_t n, int64_t k, double alpha,
            const double* A, int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc) {
    CT_NULLCHK(h, h);
    if (prec == CT_PREC_FP64_TC) {
        if (!ct_tc_available(h)) {
            ct_seterr(h, "FP64 tensor-core GEMM needs an sm_103 device");
            return CT_ERR_UNSUPPORTED;
        }
    } else {
        CT_TRY(check_prec(h, prec));
    }
    if (m < 0 || n < 0 || k < 0) return CT_ERR_SHAPE;
    if (m == 0 || n == 0) return CT_OK;
    CT_NULLCHK(h, C);
    if (k > 0) {
        CT_NULLCHK(h, A);
        CT_NULLCHK(h, B);
    }
    // row-major op(A)[m,k]: trans_a=0 -> A[i*lda + p], trans_a=1 -> A[p*lda + i]
    if ((!trans_a && lda < k) || (trans_a && lda < m) || (!trans_b && ldb < n) || (trans_b && ldb < k) || ldc < n) {
        ct_seterr(h, "ct_gemm: leading dimension too small");
        return CT_ERR_SHAPE;
    }
    if (prec == CT_PREC_TF32X3 && k > 0) {
        CT_TRY(ct_reserve(h, ct_tc_gemm_ws_bytes(m, n, k)));
        Arena ar(h);
        CT_TRY(ct_tc_gemm(h, ar, trans_a, trans_b, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc));
        return CT_OK;
    }
    if (prec == CT_PREC_FP64_TC && k > 0) {
        // op(A)(i,p) = trans_a ? A[p*lda + i] : A[i*lda + p]; B(j,p) = op(B)[p][j]
        CT_TRY(ct_oz_gemm(h, m, n, k, A, trans_a ? 1 : lda, trans_a ? lda : 1, B, trans_b ? ldb : 1,
                          trans_b ? 1 : ldb, alpha, beta, C, ldc));
        return CT_OK;
    }
    GemmDesc g{};
    g.M = m; g.N = n; g.K = k;
    g.A = A; g.sAm = trans_a ? 1 : lda; g.sAk = trans_a ? lda : 1;
    g.B = B; g.sBk = trans_b ? 1 : ldb; g.sBn = trans_b ? ldb : 1;
    g.C = C; g.sCm = ldc; g.sCn = 1;
    g.alpha = alpha; g.beta = beta; g.nb1 = 1; g.nb0 = 1;
    return ct_gemm_f64_launch(h, g);
}

int ct_permute(ct_handle* h, const double* in, double* out, int rank, const int64_t* shape, const int32_t* perm) {
    CT_NULLCHK(h, h);
    CT_NULLCHK(h, in);
    CT_NULLCHK(h, out);
    CT_NULLCHK(h, shape);
    CT_NULLCHK(h, perm);
    for (int i = 0; i < rank; ++i)
        if (shape[i] < 0) return CT_ERR_SHAPE;
    return ct_permute_launch(h, in, out, rank, shape, perm);
}

int ct_vec_dot(ct_handle* h, int64_t n, const double* x, const double* y, double* result_host) {
    CT_NULLCHK(h, h);
    CT_NULLCHK(h, result_host);
    if (n < 0) return CT_ERR_SHAPE;
    if (n == 0) {
        *result_host = 0.0;
        return CT_OK;
    }
    CT_NULLCHK(h, x);
    CT_NULLCHK(h, y);
    CT_TRY(ct_reduce_dot(h, n, x, y, h->d_scalars + SC_DOT, nullptr));
    CT_CUDA(h, cudaMemcpyAsync(result_host, h->d_scalars + SC_DOT, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CT_CUDA(h, cudaStreamSynchronize(h->stream));
    return CT_OK;
}

int ct_vec_norm_sq(ct_handle* h, int64_t n, const double* x, double* result_host) {
    CT_NULLCHK(h, h);
    CT_NULLCHK(h, result_host);
    if (n < 0) return CT_ERR_SHAPE;
    if (n == 0) {
        *result_host = 0.0;
        return CT_OK;
    }
    CT_NULLCHK(h, x);
    CT_TRY(ct_reduce_nrm2sq(h, n, x, h->d_scalars + SC_DOT, nullptr));
    CT_CUDA(h, cudaMemcpyAsync(result_host, h->d_scalars + SC_DOT, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CT_CUDA(h, cudaStreamSynchronize(h->stream));
    return CT_OK;
}

int ct_vec_axpy(ct_handle* h, int64_t n, double alpha, const double* x, double* y) {
    CT_NULLCHK(h, h);
    if (n < 0) return CT_ERR_SHAPE;
    if (n == 0) return CT_OK;
    CT_NULLCHK(h, x);
    CT_NULLCHK(h, y);
    return ct_vec_axpy_launch(h, n, alpha, x, y);
}

int ct_vec_scale(ct_handle* h, int64_t n, double alpha, double* x) {
    CT_NULLCHK(h, h);
    if (n < 0) return CT_ERR_SHAPE;
    if (n == 0) return CT_OK;
    CT_NULLCHK(h, x);
    return ct_vec_scale_launch(h, n, alpha, x);
}

int ct_env_identity(ct_handle* h, double* E, int64_t w, int64_t D) {
    CT_NULLCHK(h, h);
    CT_NULLCHK(h, E);
    CT_POSCHK(h, w);
    CT_POSCHK(h, D);
    return ct_identity_env(h, E, w, D);
}

// ---------------------------------------------------------------------------
// two-site DMRG building blocks
// ---------------------------------------------------------------------------
int ct_theta2(ct_handle* h, int prec, const double* A_i, const double* A_ip1, double* theta, int64_t Dl, int64_t d,
              int64_t Dm, int64_t Dr) {
    CT_NULLCHK(h, h);
    CT_TRY(check_prec(h, prec));
    CT_NULLCHK(h, A_i);
    CT_NULLCHK(h, A_ip1);
    CT_NULLCHK(h, theta);
    CT_POSCHK(h, Dl);
    CT_POSCHK(h, d);
    CT_POSCHK(h, Dm);
    CT_POSCHK(h, Dr);
    CT_TRY(ct_reserve(h, ct_theta_ws_bytes(prec, Dl, d, Dm, Dr)));
    return ct_theta_run(h, prec, A_i, A_ip1, theta, Dl, d, Dm, Dr);
}

int ct_heff2_apply(ct_handle* h, int prec, const double* theta, const double* L, const double* R, const double* W1,
                   const double* W2, double* out, int64_t Dl, int64_t d, int64_t Dr, int64_t wL, int64_t wM,
                   int64_t wR) {
    CT_NULLCHK(h, h);
    CT_TRY(check_prec(h, prec));
    CT_NULLCHK(h, theta);
    CT_NULLCHK(h, L);
    CT_NULLCHK(h, R);
    CT_NULLCHK(h, W1);
    CT_NULLCHK(h, W2);
    CT_NULLCHK(h, out);
    CT_POSCHK(h, Dl);
    CT_POSCHK(h, d);
    CT_POSCHK(h, Dr);
    CT_POSCHK(h, wL);
    CT_POSCHK(h, wM);
    CT_POSCHK(h, wR);
    CT_TRY(ct_reserve(h, ct_heff_ws_bytes(prec, Dl, d, Dr, wL, wM, wR)));
    Arena ar(h);
    HeffPlan p;
    CT_TRY(ct_heff_prepare(h, ar, p, prec, L, R, W1, W2, Dl, d, Dr, wL, wM, wR));
    CT_TRY(ct_heff_run(h, p, theta, out, nullptr));
    return CT_OK;
}

int ct_env_left(ct_handle* h, int prec, const double* Lprev, const double* A, const double* W, double* Lnext,
                int64_t Dl, int64_t d, int64_t Dr, int64_t wL, int64_t wR) {
    CT_NULLCHK(h, h);
    CT_TRY(check_prec(h, prec));
    CT_NULLCHK(h, Lprev);
    CT_NULLCHK(h, A);
    CT_NULLCHK(h, W);
    CT_NULLCHK(h, Lnext);
    CT_POSCHK(h, Dl);
    CT_POSCHK(h, d);
    CT_POSCHK(h, Dr);
    CT_POSCHK(h, wL);
    CT_POSCHK(h, wR);
    CT_TRY(ct_reserve(h, ct_env_ws_bytes(prec, Dl, d, Dr, wL, wR)));
    Arena ar(h);
    return ct_env_left_run(h, ar, prec, Lprev, A, W, Lnext, Dl, d, Dr, wL, wR);
}

int ct_env_left2(ct_handle* h, int prec, const double* Lprev, const double* A_ket, const double* A_bra,
                 const double* W, double* Lnext, int64_t Dl_ket, int64_t Dl_bra, int64_t d, int64_t Dr_ket,
                 int64_t Dr_bra, int64_t wL, int64_t wR) {
    CT_NULLCHK(h, h);
    if (prec != CT_PREC_FP64) {
        ct_seterr(h, "ct_env_left2: only the FP64 form takes a bra different from the ket");
        return CT_ERR_UNSUPPORTED;
    }
    CT_NULLCHK(h, Lprev);
    CT_NULLCHK(h, A_ket);
    CT_NULLCHK(h, A_bra);
    CT_NULLCHK(h, Lnext);
    CT_POSCHK(h, Dl_ket);
    CT_POSCHK(h, Dl_bra);
    CT_POSCHK(h, d);
    CT_POSCHK(h, Dr_ket);
    CT_POSCHK(h, Dr_bra);
    CT_POSCHK(h, wL);
    CT_POSCHK(h, wR);
    if (!W && (wL != 1 || wR != 1)) {
        ct_seterr(h, "ct_env_left2: without an MPO site wL and wR must be 1");
        return CT_ERR_SHAPE;
    }
    CT_TRY(ct_reserve(h, ct_env2_ws_bytes(Dl_ket, Dl_bra, d, Dr_ket, Dr_bra, wL, wR)));
    Arena ar(h);
    return ct_env_left2_run(h, ar, Lprev, A_ket, A_bra, W, Lnext, Dl_ket, Dl_bra, d, Dr_ket, Dr_bra, wL, wR);
}

int ct_mpo_compose_site(ct_handle* h, const double* Wa, const double* Wb, double* Wout, int64_t wLa,
                        int64_t d_in, int64_t d_mid, int64_t wRa, int64_t wLb, int64_t d_out, int64_t wRb) {
    CT_NULLCHK(h, h);
    CT_NULLCHK(h, Wa);
    CT_NULLCHK(h, Wb);
    CT_NULLCHK(h, Wout);
    CT_POSCHK(h, wLa);
    CT_POSCHK(h, d_in);
    CT_POSCHK(h, d_mid);
    CT_POSCHK(h, wRa);
    CT_POSCHK(h, wLb);
    CT_POSCHK(h, d_out);
    CT_POSCHK(h, wRb);
    return ct_mpo_compose_launch(h, Wa, Wb, Wout, wLa, d_in, d_mid, wRa, wLb, d_out, wRb);
}

int ct_apply_mpo_site(ct_handle* h, const double* A, const double* W, double* out, int64_t Dl, int64_t d,
                      int64_t Dr, int64_t wL, int64_t d_out, int64_t wR) {
    CT_NULLCHK(h, h);
    CT_NULLCHK(h, A);
    CT_NULLCHK(h, W);
    CT_NULLCHK(h, out);
    CT_POSCHK(h, Dl);
    CT_POSCHK(h, d);
    CT_POSCHK(h, Dr);
    CT_POSCHK(h, wL);
    CT_POSCHK(h, d_out);
    CT_POSCHK(h, wR);
    return ct_apply_mpo_launch(h, A, W, out, Dl, d, Dr, wL, d_out, wR);
}

int ct_env_right(ct_handle* h, int prec, const double* Rnext, const double* A, const double* W, double* Rprev,
                 int64_t Dl, int64_t d, int64_t Dr, int64_t wL, int64_t wR) {
    CT_NULLCHK(h, h);
    CT_TRY(check_prec(h, prec));
    CT_NULLCHK(h, Rnext);
    CT_NULLCHK(h, A);
    CT_NULLCHK(h, W);
    CT_NULLCHK(h, Rprev);
    CT_POSCHK(h, Dl);
    CT_POSCHK(h, d);
    CT_POSCHK(h, Dr);
    CT_POSCHK(h, wL);
    CT_POSCHK(h, wR);
    CT_TRY(ct_reserve(h, ct_env_ws_bytes(prec, Dl, d, Dr, wL, wR)));
    Arena ar(h);
    return ct_env_right_run(h, ar, prec, Rnext, A, W, Rprev, Dl, d, Dr, wL, wR);
}

int ct_lanczos2(ct_handle* h, int prec, const double* theta_in, double* theta_out, const double* L, const double* R,
                const double* W1, const double* W2, int64_t Dl, int64_t d, int64_t Dr, int64_t wL, int64_t wM,
                int64_t wR, int max_iter, double tol, int max_rotations, int reorth, double* energy_host,
                int* numiter_host, double* alpha_host, double* beta_host) {
    CT_NULLCHK(h, h);
    CT_TRY(check_prec(h, prec));
    CT_NULLCHK(h, theta_in);
    CT_NULLCHK(h, theta_out);
    CT_NULLCHK(h, L);
    CT_NULLCHK(h, R);
    CT_NULLCHK(h, W1);
    CT_NULLCHK(h, W2);
    CT_NULLCHK(h, energy_host);
    CT_POSCHK(h, Dl);
    CT_POSCHK(h, d);
    CT_POSCHK(h, Dr);
    CT_POSCHK(h, wL);
    CT_POSCHK(h, wM);
    CT_POSCHK(h, wR);
    if (theta_in == theta_out) {
        ct_seterr(h, "ct_lanczos2: theta_in and theta_out must not alias");
        return CT_ERR_INVALID;
    }
    CT_TRY(ct_reserve(h, ct_lanczos_ws_bytes(prec, Dl, d, Dr, wL, wM, wR, max_iter)));
    Arena ar(h);
    LanczosResult res;
    CT_TRY(ct_lanczos_run(h, ar, prec, theta_in, theta_out, L, R, W1, W2, Dl, d, Dr, wL, wM, wR, max_iter, tol,
                          max_rotations, reorth, &res));
    int nk = 0;
    CT_CUDA(h, cudaMemcpyAsync(energy_host, res.d_energy, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CT_CUDA(h, cudaMemcpyAsync(&nk, res.d_numiter, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    if (alpha_host)
        CT_CUDA(h, cudaMemcpyAsync(alpha_host, h->d_scalars + SC_ALPHA, max_iter * sizeof(double),
                                   cudaMemcpyDeviceToHost, h->stream));
    if (beta_host && max_iter > 1)
        CT_CUDA(h, cudaMemcpyAsync(beta_host, h->d_scalars + SC_BETA, (max_iter - 1) * sizeof(double),
                                   cudaMemcpyDeviceToHost, h->stream));
    CT_TRY(check_status(h));
    if (numiter_host) *numiter_host = nk;
    return CT_OK;
}

int ct_svd_trunc(ct_handle* h, const double* M, int64_t m, int64_t n, int64_t chi_max, double eps_trunc, double* U,
                 double* S, double* Vt, int64_t* chi_host) {
    CT_NULLCHK(h, h);
    CT_NULLCHK(h, chi_host);
    if (m < 0 || n < 0 || chi_max < 0) return CT_ERR_SHAPE;
    if (m == 0 || n == 0) {
        *chi_host = 0;
        return CT_OK;
    }
    CT_NULLCHK(h, M);
    CT_NULLCHK(h, U);
    CT_NULLCHK(h, S);
    CT_NULLCHK(h, Vt);
    CT_TRY(ct_reserve(h, ct_svd_ws_bytes(m, n, 2)));
    Arena ar(h);
    // a NaN or infinite entry is an error (LAPACK's dgesdd fails on it, svd.mojo:74-76)
    CT_TRY(ct_reduce_nrm2sq(h, m * n, M, h->d_scalars + SC_DOT, nullptr));
    CT_TRY(ct_check_finite(h, h->d_scalars + SC_DOT, nullptr));
    SvdOut o;
    CT_TRY(ct_svd_run(h, ar, M, m, n, chi_max, eps_trunc, 2, U, Vt, S, &o));
    CT_TRY(check_status(h));
    *chi_host = o.chi;
    return CT_OK;
}

int ct_qr(ct_handle* h, const double* A, int64_t m, int64_t n, double* Q, double* R, int* completed_host) {
    CT_NULLCHK(h, h);
    if (m < 0 || n < 0) return CT_ERR_SHAPE;
    if (completed_host) *completed_host = 0;
    if (m == 0 || n == 0) return CT_OK;
    CT_NULLCHK(h, A);
    CT_NULLCHK(h, Q);
    CT_NULLCHK(h, R);
    if (!ct_tc_available(h)) {
        ct_seterr(h, "ct_qr: the orthonormalisation's correction step needs the sm_103a tensor-core path");
        return CT_ERR_UNSUPPORTED;
    }
    CT_TRY(ct_reserve(h, ct_qr_ws_bytes(m, n)));
    Arena ar(h);
    int done = 0;
    CT_TRY(ct_qr_run(h, ar, A, m, n, Q, R, &done));
    CT_TRY(check_status(h));
    if (completed_host) *completed_host = done;
    return CT_OK;
}

int ct_svd_split(ct_handle* h, int prec, const double* theta, int64_t Dl, int64_t d, int64_t Dr, int64_t chi_max,
                 double eps_trunc, int left_to_right, double* A_out, double* B_out, double* S_out, int64_t* chi_host,
                 double* discarded_host) {
    CT_NULLCHK(h, h);
    CT_TRY(check_prec(h, prec));
    CT_NULLCHK(h, theta);
    CT_NULLCHK(h, A_out);
    CT_NULLCHK(h, B_out);
    CT_NULLCHK(h, chi_host);
    CT_POSCHK(h, Dl);
    CT_POSCHK(h, d);
    CT_POSCHK(h, Dr);
    if (chi_max < 0) return CT_ERR_SHAPE;
    const int64_t m = Dl * d, n = d * Dr;
    const int mode = left_to_right ? 0 : 1;
    CT_TRY(ct_reserve(h, ct_split_ws_bytes(prec, m, n, chi_max, mode)));
    Arena ar(h);
    // |theta|^2 in FP64 on the device (dmrg.mojo:176)
    CT_TRY(ct_reduce_nrm2sq(h, m * n, theta, h->d_scalars + SC_THETA_NSQ, nullptr));
    CT_TRY(ct_check_finite(h, h->d_scalars + SC_THETA_NSQ, nullptr));
    double tn = 0.0;
    CT_CUDA(h, cudaMemcpyAsync(&tn, h->d_scalars + SC_THETA_NSQ, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    SvdOut o;
    CT_TRY(ct_split_run(h, ar, prec, theta, m, n, chi_max, eps_trunc, mode, A_out, B_out, S_out,
                        h->d_scalars + SC_THETA_NSQ, &o));
    CT_TRY(check_status(h));
    *chi_host = o.chi;
    if (discarded_host) *discarded_host = (tn > 0.0) ? (tn - o.sum_s2_kept) / tn : 0.0;
    return CT_OK;
}

int ct_svd_split_warm(ct_handle* h, const double* theta, int64_t Dl, int64_t d, int64_t Dr, int64_t chi,
                      int left_to_right, const double* basis_in, int power_steps,
                      double* basis_out, double* A_out, double* B_out, int* accepted, double* discarded_host,
                      double* pivots_host) {
    CT_NULLCHK(h, h);
    CT_NULLCHK(h, theta);
    CT_NULLCHK(h, basis_in);
    CT_NULLCHK(h, basis_out);
    CT_NULLCHK(h, A_out);
    CT_NULLCHK(h, B_out);
    CT_NULLCHK(h, accepted);
    CT_POSCHK(h, Dl);
    CT_POSCHK(h, d);
    CT_POSCHK(h, Dr);
    const int64_t m = Dl * d, n = d * Dr;
    if (chi <= 0 || chi > (m < n ? m : n)) return CT_ERR_SHAPE;
    if (!ct_tc_available(h)) return CT_ERR_UNSUPPORTED;
    CT_TRY(ct_reserve(h, ct_split_subspace_ws_bytes(m, n, chi)));
    Arena ar(h);
    CT_TRY(ct_reduce_nrm2sq(h, m * n, theta, h->d_scalars + SC_THETA_NSQ, nullptr));
    CT_TRY(ct_check_finite(h, h->d_scalars + SC_THETA_NSQ, nullptr));
    SvdOut o;
    bool ok = false;
    if (power_steps < 0) return CT_ERR_INVALID;
    CT_TRY(ct_split_subspace(h, ar, theta, m, n, chi, left_to_right ? 0 : 1, basis_in, basis_out, A_out, B_out,
                             h->d_scalars + SC_THETA_NSQ, 0.0, -1.0, 0.0, 0.0, power_steps, false, 0, &o, &ok));
    CT_TRY(check_status(h));
    *accepted = ok ? 1 : 0;
    if (discarded_host)
        *discarded_host = (o.sum_s2_all > 0.0) ? (o.sum_s2_all - o.sum_s2_kept) / o.sum_s2_all : 0.0;
    if (pivots_host) {
        pivots_host[0] = o.min_pivot;
        pivots_host[1] = o.min_pivot2;
        pivots_host[2] = o.chol_fail;
    }
    return CT_OK;
}

int ct_kernel_timing(ct_handle* h, int enable) {
    CT_NULLCHK(h, h);
    CT_TRY(ct_ktime_harvest(h));
    h->ktime_on = enable != 0;
    h->ktime_open = 0;
    h->ktime_dropped = 0;
    for (int c = 0; c < KT_NCLASSES; ++c) {
        h->ktime_count[c] = 0;
        h->ktime_ms[c] = 0.0;
        h->ktime_flops[c] = 0.0;
    }
    return CT_OK;
}

int ct_kernel_timing_read_class(ct_handle* h, int cls, int64_t* count, double* ms, double* flops) {
    CT_NULLCHK(h, h);
    if (!count || !ms || !flops || cls < 0 || cls >= KT_NCLASSES) return CT_ERR_INVALID;
    CT_TRY(ct_ktime_harvest(h));
    *count = h->ktime_count[cls];
    *ms = h->ktime_ms[cls];
    *flops = h->ktime_flops[cls];
    return CT_OK;
}

int ct_kernel_timing_read(ct_handle* h, int64_t* launches, double* ms, double* flops) {
    return ct_kernel_timing_read_class(h, KT_TC_GEMM, launches, ms, flops);
}

}  // extern "C"

namespace {
constexpr int KTIME_SLOTS = 16384;
}

// Sum the elapsed times of the pending event pairs per class (waits for the last one).
int ct_ktime_harvest(ct_handle* h) {
    if (h->ktime_pending == 0 || h->ktime_open > 0) return CT_OK;
    CT_CUDA(h, cudaEventSynchronize(h->ktime_ev[2 * (h->ktime_pending - 1) + 1]));
    for (int i = 0; i < h->ktime_pending; ++i) {
        float ms = 0.f;
        CT_CUDA(h, cudaEventElapsedTime(&ms, h->ktime_ev[2 * i], h->ktime_ev[2 * i + 1]));
        const int c = h->ktime_slot_cls[i];
        const double fl = h->ktime_slot_flops[i];
        h->ktime_ms[c] += ms;
        h->ktime_flops[c] += fl;
        h->ktime_count[c] += 1;
        if (c == KT_HEFF_APPLY) {
            // running bucket of the largest applies (relative tolerance 1e-9 on the FLOP count)
            const double top = h->ktime_count[KT_HEFF_LARGEST] > 0
                                   ? h->ktime_flops[KT_HEFF_LARGEST] / (double)h->ktime_count[KT_HEFF_LARGEST]
                                   : 0.0;
            if (fl > top * (1.0 + 1e-9)) {
                h->ktime_count[KT_HEFF_LARGEST] = 0;
                h->ktime_ms[KT_HEFF_LARGEST] = 0.0;
                h->ktime_flops[KT_HEFF_LARGEST] = 0.0;
            }
            if (fl >= top * (1.0 - 1e-9)) {
                h->ktime_count[KT_HEFF_LARGEST] += 1;
                h->ktime_ms[KT_HEFF_LARGEST] += ms;
                h->ktime_flops[KT_HEFF_LARGEST] += fl;
            }
        }
    }
    h->ktime_pending = 0;
    return CT_OK;
}

int ct_ktime_begin(ct_handle* h, int cls, double flops, int* slot) {
    *slot = -1;
    if (!h->ktime_on) return CT_OK;
    if (h->ktime_ev.empty()) {
        h->ktime_ev.resize(2 * KTIME_SLOTS, nullptr);
        h->ktime_slot_flops.resize(KTIME_SLOTS, 0.0);
        h->ktime_slot_cls.resize(KTIME_SLOTS, 0);
        for (auto& e : h->ktime_ev) CT_CUDA(h, cudaEventCreate(&e));
    }
    // read the pool back before it fills, at a moment with no open region (a
    // region nests only a few others, so 64 spare slots are enough)
    if (h->ktime_pending >= KTIME_SLOTS - 64 && h->ktime_open == 0) CT_TRY(ct_ktime_harvest(h));
    if (h->ktime_pending == KTIME_SLOTS) {
        h->ktime_dropped++;
        return CT_OK;
    }
    *slot = h->ktime_pending++;
    h->ktime_open++;
    h->ktime_slot_flops[*slot] = flops;
    h->ktime_slot_cls[*slot] = cls;
    CT_CUDA(h, cudaEventRecord(h->ktime_ev[2 * *slot], h->stream));
    return CT_OK;
}

int ct_ktime_end(ct_handle* h, int slot) {
    if (slot < 0) return CT_OK;
    h->ktime_open--;
    CT_CUDA(h, cudaEventRecord(h->ktime_ev[2 * slot + 1], h->stream));
    return CT_OK;
}
