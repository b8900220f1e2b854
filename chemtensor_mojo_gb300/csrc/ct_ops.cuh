// Internal interfaces of the contraction chains and the Lanczos driver.
#pragma once
#include "ct_common.cuh"

struct HeffPlan {
    int prec = CT_PREC_FP64;
    const double *L = nullptr, *R = nullptr, *W1 = nullptr, *W2 = nullptr;
    int64_t Dl = 0, d = 0, Dr = 0, wL = 0, wM = 0, wR = 0;
    // FP64 form
    double* T1 = nullptr;
    double* T3 = nullptr;
    double* W12 = nullptr;
    // mixed form (ct_tc.cu): operand planes of the bond, constructed in place
    void* tc = nullptr;
    alignas(16) unsigned char tc_store[512];
};

struct LanczosResult {
    double* d_energy = nullptr;
    int* d_numiter = nullptr;
    int applies_upper = 0;
};

size_t ct_heff_ws_bytes(int prec, int64_t Dl, int64_t d, int64_t Dr, int64_t wL, int64_t wM, int64_t wR);
int ct_heff_prepare(ct_handle* h, Arena& ar, HeffPlan& p, int prec, const double* L, const double* R,
                    const double* W1, const double* W2, int64_t Dl, int64_t d, int64_t Dr, int64_t wL,
                    int64_t wM, int64_t wR);
int ct_heff_run(ct_handle* h, const HeffPlan& p, const double* theta, double* out, const int* skip);

size_t ct_env_ws_bytes(int prec, int64_t Dl, int64_t d, int64_t Dr, int64_t wL, int64_t wR);
int ct_env_left_run(ct_handle* h, Arena& ar, int prec, const double* Lp, const double* A, const double* W,
                    double* Ln, int64_t Dl, int64_t d, int64_t Dr, int64_t wL, int64_t wR);
int ct_env_right_run(ct_handle* h, Arena& ar, int prec, const double* Rn, const double* A, const double* W,
                     double* Rp, int64_t Dl, int64_t d, int64_t Dr, int64_t wL, int64_t wR);
size_t ct_env2_ws_bytes(int64_t Dlk, int64_t Dlb, int64_t d, int64_t Drk, int64_t Drb, int64_t wL, int64_t wR);
// fp64_tc: the two large products on the BF16 tensor cores (ct_oz_gemm_ex, FP64-accurate)
int ct_env_left2_run(ct_handle* h, Arena& ar, const double* Lp, const double* Ak, const double* Ab,
                     const double* W, double* Ln, int64_t Dlk, int64_t Dlb, int64_t d, int64_t Drk, int64_t Drb,
                     int64_t wL, int64_t wR, bool fp64_tc = false);
// FP64 products on the BF16 tensor cores for this size (CTDMRG_FP64_TC=0 disables them)
bool ct_fp64_tc_enabled(ct_handle* h, int64_t M, int64_t N, int64_t K);
size_t ct_theta_ws_bytes(int prec, int64_t Dl, int64_t d, int64_t Dm, int64_t Dr);
int ct_theta_run(ct_handle* h, int prec, const double* Ai, const double* Aj, double* theta, int64_t Dl,
                 int64_t d, int64_t Dm, int64_t Dr);

size_t ct_lanczos_ws_bytes(int prec, int64_t Dl, int64_t d, int64_t Dr, int64_t wL, int64_t wM, int64_t wR,
                           int max_iter);
int ct_lanczos_run(ct_handle* h, Arena& ar, int prec, const double* theta_in, double* theta_out, const double* L,
                   const double* R, const double* W1, const double* W2, int64_t Dl, int64_t d, int64_t Dr,
                   int64_t wL, int64_t wM, int64_t wR, int max_iter, double tol, int max_rotations, int reorth,
                   LanczosResult* res);

// vector helpers (ct_vec.cu)
int ct_vec_axpy_launch(ct_handle* h, int64_t n, double alpha, const double* x, double* y);
int ct_vec_scale_launch(ct_handle* h, int64_t n, double alpha, double* x);
int ct_lanczos_init(ct_handle* h, int max_iter);

// SVD workspace (ct_svd.cu)
size_t ct_svd_ws_bytes(int64_t m, int64_t n, int mode);
int ct_svd_run(ct_handle* h, Arena& ar, const double* M, int64_t m, int64_t n, int64_t chi_max,
               double eps_trunc, int mode, double* A, double* B, double* S, SvdOut* out);

// mixed-form SVD (ct_svd_mixed.cu); d_total = device |theta|^2
size_t ct_svd_mixed_ws_bytes(int64_t m, int64_t n, int64_t chi_max, int mode);
// qcache (nvec x nvec FP32, may be null): rotations of the previous split of the
// same bond; warm != 0 starts the Jacobi from them and the cache is refreshed.
int ct_svd_mixed_run(ct_handle* h, Arena& ar, const double* M, int64_t m, int64_t n, int64_t chi_max,
                     double eps_trunc, int mode, double* A, double* B, double* S, const double* d_total, SvdOut* out,
                     float* qcache = nullptr, int warm = 0);
// the FP64 Jacobi runs in one CTA below this many doubles of X and Q
static inline bool ct_svd_is_small(int64_t m, int64_t n, int mode) {
    const int64_t nvec = mode ? n : m, len = mode ? m : n;
    return (nvec * len + nvec * nvec) * 8 <= 200 * 1024;
}
// split dispatcher: FP64 Jacobi, or the mixed SVD for large TF32x3 problems
size_t ct_split_ws_bytes(int prec, int64_t m, int64_t n, int64_t chi_max, int mode);
int ct_split_run(ct_handle* h, Arena& ar, int prec, const double* M, int64_t m, int64_t n, int64_t chi_max,
                 double eps_trunc, int mode, double* A, double* B, double* S, const double* d_total, SvdOut* out,
                 float* qcache = nullptr, int warm = 0);

// FP64 GEMM on the BF16 tensor cores (ct_ozaki.cu): C[m*ldc + n] = alpha * sum_k
// A(m,k) B(n,k) + beta * C, A(m,k) = A[m*a_sr + k*a_sk], B(n,k) = B[n*b_sr + k*b_sk]
// (slices in a handle-owned buffer that grows on demand; a Gram product A A^T slices once)
// Two-level rows: element (r, k) of an operand at p[(r / R0) * s1 + (r % R0) * s0 + k * sk]
// (R0 = 0: one level), row m of C at p[(m / M0) * s1 + (m % M0) * s0] with contiguous columns.
struct OzMat {
    const double* p;
    int64_t R0, s1, s0, sk;
};
struct OzOut {
    double* p;
    int64_t M0, s1, s0;
};
int ct_oz_gemm_ex(ct_handle* h, int64_t M, int64_t N, int64_t K, const OzMat& A, const OzMat& B, double alpha,
                  double beta, const OzOut& C, int lower = 0);
size_t ct_oz_gemm_ws_bytes(int64_t M, int64_t N, int64_t K);
int ct_oz_gemm(ct_handle* h, int64_t M, int64_t N, int64_t K, const double* A, int64_t a_sr, int64_t a_sk,
               const double* B, int64_t b_sr, int64_t b_sk, double alpha, double beta, double* C, int64_t ldc,
               int lower = 0);

// warm-started subspace split (ct_svd_subspace.cu)
size_t ct_split_subspace_ws_bytes(int64_t m, int64_t n, int64_t c);
// mode 0 (left-to-right): basis_in = V rows (c x n) kept by the last right-to-left
// split of the bond, basis_out <- Q rows (c x m); mode 1: basis_in = Q rows,
// basis_out <- V rows.  disc_ref: discarded weight at the previous truncating
// visit of the bond (< 0: unknown).  *accepted = false: outputs are not valid,
// use the SVD.
// thin QR A[m,n] = Q[m,k] R[k,n] in FP64 (ct_svd_subspace.cu)
size_t ct_qr_ws_bytes(int64_t m, int64_t n);
int ct_qr_run(ct_handle* h, Arena& ar, const double* A, int64_t m, int64_t n, double* Q, double* R, int* completed);
int ct_split_subspace(ct_handle* h, Arena& ar, const double* M, int64_t m, int64_t n, int64_t c, int mode,
                      const double* basis_in, double* basis_out, double* Aout, double* Bout,
                      const double* d_total, double eps_trunc, double disc_ref, double stale_mult,
                      double stale_abs, int power_steps, bool complete, uint64_t seed, SvdOut* out,
                      bool* accepted);
// first-visit start basis: kept rows (may be null) then random Gaussian rows
int ct_cold_basis(ct_handle* h, const double* prev, int64_t c_prev, int64_t c, int64_t len, uint64_t seed,
                  double* X);
int ct_basis_from_split(ct_handle* h, int mode, const double* Aout, const double* Bout, int64_t m, int64_t n,
                        int64_t c, double* basis);

// mixed form (ct_tc.cu)
size_t ct_tc_heff_ws_bytes(int64_t Dl, int64_t d, int64_t Dr, int64_t wL, int64_t wM, int64_t wR);
int ct_tc_heff_prepare(ct_handle* h, Arena& ar, HeffPlan& p);
int ct_tc_heff_run(ct_handle* h, const HeffPlan& p, const double* theta, double* out, const int* skip);
size_t ct_tc_env_ws_bytes(int64_t Dl, int64_t d, int64_t Dr, int64_t wL, int64_t wR);
size_t ct_tc_heff1_ws_bytes(int64_t Dl, int64_t d, int64_t Dr, int64_t wl, int64_t wr);
int ct_tc_heff1_run(ct_handle* h, Arena& ar, const double* L, const double* A, const double* W, const double* R,
                    double* out, int64_t Dl, int64_t d, int64_t Dr, int64_t wl, int64_t wr);
int ct_tc_env_left_run(ct_handle* h, Arena& ar, const double* Lp, const double* A, const double* W, double* Ln,
                       int64_t Dl, int64_t d, int64_t Dr, int64_t wL, int64_t wR);
int ct_tc_env_right_run(ct_handle* h, Arena& ar, const double* Rn, const double* A, const double* W, double* Rp,
                        int64_t Dl, int64_t d, int64_t Dr, int64_t wL, int64_t wR);
int ct_tc_gemm(ct_handle* h, Arena& ar, int trans_a, int trans_b, int64_t m, int64_t n, int64_t k, double alpha,
               const double* A, int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc);
size_t ct_tc_gemm_ws_bytes(int64_t m, int64_t n, int64_t k);
// same, with C in FP64 (out_fp64=1) or FP32 (beta must be 0 for FP32)
int ct_tc_gemm_ex(ct_handle* h, Arena& ar, int trans_a, int trans_b, int64_t m, int64_t n, int64_t k, double alpha,
                  const double* A, int64_t lda, const double* B, int64_t ldb, double beta, void* C, int out_fp64,
                  int64_t ldc);
