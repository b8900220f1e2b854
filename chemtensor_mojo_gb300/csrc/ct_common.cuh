// Shared definitions of libctdmrg: handle, scratch arena, error plumbing,
// launch helpers and device-side reduction primitives.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include <atomic>
#include <string>
#include <vector>

#include "../../include/ctdmrg.h"

// ---------------------------------------------------------------------------
// handle
// ---------------------------------------------------------------------------
struct ct_handle {
    int device = 0;
    int num_sms = 152;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int* d_status = nullptr;        // sticky first device error code
    double* d_scalars = nullptr;    // small device scalars (CT_NSCALARS doubles)
    double* d_partials = nullptr;   // reduction partials (CT_NPARTIALS doubles)
    int* d_flags = nullptr;         // small int scratch (CT_NFLAGS ints)
    // scratch arena: one device allocation, carved per call
    char* ws = nullptr;
    size_t ws_cap = 0;
    size_t ws_limit = 0;            // 0 = unlimited
    std::string err;
    // bond bases kept by the mixed-form splits, to warm-start the subspace split
    // of the next visit of the bond: entry 2i holds the c rows over (a_{i-1}, s_i)
    // of the last left-to-right split of bond i, entry 2i+1 the c rows over
    // (s_{i+1}, a_{i+1}) of the last right-to-left one.  FP64, freed by ct_destroy.
    struct BasisCache {
        double* p = nullptr;
        int64_t cap = 0, len = -1, c = -1;
        double disc = -1.0;   // discarded weight of the split that wrote it
    };
    std::vector<BasisCache> basis_cache;
    // cap on the one-sided Jacobi sweeps of every SVD on this handle (0 = the
    // kernels' own caps); a split that needs more ends with CT_ERR_NOCONV
    int svd_max_sweeps = 0;
    // diagnostics: Jacobi sweeps of the last SVD split, and the running total
    int last_svd_sweeps = 0;
    int64_t total_svd_sweeps = 0;
    int64_t mixed_fp64_splits = 0;   // mixed splits handed to the FP64 Jacobi (ct_svd_mixed.cu)
    // FP64 GEMM split-K partial sums (grown on demand, freed by ct_destroy)
    double* splitk = nullptr;
    size_t splitk_cap = 0;   // doubles
    void* oz_ws = nullptr;   // slices of the FP64 tensor-core GEMM (ct_ozaki.cu)
    size_t oz_ws_bytes = 0;
    // allocation-free mode (the stack handle of ct_heff2_apply_noalloc): the
    // launchers never call cudaMalloc; split-K partials come from the fixed
    // region below, and K is split only as far as that region holds
    bool no_alloc = false;
    double* splitk_fixed = nullptr;
    size_t splitk_fixed_cap = 0;   // doubles
    // stream-K scratch of the persistent tensor-core GEMM (lazily sized, freed by ct_destroy)
    float* tc_sk_part = nullptr;
    int* tc_sk_flag = nullptr;
    int64_t tc_sk_floats = 0;       // floats held by tc_sk_part
    // stream-K partials and arrival counters of the chunked tensor-core GEMM's hybrid
    // schedule (grown on demand after a stream synchronisation, freed by ct_destroy)
    float* tc_hy_part = nullptr;
    int64_t tc_hy_part_floats = 0;
    unsigned long long* tc_hy_cnt = nullptr;
    int64_t tc_hy_cnt_n = 0;
    unsigned tc_hy_epoch = 0;       // tag of the last launch (never 0 once used)
    // tensor-core path state
    bool tc_checked = false;
    bool tc_ok = false;
    // optional live timing (ct_kernel_timing): an event pair per timed region on
    // the handle's stream, summed per class when the pool fills or on request
    bool ktime_on = false;
    std::vector<cudaEvent_t> ktime_ev;   // 2 per slot
    std::vector<double> ktime_slot_flops;
    std::vector<int> ktime_slot_cls;
    int ktime_pending = 0;
    int ktime_open = 0;              // regions begun and not yet ended
    int64_t ktime_dropped = 0;       // regions not timed: pool full while a region was open
    int64_t ktime_count[5] = {0, 0, 0, 0, 0};
    double ktime_ms[5] = {0, 0, 0, 0, 0}, ktime_flops[5] = {0, 0, 0, 0, 0};
};

// live timing classes; KT_HEFF_LARGEST is derived: the H_eff applies with the
// largest FLOP count seen (the centre bond at chi_max).  KT_LANCZOS_VEC: the
// Krylov vector work of each reorthogonalised Lanczos step (alpha, recurrence,
// Gram-Schmidt pass, next vector), its "flops" field holding algorithmic bytes.
// KT_OZ_GEMM: the FP64 GEMM on the BF16 tensor cores (2 M N K per launch).
enum { KT_TC_GEMM = 0, KT_HEFF_APPLY = 1, KT_HEFF_LARGEST = 2, KT_LANCZOS_VEC = 3, KT_OZ_GEMM = 4, KT_NCLASSES = 5 };
// start a timed region of class cls (slot = -1 when timing is off); end it after the launches
int ct_ktime_begin(ct_handle* h, int cls, double flops, int* slot);
int ct_ktime_end(ct_handle* h, int slot);
int ct_ktime_harvest(ct_handle* h);

enum { CT_NSCALARS = 1024, CT_NPARTIALS = 8192, CT_NFLAGS = 256, CT_MAX_KRYLOV_SLOTS = 128 };

// scalar slots inside d_scalars
enum {
    SC_DOT = 0,            // generic reduction result
    SC_NORM = 1,
    SC_ENERGY = 2,
    SC_TMP0 = 3,
    SC_TMP1 = 4,
    SC_DISCARD = 5,
    SC_THETA_NSQ = 6,
    SC_RITZ = 64,          // Ritz coefficients (<= 128)
    SC_ALPHA = 256,        // Lanczos alpha (<= 128)
    SC_BETA = 512,         // Lanczos beta (<= 128)
    SC_MISC = 768,         // scratch (<= 128): Thomas coefficients, reorthogonalisation
    SC_SVD_FROB2 = 968,    // mixed SVD: |M|_F^2
    SC_SPLIT_PIV = 970,    // subspace split: smallest Cholesky pivot of each pass (2)
    SC_ORTH_EMAX = 972,    // subspace split: largest |Q Q^T - I| seen by the second pass
    SC_SVD_MINKEPT = 973   // Jacobi split: smallest kept singular value
};
static_assert(SC_MISC + CT_MAX_KRYLOV_SLOTS <= SC_SVD_FROB2 && SC_SPLIT_PIV + 2 <= SC_ORTH_EMAX &&
                  SC_ORTH_EMAX < SC_SVD_MINKEPT && SC_SVD_MINKEPT + 1 <= CT_NSCALARS,
              "scalar slots overlap or overflow d_scalars");
// int slots inside d_flags
enum { FL_STOP = 0, FL_NUMITER = 1, FL_ROT = 2, FL_CHI = 3, FL_TMP = 4, FL_CNT = 8, FL_REDO = 9, FL_REDO64 = 10 };

#define CT_MAX_KRYLOV 128

void ct_seterr(ct_handle* h, const char* fmt, ...);

// process-wide count of kernel launches issued by this library
extern std::atomic<long long> g_ct_launches;
static inline void ct_note_launch() { g_ct_launches.fetch_add(1, std::memory_order_relaxed); }

#define CT_CUDA(h, x)                                                                      \
    do {                                                                                   \
        cudaError_t e_ = (x);                                                              \
        if (e_ != cudaSuccess) {                                                           \
            ct_seterr((h), "%s:%d %s -> %s", __FILE__, __LINE__, #x, cudaGetErrorString(e_)); \
            return CT_ERR_CUDA;                                                            \
        }                                                                                  \
    } while (0)

#define CT_TRY(x)                  \
    do {                           \
        int s_ = (x);              \
        if (s_ != CT_OK) return s_; \
    } while (0)

#define CT_LAUNCH_CHECK(h) CT_CUDA(h, cudaGetLastError())

static inline int64_t ct_cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }
static inline int64_t ct_round_up(int64_t a, int64_t b) { return ct_cdiv(a, b) * b; }

// Scratch arena: reserve() grows (synchronising) before carving; carve() hands
// out 256-byte aligned pieces in order.  A call's pieces live until the next
// reserve() of that handle.
struct Arena {
    ct_handle* h;
    size_t off = 0;
    explicit Arena(ct_handle* hh) : h(hh) {}
    template <class T>
    T* take(size_t count) {
        size_t bytes = (count * sizeof(T) + 255) & ~size_t(255);
        if (off + bytes > h->ws_cap) return nullptr;
        T* p = reinterpret_cast<T*>(h->ws + off);
        off += bytes;
        return p;
    }
};
int ct_reserve(ct_handle* h, size_t bytes);
static inline size_t ct_bytes(size_t count, size_t elem) { return (count * elem + 255) & ~size_t(255); }

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ double ct_warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float ct_warp_sumf(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum; every thread gets the result.  sm must hold >= 32 doubles.
template <int NT>
__device__ __forceinline__ double ct_block_sum(double v, double* sm) {
    v = ct_warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sm[wid] = v;
    __syncthreads();
    double r = 0.0;
    if (wid == 0) {
        r = (lane < NT / 32) ? sm[lane] : 0.0;
        r = ct_warp_sum(r);
        if (lane == 0) sm[0] = r;
    }
    __syncthreads();
    r = sm[0];
    return r;
}

// Sort key of a singular value for the descending rank kernels: NaN sorts last.
// Ranking compares keys with '>' and '==' (ties by index), which is a strict total
// order only without NaN; with it every comparison is false, several entries get
// the same rank and parts of the permutation are never written.
__device__ __forceinline__ double ct_rank_key(double s) { return isnan(s) ? -INFINITY : s; }

__device__ __forceinline__ void ct_set_status(int* st, int code) {
    if (st) atomicCAS(st, 0, code);
}

// kernels that belong to an early-terminating loop read this flag first
__device__ __forceinline__ bool ct_skip(const int* skip) { return skip != nullptr && *(volatile const int*)skip != 0; }

// ---------------------------------------------------------------------------
// internal entry points shared between translation units
// ---------------------------------------------------------------------------
struct GemmDesc {
    int64_t M, N, K;
    const double* A; int64_t sAm, sAk;
    const double* B; int64_t sBk, sBn;
    double* C; int64_t sCm, sCn;
    double alpha, beta;
    int64_t nb1, nb0;                      // batch = nb1 x nb0
    int64_t sA1, sA0, sB1, sB0, sC1, sC0;  // batch strides
    const int* skip;
    int tri;   // 0: full; 1: write only C tiles on or below the diagonal (symmetric C);
               // 2: A is lower triangular (A(m, k) = 0 for k > m), skip those k
    // set by the launcher: split-K partial sums (ksplit > 1) go to part[ks][M][N]
    int64_t ksplit;
    double* part;
};
int ct_gemm_f64_launch(ct_handle* h, const GemmDesc& g);

// out(o, j, i) = sum_k Wt[j, k] * in(o, k, i);  j = j1 * J0 + j0
struct MpoDesc {
    int64_t O, K, J, I;
    const double* in; int64_t sIo, sIk, sIi;
    double* out; int64_t sOo, sOi; int64_t J0, sOj1, sOj0;
    const double* Wt;   // device [J][K]
    const int* skip;
};
int ct_mpo_apply_f64_launch(ct_handle* h, const MpoDesc& m);

// W-matrix builders (device) for the contractions
int ct_build_w12(ct_handle* h, const double* W1, const double* W2, double* W12t, int64_t wL,
                 int64_t d, int64_t wM, int64_t wR);
int ct_build_wt_left(ct_handle* h, const double* W, double* Wt, int64_t wL, int64_t d, int64_t wR);
int ct_build_wt_right(ct_handle* h, const double* W, double* Wt, int64_t wL, int64_t d, int64_t wR);
// MPO x MPO and MPO x MPS site products (ct_mpo.cu)
int ct_mpo_compose_launch(ct_handle* h, const double* Wa, const double* Wb, double* Wout, int64_t wLa,
                          int64_t d_in, int64_t d_mid, int64_t wRa, int64_t wLb, int64_t d_out, int64_t wRb);
int ct_apply_mpo_launch(ct_handle* h, const double* A, const double* W, double* out, int64_t Dl, int64_t d,
                        int64_t Dr, int64_t wL, int64_t d_out, int64_t wR);

// vector kernels (ct_vec.cu)
int ct_reduce_dot(ct_handle* h, int64_t n, const double* x, const double* y, double* d_out,
                  const int* skip);
int ct_reduce_nrm2sq(ct_handle* h, int64_t n, const double* x, double* d_out, const int* skip);
int ct_scale_by_inv_sqrt(ct_handle* h, int64_t n, const double* x, double* y,
                         const double* d_nsq, const int* skip, int zero_code);
int ct_fill(ct_handle* h, double* x, int64_t n, double v);
// sets the status word to CT_ERR_NONFINITE when the device scalar *d_x is NaN or
// infinite (enqueued, no synchronisation; the caller's next status check sees it)
int ct_check_finite(ct_handle* h, const double* d_x, const int* skip);
int ct_copy(ct_handle* h, double* dst, const double* src, int64_t n);
int ct_permute_launch(ct_handle* h, const double* in, double* out, int rank, const int64_t* shape,
                      const int32_t* perm);
int ct_identity_env(ct_handle* h, double* E, int64_t w, int64_t D);
// E[w, Dk, Db] = delta(k, b) for k, b < min(Dk, Db) in every channel
int ct_identity_env_rect(ct_handle* h, double* E, int64_t w, int64_t Dk, int64_t Db);

// Lanczos pieces
int ct_lanczos_update(ct_handle* h, int64_t n, double* w, const double* vj, const double* vjm1,
                      int j, double beta_threshold, const int* skip);
int ct_lanczos_next(ct_handle* h, int64_t n, const double* w, double* vnext, int j, const int* skip);
int ct_lanczos_alpha(ct_handle* h, int64_t n, const double* vj, const double* w, int j,
                     const int* skip);
// (gate != null: the kernels run only when *gate != 0, set by the FP32 pass)
int ct_lanczos_reorth_pass(ct_handle* h, int64_t n, double* w, const double* V, int64_t ldv, int j,
                           double beta_threshold, const int* skip);
int ct_lanczos_update_nonorm(ct_handle* h, int64_t n, double* w, const double* vj, const double* vjm1, int j,
                             const int* skip);
// the same pass against an FP32 copy of the basis; v_{j+1} with its FP32 copy
int ct_lanczos_reorth_pass32(ct_handle* h, int64_t n, double* w, const float* V32, int64_t ldv, int j,
                             double beta_threshold, const int* skip, double ratio64);
int ct_lanczos_reorth_redo(ct_handle* h, int64_t n, double* w, const double* V, const float* V32, int64_t ldv, int j,
                           double beta_threshold, const int* skip);
int ct_lanczos_next32(ct_handle* h, int64_t n, const double* w, double* vnext, float* vnext32, int j,
                      const int* skip);
int ct_f64_to_f32(ct_handle* h, int64_t n, const double* x, float* y, const int* skip);
int ct_tridiag_eig(ct_handle* h, int max_iter, double tol, int max_rotations);
int ct_ritz(ct_handle* h, int64_t n, const double* V, int64_t ldv, double* out);

// SVD (ct_svd.cu)
struct SvdOut {
    int64_t chi = 0;
    double sum_s2_all = 0.0;  // sum of all min(m,n) s^2 (sorted order)
    double sum_s2_kept = 0.0;
    double min_pivot = 0.0;   // subspace split: smallest Cholesky pivot of the first pass,
    double min_pivot2 = 0.0;  // of the second pass,
    int chol_fail = 0;        // and whether a pivot was not positive
    int replaced = 0;         // rows replaced by the rank completion of a first visit
    int stale = 0;            // refused: more weight lost than the staleness bound allows
};
// tensor-core path (ct_tc.cu)
struct TcGemm;
int ct_tc_available(ct_handle* h);
