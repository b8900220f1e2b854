/*
 * ctdmrg.h -- C ABI of libctdmrg.so, the GB300 (sm_103a) two-site DMRG path.
 *
 * Conventions (the same as the reference's native shim, native/svd_shim.c:1-23):
 *   - every entry point returns an int status: CT_OK (0) or a negative CT_ERR_*;
 *   - every tensor pointer is a caller-owned DEVICE pointer to a row-major,
 *     contiguous FP64 array in the reference layouts
 *         MPS site  A[Dl, d, Dr]            (src/state/mps_state.mojo:13-49)
 *         MPO site  W[wl, d_in, d_out, wr]  (src/state/mpo_state.mojo:10-54)
 *         env       E[w, D_ket, D_bra]      (src/state/environments.mojo:110-131)
 *         theta     th[Dl, d, d, Dr]        (src/algorithms/dmrg.mojo:93-140)
 *     unless a parameter says it is a host pointer (suffix _host);
 *   - scratch memory is owned by the handle; a handle is not thread-safe,
 *     use one handle per host thread;
 *   - all work is enqueued on the handle's stream; entry points that return a
 *     host scalar synchronise that stream.
 *
 * Precision forms (ct_prec):
 *   CT_PREC_FP64    plain form, FP64 everywhere.
 *   CT_PREC_TF32X3  contractions on tcgen05 tensor cores in TF32 with
 *                   3xTF32 split compensation and FP32 accumulation; all
 *                   storage, Lanczos, eigensolve, SVD and reductions FP64.
 *   CT_PREC_FP64_TC (ct_gemm, ct_mps_expectation) FP64 products emulated on
 *                   the BF16 tensor cores: each operand row cut into 8 exact
 *                   7-bit slices, 36 slice products per FP64 product summed
 *                   exactly in FP32 per 512 of K, combined in FP64; about as
 *                   accurate as an FP64 GEMM (~3e-15 of |A||B|).
 */
#ifndef CTDMRG_H
#define CTDMRG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CTDMRG_VERSION 1

#if defined(__GNUC__)
#define CT_API __attribute__((visibility("default")))
#else
#define CT_API
#endif

enum ct_status {
    CT_OK = 0,
    CT_ERR_INVALID = -1,     /* bad argument (null pointer, bad enum)            */
    CT_ERR_CUDA = -2,        /* a CUDA runtime call failed                       */
    CT_ERR_OOM = -3,         /* device allocation failed / allocation limit hit  */
    CT_ERR_NOCONV = -4,      /* an iterative device solver hit its iteration cap */
    CT_ERR_ZERO_NORM = -5,   /* Lanczos start vector has zero norm               */
    CT_ERR_SHAPE = -6,       /* inconsistent shapes                              */
    CT_ERR_UNSUPPORTED = -7, /* shape/precision not supported by this library    */
    CT_ERR_NONFINITE = -8,   /* NaN/Inf in an input norm or an eigenvalue         */
    CT_ERR_EMPTY = -9,       /* truncation kept zero singular values             */
    CT_ERR_TOO_LARGE = -10   /* problem exceeds the static scratch of a no-alloc entry */
};

enum ct_prec { CT_PREC_FP64 = 0, CT_PREC_TF32X3 = 1, CT_PREC_FP64_TC = 2 };

typedef struct ct_handle ct_handle;

/* ---- lifecycle (no reference counterpart: MAX's DeviceContext, dmrg.mojo:2) */
CT_API int ct_create(int device, void* stream, ct_handle** out);
CT_API int ct_destroy(ct_handle* h);
CT_API int ct_set_stream(ct_handle* h, void* stream);
CT_API int ct_synchronize(ct_handle* h);
/* reads and clears the device status word (sticky first error of a kernel) */
CT_API int ct_get_status(ct_handle* h, int* status_out);
CT_API const char* ct_error_string(int status);
CT_API const char* ct_last_error(ct_handle* h);
CT_API int ct_version(void);
/* number of kernels this library has launched in the process (all handles) */
CT_API int64_t ct_launch_count(void);
/* bytes of handle-owned scratch currently reserved */
CT_API int ct_workspace_bytes(ct_handle* h, int64_t* bytes_out);
/* Jacobi sweeps of the last SVD split on this handle and the running total */
CT_API int ct_svd_sweeps(ct_handle* h, int* last_host, int64_t* total_host);
/* cap on handle-owned scratch in bytes (0 = unlimited); growth beyond it -> CT_ERR_OOM */
CT_API int ct_set_workspace_limit(ct_handle* h, int64_t bytes);
/* cap on the one-sided Jacobi sweeps of every SVD on this handle (0 = the
 * built-in caps, 60 for one-CTA problems and 48 for the cooperative kernel;
 * larger values are clamped to those).  A split that has not converged within
 * the cap returns CT_ERR_NOCONV, the counterpart of LAPACK dgesdd's info > 0,
 * which the reference turns into an error (src/mylinalg/svd.mojo:74-76).     */
CT_API int ct_set_svd_max_sweeps(ct_handle* h, int max_sweeps);

/* ---- dense tensor core (src/m_tensor/dense_tensor.mojo) --------------------
 * Row-major C[m,n] = alpha * op(A) op(B) + beta * C, op = identity or transpose.
 * The 2-D core of dense_tensor_dot (dense_tensor.mojo:963-1328); the axis
 * bookkeeping of dense_tensor_dot lives in the host layer.               */
CT_API int ct_gemm(ct_handle* h, int prec, int trans_a, int trans_b, int64_t m, int64_t n, int64_t k,
            double alpha, const double* A, int64_t lda, const double* B, int64_t ldb,
            double beta, double* C, int64_t ldc);
/* out[i] = in[perm-index] : physical N-D permute, rank <= 6
 * (DenseTensor.transpose, dense_tensor.mojo:460-545)                       */
CT_API int ct_permute(ct_handle* h, const double* in, double* out, int rank, const int64_t* shape,
               const int32_t* perm);
/* vector ops (dense_tensor.mojo:637-754): FP64 reductions on the device   */
CT_API int ct_vec_dot(ct_handle* h, int64_t n, const double* x, const double* y, double* result_host);
CT_API int ct_vec_norm_sq(ct_handle* h, int64_t n, const double* x, double* result_host);
CT_API int ct_vec_axpy(ct_handle* h, int64_t n, double alpha, const double* x, double* y);
CT_API int ct_vec_scale(ct_handle* h, int64_t n, double alpha, double* x);
/* identity boundary environment E[w, D, D] (dmrg.mojo:74-84)              */
CT_API int ct_env_identity(ct_handle* h, double* E, int64_t w, int64_t D);

/* ---- two-site DMRG building blocks (src/algorithms/dmrg.mojo) ------------ */
/* theta[Dl,d,d,Dr] = A_i[Dl*d, Dm] . A_ip1[Dm, d*Dr]  (build_two_site_theta, dmrg.mojo:93-140) */
CT_API int ct_theta2(ct_handle* h, int prec, const double* A_i, const double* A_ip1, double* theta,
              int64_t Dl, int64_t d, int64_t Dm, int64_t Dr);
/* out = H_eff theta (apply_two_site_heff, dmrg.mojo:254-374).
 * L[wL,Dl,Dl], R[wR,Dr,Dr], W1[wL,d,d,wM], W2[wM,d,d,wR].                  */
CT_API int ct_heff2_apply(ct_handle* h, int prec, const double* theta, const double* L, const double* R,
                   const double* W1, const double* W2, double* out, int64_t Dl, int64_t d,
                   int64_t Dr, int64_t wL, int64_t wM, int64_t wR);
/* Lnext[wR,Dr,Dr] from Lprev[wL,Dl,Dl], A[Dl,d,Dr], W[wL,d,d,wR]
 * (update_left_environment, environments.mojo:99-201)                      */
CT_API int ct_env_left(ct_handle* h, int prec, const double* Lprev, const double* A, const double* W,
                double* Lnext, int64_t Dl, int64_t d, int64_t Dr, int64_t wL, int64_t wR);
/* Rprev[wL,Dl,Dl] from Rnext[wR,Dr,Dr], A[Dl,d,Dr], W[wL,d,d,wR]
 * (update_right_environment, environments.mojo:309-417)                    */
CT_API int ct_env_right(ct_handle* h, int prec, const double* Rnext, const double* A, const double* W,
                 double* Rprev, int64_t Dl, int64_t d, int64_t Dr, int64_t wL, int64_t wR);
/* Lanczos ground state of H_eff (lanczos_two_site_optimize, dmrg.mojo:486-756).
 * theta_in is not modified; theta_out gets the normalised Ritz vector.
 * max_rotations: Jacobi rotation cap of the tridiagonal eigensolve (the
 * reference uses 200, dmrg.mojo:510); 0 = run the same Jacobi to convergence.
 * reorth != 0 adds full FP64 reorthogonalisation against the Krylov basis.
 * alpha_host/beta_host (may be NULL) receive max_iter / max_iter-1 values.  */
CT_API int ct_lanczos2(ct_handle* h, int prec, const double* theta_in, double* theta_out,
                const double* L, const double* R, const double* W1, const double* W2,
                int64_t Dl, int64_t d, int64_t Dr, int64_t wL, int64_t wM, int64_t wR,
                int max_iter, double tol, int max_rotations, int reorth,
                double* energy_host, int* numiter_host, double* alpha_host, double* beta_host);
/* Truncated thin SVD of a row-major M[m,n] on the device
 * (dense_tensor_svd_trunc_lapack_f64, dense_tensor.mojo:1483-1592).
 * Writes the kept factors compactly: U[m, chi], S[chi], Vt[chi, n] (row-major,
 * capacity k = min(m,n) for chi), chi chosen by the reference rule.         */
CT_API int ct_svd_trunc(ct_handle* h, const double* M, int64_t m, int64_t n, int64_t chi_max,
                 double eps_trunc, double* U, double* S, double* Vt, int64_t* chi_host);
/* Thin QR of a row-major A[m,n] on the device, FP64 (dense_tensor_qr,
 * dense_tensor.mojo:1333-1433): Q[m,k] with orthonormal columns, R[k,n] upper
 * triangular (trapezoidal for n > m), k = min(m,n), diag(R) >= 0.  LAPACK's
 * Householder factors equal these up to the signs of Q's columns and R's rows
 * (the reference's own tests check the properties only).  Columns dependent on
 * the ones before them get completed Q columns; *completed_host (may be NULL)
 * returns how many.                                                          */
CT_API int ct_qr(ct_handle* h, const double* A, int64_t m, int64_t n, double* Q, double* R, int* completed_host);
/* Two-site split (split_two_site_theta_svd, dmrg.mojo:143-252).
 * A_out[Dl,d,chi], B_out[chi,d,Dr] (capacity min(Dl*d, d*Dr) for chi),
 * S_out (may be NULL) gets the kept singular values, descending.
 * prec CT_PREC_FP64: one-sided Jacobi in FP64.  CT_PREC_TF32X3 (problems too
 * large for one CTA): FP32 Jacobi for the subspace, FP64 re-orthonormalised
 * canonical factor, tensor-core projection for the centre factor.         */
CT_API int ct_svd_split(ct_handle* h, int prec, const double* theta, int64_t Dl, int64_t d, int64_t Dr,
                 int64_t chi_max, double eps_trunc, int left_to_right, double* A_out,
                 double* B_out, double* S_out, int64_t* chi_host, double* discarded_host);

/* ---- sweep driver (dmrg_two_site, dmrg.mojo:377-483) ---------------------- */
typedef struct ct_dmrg_params {
    int num_sweeps;
    int chi_max;
    double eps_trunc;
    int max_krylov_iter;
    double krylov_tol;
    double energy_tol;
    int two_site;        /* must be 1 (dmrg.mojo:416-417)                      */
    int verbose;
    int prec;            /* ct_prec                                            */
    int max_rotations;   /* 200 = reference Jacobi cap; 0 = converged          */
    int reorth;          /* full FP64 reorthogonalisation (always on in the mixed form) */
    int final_rayleigh;  /* also return <psi|H|psi>/<psi|psi> of the final MPS,
                            contracted in FP64 (stats.energy_rayleigh)          */
    int keep_bases;      /* mixed form: the first half-sweep's large splits may
                            start from the bond bases kept by the previous call
                            on this handle.  Only valid when the MPS passed in
                            is the one that call returned and the MPO is the
                            same; 0 forgets them at the start of the call.     */
    int split_power_steps; /* mixed form, bonds where chi_max binds: power steps
                            of the warm-started subspace split (0 is enough
                            for |dE/E| <= 1e-9 on the benchmark chain); -1
                            always runs the Jacobi SVD instead                */
    int cold_power_steps;  /* mixed form, a large bond with no kept basis (first
                            visit, or chi_max just raised): -1 runs the Jacobi
                            SVD; >= 0 runs the subspace split from the rows the
                            bond kept at a smaller chi (if any) plus random
                            Gaussian rows, with this many power steps first
                            (2 or more: the truncation of that first visit is
                            then close to, not equal to, the SVD's)          */
} ct_dmrg_params;

typedef struct ct_dmrg_stats {
    double seconds_total;      /* host wall clock of the call                   */
    double seconds_lanczos;    /* summed device time (CUDA events) per phase    */
    double seconds_svd;
    double seconds_env;
    double heff_flops;         /* algorithmic FLOPs of all H_eff applies        */
    double env_flops;
    int64_t heff_applies;
    int64_t local_updates;
    double max_discarded;      /* largest discarded weight over the run         */
    double energy_rayleigh;    /* FP64 Rayleigh quotient (NaN unless requested)  */
    int64_t subspace_splits;   /* mixed form: warm-started subspace splits      */
    int64_t exact_splits;      /* Jacobi-SVD splits                              */
    double seconds_subspace;   /* part of seconds_svd spent in subspace splits   */
    int64_t cold_splits;       /* subspace splits started from random rows       */
    int64_t completed_rows;    /* rows a first visit's rank completion replaced  */
    double seconds_rayleigh;   /* the final FP64 <H> (final_rayleigh), included in seconds_total */
    int64_t stale_retries;     /* warm splits retried with one more power step   */
    int64_t fp64_handovers;    /* mixed form: splits handed to the FP64 Jacobi
                                  because eps_trunc may decide chi               */
} ct_dmrg_stats;

/* Runs the sweeps in place.  mps_sites[i] are caller-owned device buffers of
 * capacity site_capacity[i] doubles; bond_dims (length nsites+1) is read and
 * updated.  mpo_sites[i] are device pointers, mpo_dims (length nsites+1) the
 * MPO bond dimensions.  sweep_energies_host (length num_sweeps, may be NULL)
 * gets the energy of every sweep run; discarded_host (length
 * num_sweeps*2*(nsites-1), may be NULL) every local discarded weight.      */
CT_API int ct_dmrg_two_site(ct_handle* h, const ct_dmrg_params* params, int nsites, int d,
                     const int64_t* mpo_dims, const double* const* mpo_sites,
                     int64_t* bond_dims, double* const* mps_sites,
                     const int64_t* site_capacity, double* energy_host,
                     double* sweep_energies_host, int* sweeps_done_host,
                     double* discarded_host, ct_dmrg_stats* stats_host);

/* Right-canonicalise an MPS in place with device SVD splits (no truncation);
 * site 0 is normalised.  No reference counterpart that works
 * (mps_state.mojo:170-217 is dead code); the configs ask for a
 * right-normalised start.                                                   */
CT_API int ct_mps_right_normalize(ct_handle* h, int nsites, int d, int64_t* bond_dims,
                           double* const* mps_sites);

/* <psi|H|psi> and <psi|psi> through left environments on the device
 * (expectation_value, environments.mojo:475-532).  prec CT_PREC_FP64: SIMT
 * FP64 GEMMs; CT_PREC_FP64_TC: the environment GEMMs on the BF16 tensor
 * cores with FP64-accurate slicing (the mixed form's final Rayleigh
 * quotient); CT_PREC_TF32X3 is taken as CT_PREC_FP64.                       */
CT_API int ct_mps_expectation(ct_handle* h, int prec, int nsites, int d, const int64_t* mpo_dims,
                       const double* const* mpo_sites, const int64_t* bond_dims,
                       const double* const* mps_sites, double* energy_host, double* norm_sq_host);

/* ---- observables with two different states (FP64 form) -------------------
 * One left-environment step with bra != ket:
 *   Lnext[wR,Drk,Drb] = sum Lprev[wL,Dlk,Dlb] A_ket[Dlk,s,Drk] W[wL,s,s',wR] A_bra[Dlb,s',Drb]
 * (update_left_environment_two_mps, environments.mojo:535-590).  With
 * W == NULL (wL = wR = 1) it is the overlap transfer step
 * Lprev[Dlk,Dlb] -> Lnext[Drk,Drb] of _mps_contraction_step_left
 * (environments.mojo:767-862).  prec must be CT_PREC_FP64.                   */
CT_API int ct_env_left2(ct_handle* h, int prec, const double* Lprev, const double* A_ket, const double* A_bra,
                        const double* W, double* Lnext, int64_t Dl_ket, int64_t Dl_bra, int64_t d,
                        int64_t Dr_ket, int64_t Dr_bra, int64_t wL, int64_t wR);

/* <bra|mpo|ket> (expectation_value_two_mps, environments.mojo:698-730) or,
 * with mpo_sites == NULL, <bra|ket> (mps_vdot_direct / mps_overlap,
 * environments.mojo:971-1025).  The left boundary is the identity over
 * min(ket_dims[0], bra_dims[0]); the final environment must be a scalar
 * (CT_ERR_SHAPE otherwise, where the reference raises).                     */
CT_API int ct_mps_expectation2(ct_handle* h, int prec, int nsites, int d, const int64_t* mpo_dims,
                               const double* const* mpo_sites, const int64_t* bra_dims,
                               const double* const* bra_sites, const int64_t* ket_dims,
                               const double* const* ket_sites, double* value_host);

/* One site of mpo_compose (environments.mojo:1086-1132):
 *   Wout[(al,bl), i, o, (ar,br)] = sum_m Wa[al,i,m,ar] Wb[bl,m,o,br]        */
CT_API int ct_mpo_compose_site(ct_handle* h, const double* Wa, const double* Wb, double* Wout, int64_t wLa,
                               int64_t d_in, int64_t d_mid, int64_t wRa, int64_t wLb, int64_t d_out,
                               int64_t wRb);

/* One site of apply_mpo (environments.mojo:1135-1189):
 *   out[(w,a), t, (v,b)] = sum_s A[a,s,b] W[w,s,t,v]                         */
CT_API int ct_apply_mpo_site(ct_handle* h, const double* A, const double* W, double* out, int64_t Dl,
                             int64_t d, int64_t Dr, int64_t wL, int64_t d_out, int64_t wR);

/* ---- host-side seeded initial state (rng_c_compat.mojo:14-231) ------------
 * Fills HOST buffers: sites[i] gets dims[i]*d*dims[i+1] doubles holding the
 * float32 values of create_random_mps_c_compatible; dims (length nsites+1)
 * is written.  With sites_host == NULL only dims is computed.               */
CT_API int ct_random_mps_host(int nsites, int d, int chi_max, uint64_t seed, int64_t* dims,
                       double* const* sites_host);
/* first n values of randnf() for a seed (used by tests)                    */
CT_API int ct_rng_randnf_host(uint64_t seed, int64_t n, float* out);

/* ---- adjoint energy gradient (no reference counterpart) -------------------
 * Gradient of E(A) = <psi|H|psi>/<psi|psi> with respect to every site tensor
 * of a (not necessarily canonical) MPS, by the hand-written adjoint of the
 * environment chain.  grad_sites[i] are caller-owned device buffers shaped
 * like mps_sites[i].  checkpoint_every > 0 stores only every k-th left
 * environment and recomputes the others (memory ~ L/k environments).
 * prec CT_PREC_FP64: FP64 throughout.  CT_PREC_TF32X3: environments and
 * one-site effective Hamiltonians on the tensor cores (FP32-level products).
 * Every environment is rescaled by a power of two after each step, so
 * unnormalised chains neither under- nor overflow.                        */
CT_API int ct_energy_grad(ct_handle* h, int prec, int nsites, int d, const int64_t* mpo_dims,
                   const double* const* mpo_sites, const int64_t* bond_dims,
                   const double* const* mps_sites, double* const* grad_sites,
                   int checkpoint_every, double* energy_host);

/* Warm-started split of theta[Dl,d,d,Dr] into exactly chi states, the mixed
 * form's replacement of ct_svd_split on bonds where chi_max binds (no
 * reference counterpart: the reference always runs a full SVD).  basis_in
 * holds chi orthonormal rows kept by the previous visit of the bond from the
 * other direction: rows over (s_{i+1}, a_{i+1}) (chi x d*Dr) for a
 * left-to-right split, over (a_{i-1}, s_i) (chi x Dl*d) for a right-to-left
 * one.  power_steps >= 0 refines the basis before the split.
 * Writes A [Dl,d,chi], B [chi,d,Dr] (A left-canonical for
 * left_to_right, B right-canonical otherwise) and the basis this split keeps
 * (chi x Dl*d, resp. chi x d*Dr) to basis_out.  *accepted = 0 when the
 * basis no longer tracks theta's dominant subspace (outputs not valid: use
 * ct_svd_split).  pivots_host (3 doubles, may be NULL): the smallest Cholesky
 * pivot of each CholeskyQR pass and a failure flag.  Requires the tensor
 * cores (CT_ERR_UNSUPPORTED otherwise).                                     */
CT_API int ct_svd_split_warm(ct_handle* h, const double* theta, int64_t Dl, int64_t d, int64_t Dr, int64_t chi,
                             int left_to_right, const double* basis_in, int power_steps,
                             double* basis_out, double* A_out, double* B_out, int* accepted,
                             double* discarded_host, double* pivots_host);

/* ---- allocation-free H_eff apply (no counterpart in the reference) --------
 * For callers that cannot let a library allocate device memory, e.g. a Mojo/MAX
 * host whose DeviceContext allocator owns every buffer, or a caller under a
 * fixed device-memory budget.  Same FP64 result as ct_heff2_apply (same
 * kernels), enqueued on `stream`; takes no handle and calls no cudaMalloc.
 * Its intermediates live in one static device array of
 * CT_NOALLOC_SCRATCH_DOUBLES doubles (16 MiB) held by every GPU that loads the
 * library until exit; sizes that need more than that
 * (T1 + T3 = 2 * Dl*d*d*Dr*max(wL,wR) doubles, plus the fused MPO matrix)
 * return CT_ERR_TOO_LARGE.  The first call on a device looks up the array's
 * address (make it before any stream capture).  All calls share the array:
 * calls that overlap on the GPU race.                                       */
#define CT_NOALLOC_SCRATCH_DOUBLES (1u << 21)
CT_API int ct_heff2_apply_noalloc(void* stream, const double* theta, const double* L, const double* R,
                                  const double* W1, const double* W2, double* out, int64_t Dl, int64_t d,
                                  int64_t Dr, int64_t wL, int64_t wM, int64_t wR);

/* ---- measurement hook (no reference counterpart) --------------------------
 * Average device time of one launch of the TF32x3 tcgen05 GEMM kernel on an
 * m x n x k problem with operands already split and resident in HBM.       */
CT_API int ct_tc_gemm_time(ct_handle* h, int64_t m, int64_t n, int64_t k, int reps, double* ms_per_launch);

/* The TF32x3 GEMM launcher's plan for a plain m x n x k product on num_sms
 * SMs, computed on the host (no device needed): out[0] tile width (128, 192,
 * 224 or 256), out[1] 1 when C^T = B A^T is computed instead, out[2] tiles,
 * out[3] whole tiles of the hybrid schedule, out[4] CTAs sharing the stream-K
 * k-blocks (0: no stream-K part), out[5] stream-K k-blocks, out[6] most pieces
 * of one stream-K tile, out[7] k-blocks (32 of K) per tile. */
CT_API int ct_tc_gemm_plan(int64_t m, int64_t n, int64_t k, int num_sms, int64_t* out);

/* Live timing of the tensor-core GEMM inside real work (no reference
 * counterpart).  ct_kernel_timing(h, 1) resets the totals and makes every
 * TF32x3 GEMM launch on h record a CUDA event pair on h's stream;
 * ct_kernel_timing_read waits for the recorded launches and returns their
 * count, summed device milliseconds and summed algorithmic FLOPs
 * (2 M N K, K rounded up to 32).  ct_kernel_timing(h, 0) stops recording. */
CT_API int ct_kernel_timing(ct_handle* h, int enable);
CT_API int ct_kernel_timing_read(ct_handle* h, int64_t* launches, double* ms, double* flops);
/* Same per class: 0 = TF32x3 GEMM launches (as above), 1 = whole H_eff applies
 * inside Lanczos (FLOPs = 4 D d^2 chi^3 + 4 D^2 d^3 chi^2 per apply, as in
 * ct_dmrg_stats.heff_flops), 2 = the applies of class 1 with the largest FLOP
 * count seen (the centre bond at chi_max), 3 = the Krylov vector work of each
 * reorthogonalised Lanczos step (algorithmic bytes in place of FLOPs), 4 = the
 * FP64 GEMM launches on the BF16 tensor cores (2 M N K).                     */
CT_API int ct_kernel_timing_read_class(ct_handle* h, int cls, int64_t* count, double* ms, double* flops);

#ifdef __cplusplus
}
#endif

#endif /* CTDMRG_H */
