// Device SVD split: one-sided (Hestenes) Jacobi in FP64 + the reference's
// truncation rule, replacing the host LAPACK dgesdd round trip of
// dense_tensor_svd_trunc_lapack_f64 (dense_tensor.mojo:1483-1592) and the
// host-side S absorption of split_two_site_theta_svd (dmrg.mojo:143-252).
//
// The factor that must come out orthonormal is the one that is accumulated:
//   left-to-right  (A = U, B = S Vt): rotate the ROWS of M; the accumulated
//                  rotations are U, the rotated rows are S Vt;
//   right-to-left  (A = U S, B = Vt): rotate the COLUMNS of M; the
//                  accumulated rotations are V, the rotated columns are U S.
// No division by a singular value is needed in either sweep direction.
//
// Small problems run in one CTA with everything in shared memory (no host
// round trip); large ones run one launch per round-robin round, n/2 pairs in
// parallel, with a rotation counter read back once per sweep.
#include "ct_ops.cuh"
#include "ct_jacobi_coop.cuh"

namespace {

constexpr int SVD_NT = 256;
constexpr int SVD_MAX_SWEEPS = 60;
constexpr int FL_SVD_SWEEPS = 19;   // d_flags slot: sweeps of the last Jacobi (the cooperative one's too)
constexpr double SVD_EPS2 = 2.2204460492503131e-16 * 2.2204460492503131e-16;

__device__ __forceinline__ void tournament_pair(int P, int r, int k, int& p, int& q) {
    if (k == 0) {
        p = P - 1;
        q = r;
    } else {
        p = (r + k) % (P - 1);
        q = (r - k + (P - 1)) % (P - 1);
    }
}

// Rotation that orthogonalises two vectors with |x_p|^2=a, |x_q|^2=b, <x_p,x_q>=c.
// Vectors with |x|^2 <= floor (numerically zero next to |M|_F) are left alone:
// rotating rounding noise never converges.
__device__ __forceinline__ bool jacobi_rot(double a, double b, double c, double tol, double floor, double& cs,
                                           double& sn) {
    if (a <= floor || b <= floor) return false;
    if (c == 0.0 || !(fabs(c) > tol * sqrt(a * b))) return false;
    const double zeta = (b - a) / (2.0 * c);
    double t;
    if (fabs(zeta) > 1e150) t = 0.5 / zeta;
    else t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
    cs = 1.0 / sqrt(1.0 + t * t);
    sn = cs * t;
    return true;
}

// ---- init: X (nvec x len) from M, Q = I ---------------------------------------
__global__ void svd_init_kernel(const double* M, int64_t m, int64_t n, int cols, double* X, int64_t ldx,
                                double* Q, int64_t nvec) {
    const int64_t len = cols ? m : n;
    const int64_t tot = nvec * len;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = t / len, e = t % len;
        X[v * ldx + e] = cols ? M[e * n + v] : M[v * n + e];
    }
    const int64_t tq = nvec * nvec;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < tq; t += (int64_t)gridDim.x * blockDim.x)
        Q[t] = ((t / nvec) == (t % nvec)) ? 1.0 : 0.0;
}

// ---- small path: whole Jacobi in one CTA, X and Q in shared memory ------------
__global__ void __launch_bounds__(SVD_NT) svd_small_kernel(double* Xg, int64_t len, int64_t ldx, double* Qg,
                                                           int nvec, double tol, int max_sweeps, int* status,
                                                           int* sweeps_out) {
    extern __shared__ double ssm[];
    double* X = ssm;                         // nvec x len
    double* Q = ssm + (int64_t)nvec * len;   // nvec x nvec
    for (int64_t t = threadIdx.x; t < (int64_t)nvec * len; t += SVD_NT) X[t] = Xg[(t / len) * ldx + t % len];
    for (int64_t t = threadIdx.x; t < (int64_t)nvec * nvec; t += SVD_NT) Q[t] = Qg[t];
    __syncthreads();
    __shared__ double red[32];
    double f2 = 0.0;
    for (int64_t t = threadIdx.x; t < (int64_t)nvec * len; t += SVD_NT) f2 = fma(X[t], X[t], f2);
    const double floor = SVD_EPS2 * ct_block_sum<SVD_NT>(f2, red);
    const int P = nvec + (nvec & 1);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = SVD_NT / 32;
    bool converged = false;
    int sweep = 0;
    for (; sweep < max_sweeps; ++sweep) {
        int rotated = 0;
        for (int r = 0; r < P - 1; ++r) {
            for (int k = warp; k < P / 2; k += nw) {
                int p, q;
                tournament_pair(P, r, k, p, q);
                if (p >= nvec || q >= nvec) continue;
                double* xp = X + (int64_t)p * len;
                double* xq = X + (int64_t)q * len;
                double a = 0.0, b = 0.0, c = 0.0;
                for (int64_t i = lane; i < len; i += 32) {
                    const double u = xp[i], v = xq[i];
                    a = fma(u, u, a);
                    b = fma(v, v, b);
                    c = fma(u, v, c);
                }
                a = ct_warp_sum(a);
                b = ct_warp_sum(b);
                c = ct_warp_sum(c);
                double cs, sn;
                if (jacobi_rot(a, b, c, tol, floor, cs, sn)) {
                    rotated = 1;
                    for (int64_t i = lane; i < len; i += 32) {
                        const double u = xp[i], v = xq[i];
                        xp[i] = cs * u - sn * v;
                        xq[i] = sn * u + cs * v;
                    }
                    double* qp = Q + (int64_t)p * nvec;
                    double* qq = Q + (int64_t)q * nvec;
                    for (int i = lane; i < nvec; i += 32) {
                        const double u = qp[i], v = qq[i];
                        qp[i] = cs * u - sn * v;
                        qq[i] = sn * u + cs * v;
                    }
                }
                __syncwarp();
            }
            __syncthreads();
        }
        if (!__syncthreads_or(rotated)) {
            converged = true;
            ++sweep;
            break;
        }
    }
    if (threadIdx.x == 0) {
        *sweeps_out = sweep;
        if (!converged) ct_set_status(status, CT_ERR_NOCONV);
    }
    __syncthreads();
    for (int64_t t = threadIdx.x; t < (int64_t)nvec * len; t += SVD_NT) Xg[(t / len) * ldx + t % len] = X[t];
    for (int64_t t = threadIdx.x; t < (int64_t)nvec * nvec; t += SVD_NT) Qg[t] = Q[t];
}

// sigma_j = |x_j|, one warp per vector
__global__ void svd_norms_kernel(const double* X, int64_t len, int64_t ldx, int64_t nvec, double* sig) {
    const int64_t v = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x & 31;
    if (v >= nvec) return;
    double a = 0.0;
    for (int64_t i = lane; i < len; i += 32) {
        const double u = X[v * ldx + i];
        a = fma(u, u, a);
    }
    a = ct_warp_sum(a);
    if (lane == 0) sig[v] = sqrt(a);
}

// descending order, ties by index: perm[rank(j)] = j
__global__ void svd_rank_kernel(const double* sig, int64_t nvec, int* perm) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nvec) return;
    const double sj = ct_rank_key(sig[j]);
    int64_t rank = 0;
    for (int64_t i = 0; i < nvec; ++i) {
        const double si = ct_rank_key(sig[i]);
        if (si > sj || (si == sj && i < j)) ++rank;
    }
    perm[rank] = (int)j;
}

// chi rule of dense_tensor.mojo:1528-1548, FP64, sequential sums in sorted order
__global__ void svd_trunc_kernel(const double* sig, const int* perm, int64_t k, int64_t chi_max, double eps,
                                 double* scalars, int* flags) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int64_t chi = k < chi_max ? k : chi_max;
    double total = 0.0, kept_at = 0.0;
    for (int64_t i = 0; i < k; ++i) {
        const double s = sig[perm[i]];
        total += s * s;
    }
    if (eps > 0.0 && k > 0) {
        if (total <= 0.0) {
            chi = 0;
        } else {
            double kept = 0.0;
            const int64_t limit = k < chi_max ? k : chi_max;
            chi = limit;
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
    for (int64_t i = 0; i < chi; ++i) {
        const double s = sig[perm[i]];
        kept_at += s * s;
    }
    scalars[SC_SVD_MINKEPT] = chi > 0 ? sig[perm[chi - 1]] : 0.0;
    flags[FL_CHI] = (int)chi;
    scalars[SC_TMP0] = total;
    scalars[SC_TMP1] = kept_at;
}

// outputs; vectors = rows (cols=0) or columns (cols=1) of M
__global__ void svd_gather_kernel(const double* X, int64_t ldx, const double* Q, int64_t ldq, const double* sig,
                                  const int* perm, const int* flags, int64_t m, int64_t n, int cols, int mode,
                                  double* A, double* B, double* S) {
    const int64_t chi = flags[FL_CHI];
    // A: m x chi
    const int64_t totA = m * chi;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < totA; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = t / chi, c = t % chi;
        const int64_t v = perm[c];
        double val;
        if (!cols) {
            val = Q[v * ldq + r];                        // U
            if (mode == 1) val *= sig[v];                // U S
        } else {
            val = X[v * ldx + r];                        // U S
            if (mode == 0 || mode == 2) {                // U
                const double s = sig[v];
                val = (s > 0.0) ? val / s : 0.0;
            }
        }
        A[t] = val;
    }
    // B: chi x n
    const int64_t totB = chi * n;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < totB; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = t / n, x = t % n;
        const int64_t v = perm[c];
        double val;
        if (!cols) {
            val = X[v * ldx + x];                        // S Vt
            if (mode == 1 || mode == 2) {                // Vt
                const double s = sig[v];
                val = (s > 0.0) ? val / s : 0.0;
            }
        } else {
            val = Q[v * ldq + x];                        // Vt
            if (mode == 0) val *= sig[v];                // S Vt
        }
        B[t] = val;
    }
    if (S) {
        for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < chi; t += (int64_t)gridDim.x * blockDim.x)
            S[t] = sig[perm[t]];
    }
}

// ---- Householder QR preconditioning of the cooperative Jacobi -------------------
// Cyclic one-sided Jacobi needs 40-50 sweeps on vectors whose singular values decay
// geometrically over many decades (the spectrum of a converged DMRG bond; measured in
// a sweep-by-sweep model of this kernel: 38 sweeps for exp(-0.04 k), 47 for
// exp(-0.08 k) on 512 x 512), against ~11 for the rows of the triangular factor of a
// QR of the same vectors -- the QR preconditioning of Drmac and Veselic (New fast and
// accurate Jacobi SVD algorithm I, SIAM J. Matrix Anal. Appl. 29, 2008).
//
// X0 (nvec x len, vectors as rows) = Q2 R2 with Q2 (nvec x k) orthonormal and R2
// (k x len) upper trapezoidal, k = min(nvec, len).  The Jacobi rotates the k rows of
// R2, Y = J R2, so X0 = (Q2 J^T) Y: the accumulated factor of X0's vectors is
// Q2 J^T, orthonormal to rounding whatever the singular values are, and Y holds the
// other factor scaled by sigma, as without preconditioning.
//
// Work array T = X0^T (len x nvec): row j of T is column j of X0, contiguous, so every
// Householder step reads and updates contiguous rows.  Reflector j,
//   H_j = I - coef_j u u^T,  u = (0, .., 0, u0_j, T[j][j+1 .. nvec)),
// is built from row j after H_0 .. H_{j-1} and maps it to (R2[0..j-1][j], beta_j, 0..);
// T keeps the tail of u in place and refl holds (coef, u0, beta) for each j.
constexpr int QR_NT = 256;
constexpr int64_t QR_MAX_NVEC = 12288;      // reflector + one row in 200 KB of shared memory
constexpr size_t QR_SMEM_CAP = 200 * 1024;

// dst (cols x rows, row stride rows) = src (rows x cols, row stride lds)^T through 32 x 32
// tiles.  With diag: dst is R2's upper trapezoid, dst[i][c] = src[c][i] for c > i,
// diag[i] for c == i, 0 for c < i.
__global__ void transpose_kernel(const double* src, int64_t rows, int64_t cols, int64_t lds, double* dst,
                                 const double* diag) {
    __shared__ double tile[32][33];
    const int64_t r0 = (int64_t)blockIdx.y * 32, c0 = (int64_t)blockIdx.x * 32;
    for (int dy = threadIdx.y; dy < 32; dy += blockDim.y) {
        const int64_t r = r0 + dy, c = c0 + threadIdx.x;
        if (r < rows && c < cols) tile[dy][threadIdx.x] = src[r * lds + c];
    }
    __syncthreads();
    for (int dy = threadIdx.y; dy < 32; dy += blockDim.y) {
        const int64_t c = c0 + dy, r = r0 + threadIdx.x;
        if (r >= rows || c >= cols) continue;
        double v = tile[threadIdx.x][dy];
        if (diag) v = (r > c) ? v : (r == c ? diag[c] : 0.0);
        dst[c * rows + r] = v;
    }
}

// All k Householder steps in one cooperative launch.  Step j: every CTA stages row j
// of T in shared memory and derives the same reflector from it (same data, same
// reduction order), its warps apply it to the rows j+1 .. len-1 they own, and a grid
// barrier (bounded, as in the Jacobi) ends the step.
__global__ void __launch_bounds__(QR_NT) qr_coop_kernel(double* T, int64_t len, int64_t nvec, int64_t k,
                                                        double* refl, ct_jacobi::Sync s) {
    extern __shared__ double u[];
    __shared__ double red[32];
    const int lane = threadIdx.x & 31;
    const int64_t nw = (int64_t)gridDim.x * (QR_NT / 32);
    const int64_t gw = (int64_t)blockIdx.x * (QR_NT / 32) + (threadIdx.x >> 5);
    for (int64_t j = 0; j < k; ++j) {
        const double* tj = T + j * nvec + j;
        const int64_t tl = nvec - j;
        double s2 = 0.0;
        for (int64_t i = threadIdx.x; i < tl; i += QR_NT) {
            const double x = tj[i];
            u[i] = x;
            if (i > 0) s2 = fma(x, x, s2);
        }
        s2 = ct_block_sum<QR_NT>(s2, red);
        const double alpha = u[0];
        double coef = 0.0, u0 = 0.0, beta = alpha;
        if (s2 > 0.0) {   // an already reduced column keeps H_j = I
            const double nrm = sqrt(fma(alpha, alpha, s2));
            beta = alpha >= 0.0 ? -nrm : nrm;
            u0 = alpha - beta;
            coef = 1.0 / (nrm * (fabs(alpha) + nrm));
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            u[0] = u0;
            if (blockIdx.x == 0) {
                refl[j] = coef;
                refl[k + j] = u0;
                refl[2 * k + j] = beta;
            }
        }
        __syncthreads();
        if (coef != 0.0) {
            for (int64_t r = j + 1 + gw; r < len; r += nw) {
                double* tr = T + r * nvec + j;
                double d = 0.0;
                for (int64_t i = lane; i < tl; i += 32) d = fma(u[i], tr[i], d);
                d = ct_warp_sum(d) * coef;
                for (int64_t i = lane; i < tl; i += 32) tr[i] = fma(-d, u[i], tr[i]);
            }
        }
        if (j + 1 < k && !ct_jacobi::grid_barrier(s)) return;
    }
}

// Qn (k x nvec) = J Q2^T: row v is row v of J (k x k) padded with zeros to nvec,
// with H_{k-1} .. H_0 applied.  Each CTA holds `rows` rows and the current
// reflector in shared memory; one warp per row.
__global__ void __launch_bounds__(QR_NT) qr_form_kernel(const double* T, int64_t nvec, int64_t k,
                                                        const double* refl, const double* J, int rows, double* Qn) {
    extern __shared__ double sm[];
    double* u = sm;
    double* c = sm + nvec;
    const int64_t v0 = (int64_t)blockIdx.x * rows;
    const int nr = (int)((k - v0) < rows ? (k - v0) : rows);
    for (int64_t t = threadIdx.x; t < (int64_t)nr * nvec; t += QR_NT) {
        const int64_t r = t / nvec, i = t % nvec;
        c[t] = i < k ? J[(v0 + r) * k + i] : 0.0;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int64_t j = k - 1; j >= 0; --j) {
        const double coef = refl[j];
        if (coef == 0.0) continue;
        const int64_t tl = nvec - j;
        __syncthreads();
        for (int64_t i = threadIdx.x; i < tl; i += QR_NT) u[i] = i == 0 ? refl[k + j] : T[j * nvec + j + i];
        __syncthreads();
        for (int r = warp; r < nr; r += QR_NT / 32) {
            double* cr = c + (int64_t)r * nvec + j;
            double d = 0.0;
            for (int64_t i = lane; i < tl; i += 32) d = fma(u[i], cr[i], d);
            d = ct_warp_sum(d) * coef;
            for (int64_t i = lane; i < tl; i += 32) cr[i] = fma(-d, u[i], cr[i]);
        }
    }
    __syncthreads();
    for (int64_t t = threadIdx.x; t < (int64_t)nr * nvec; t += QR_NT) Qn[v0 * nvec + t] = c[t];
}

__global__ void identity_kernel(double* Q, int64_t n) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n * n; t += (int64_t)gridDim.x * blockDim.x)
        Q[t] = (t / n == t % n) ? 1.0 : 0.0;
}

}  // namespace

static void svd_geometry(int64_t m, int64_t n, int mode, int& cols, int64_t& nvec, int64_t& len) {
    // mode 0 (A=U, B=S Vt) rotates rows; mode 1 (A=U S, B=Vt) rotates columns;
    // mode 2 (U, S, Vt) rotates the shorter side.
    if (mode == 0) cols = 0;
    else if (mode == 1) cols = 1;
    else cols = (m > n) ? 1 : 0;
    nvec = cols ? n : m;
    len = cols ? m : n;
}

// the cooperative Jacobi runs on the QR-preconditioned vectors (see qr_coop_kernel)
static bool svd_uses_qr(int64_t nvec, int64_t len) {
    return nvec >= 2 && (nvec * len + nvec * nvec) * 8 > 200 * 1024 && nvec <= QR_MAX_NVEC;
}

size_t ct_svd_ws_bytes(int64_t m, int64_t n, int mode) {
    int cols;
    int64_t nvec, len;
    svd_geometry(m, n, mode, cols, nvec, len);
    const int64_t k = nvec < len ? nvec : len;
    size_t b = ct_bytes(nvec * len, 8) + ct_bytes(nvec * nvec, 8) + ct_bytes(nvec, 8) + ct_bytes(nvec, 4);
    if (svd_uses_qr(nvec, len)) b += ct_bytes(len * nvec, 8) + ct_bytes(3 * k, 8) + ct_bytes(k * nvec, 8);
    return b;
}

static void launch_transpose(ct_handle* h, const double* src, int64_t rows, int64_t cols, int64_t lds, double* dst,
                             const double* diag) {
    const dim3 grid((unsigned)ct_cdiv(cols, 32), (unsigned)ct_cdiv(rows, 32));
    transpose_kernel<<<grid, dim3(32, 8), 0, h->stream>>>(src, rows, cols, lds, dst, diag); ct_note_launch();
}

// QR-preconditioned Jacobi of the vectors of M (rows: cols = 0, columns: cols = 1).
// On return X (k x len) holds the rotated rows Y of R2 and *Qn_out (k x nvec, row
// stride nvec) the accumulated factor J Q2^T; k = min(nvec, len).
static int svd_qr_jacobi(ct_handle* h, Arena& ar, const double* M, int64_t m, int64_t n, int cols, int64_t nvec,
                         int64_t len, double tol, double* X, double* J, double** Qn_out) {
    const int64_t k = nvec < len ? nvec : len;
    double* T = ar.take<double>(len * nvec);
    double* refl = ar.take<double>(3 * k);
    double* Qn = ar.take<double>(k * nvec);
    if (!T || !refl || !Qn) return CT_ERR_OOM;
    // T = X0^T: M itself when the vectors are M's columns, M^T when they are its rows
    if (cols) CT_CUDA(h, cudaMemcpyAsync(T, M, sizeof(double) * m * n, cudaMemcpyDeviceToDevice, h->stream));
    else launch_transpose(h, M, m, n, n, T, nullptr);
    CT_LAUNCH_CHECK(h);

    static int attr_dev = -1;
    if (attr_dev != h->device) {
        CT_CUDA(h, cudaFuncSetAttribute(qr_coop_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)QR_SMEM_CAP));
        CT_CUDA(h, cudaFuncSetAttribute(qr_form_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)QR_SMEM_CAP));
        attr_dev = h->device;
    }
    {
        const size_t smem = (size_t)nvec * sizeof(double);
        int occ = 0;
        CT_CUDA(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, qr_coop_kernel, QR_NT, smem));
        int64_t grid = (int64_t)occ * h->num_sms;
        const int64_t need = ct_cdiv(len > 1 ? len - 1 : 1, QR_NT / 32);
        if (grid > need) grid = need;
        if (grid < 1) grid = 1;
        // grid barrier scratch in d_flags, as the Jacobi's: [16] count, [17] gen, [18] abort
        int* base = h->d_flags;
        CT_CUDA(h, cudaMemsetAsync(base + 16, 0, 4 * sizeof(int), h->stream));
        ct_jacobi::Sync sy;
        sy.count = (unsigned*)(base + 16);
        sy.gen = (unsigned*)(base + 17);
        sy.abort_flag = base + 18;
        sy.sweeps = base + 19;
        sy.rot = base + 32;
        sy.status = h->d_status;
        void* args[] = {&T, &len, &nvec, (void*)&k, &refl, &sy};
        CT_CUDA(h, cudaLaunchCooperativeKernel((const void*)qr_coop_kernel, dim3((unsigned)grid), dim3(QR_NT), args,
                                               smem, h->stream));
        ct_note_launch();
    }
    // R2 (k x len) into X, J = I
    launch_transpose(h, T, len, k, nvec, X, refl + 2 * k);
    identity_kernel<<<(unsigned)std::min<int64_t>(ct_cdiv(k * k, 256), 4 * (int64_t)h->num_sms), 256, 0,
                      h->stream>>>(J, k); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    double* d_frob2 = h->d_scalars + SC_TMP0;
    CT_TRY(ct_reduce_nrm2sq(h, k * len, X, d_frob2, nullptr));
    CT_TRY(ct_jacobi::run<double>(h, X, len, J, k, tol, SVD_EPS2, d_frob2, nullptr));
    {
        int64_t rows = (int64_t)(QR_SMEM_CAP / ((size_t)nvec * sizeof(double))) - 1;
        if (rows > QR_NT / 32) rows = QR_NT / 32;
        if (rows < 1) rows = 1;
        const size_t smem = (size_t)(rows + 1) * nvec * sizeof(double);
        qr_form_kernel<<<(unsigned)ct_cdiv(k, rows), QR_NT, smem, h->stream>>>(T, nvec, k, refl, J, (int)rows, Qn);
        ct_note_launch();
        CT_LAUNCH_CHECK(h);
    }
    *Qn_out = Qn;
    return CT_OK;
}

// The canonical factor of a split (U for mode 0, V^T for mode 1) is taken from the
// accumulated rotations when the Jacobi rotates that side, and from the rotated
// vectors X / sigma otherwise.  A converged one-sided Jacobi leaves the normalised
// vectors orthogonal to its tolerance whatever sigma is, so only an exactly zero
// kept sigma needs the rotations.  The Jacobi therefore rotates the shorter side
// (64 x 4: 6 pairs instead of 2016 per sweep, ~0.1 ms instead of ~5 ms), and runs
// again on the canonical side when a kept singular value is zero.
static int svd_run_geometry(ct_handle* h, Arena& ar, const double* M, int64_t m, int64_t n, int64_t chi_max,
                            double eps_trunc, int mode, int geo_mode, double* A, double* B, double* S, SvdOut* out,
                            double* min_kept);

int ct_svd_run(ct_handle* h, Arena& ar, const double* M, int64_t m, int64_t n, int64_t chi_max, double eps_trunc,
               int mode, double* A, double* B, double* S, SvdOut* out) {
    if (m <= 0 || n <= 0) {
        out->chi = 0;
        return CT_OK;
    }
    // (the QR-preconditioned Jacobi of a large canonical side rotates only min(m, n)
    // vectors, so it needs no short-side attempt)
    int ccols;
    int64_t cnvec, clen;
    svd_geometry(m, n, mode, ccols, cnvec, clen);
    const bool long_side = ((mode == 0 && m > n) || (mode == 1 && m < n)) && !svd_uses_qr(cnvec, clen);
    if (long_side) {
        const size_t mark = ar.off;
        double min_kept = 0.0;
        CT_TRY(svd_run_geometry(h, ar, M, m, n, chi_max, eps_trunc, mode, 2, A, B, S, out, &min_kept));
        if (out->chi == 0 || min_kept > 0.0) return CT_OK;
        ar.off = mark;
    }
    double unused = 0.0;
    return svd_run_geometry(h, ar, M, m, n, chi_max, eps_trunc, mode, mode, A, B, S, out, &unused);
}

static int svd_run_geometry(ct_handle* h, Arena& ar, const double* M, int64_t m, int64_t n, int64_t chi_max,
                            double eps_trunc, int mode, int geo_mode, double* A, double* B, double* S, SvdOut* out,
                            double* min_kept) {
    int cols;
    int64_t nvec, len;
    svd_geometry(m, n, geo_mode, cols, nvec, len);
    const int64_t ldx = len;
    const int64_t k = m < n ? m : n;
    if (nvec > (int64_t)1 << 20) return CT_ERR_UNSUPPORTED;
    double* X = ar.take<double>(nvec * ldx);
    double* Q = ar.take<double>(nvec * nvec);
    double* sig = ar.take<double>(nvec);
    int* perm = ar.take<int>(nvec);
    if (!X || !Q || !sig || !perm) return CT_ERR_OOM;
    const double tol = 2.2204460492503131e-16 * sqrt((double)(len > 1 ? len : 1)) * 4.0;
    // vectors after the Jacobi and the accumulated factor (row stride ldq)
    int64_t nv = nvec;
    const int64_t ldq = nvec;
    const double* Qf = Q;
    bool small_run = false;

    if (svd_uses_qr(nvec, len)) {
        double* Qn = nullptr;
        CT_TRY(svd_qr_jacobi(h, ar, M, m, n, cols, nvec, len, tol, X, Q, &Qn));
        nv = k;
        Qf = Qn;
    } else {
        const int64_t tot = nvec * (len > nvec ? len : nvec);
        int g = (int)ct_cdiv(tot, 256);
        if (g > h->num_sms * 16) g = h->num_sms * 16;
        if (g < 1) g = 1;
        svd_init_kernel<<<g, 256, 0, h->stream>>>(M, m, n, cols, X, ldx, Q, nvec); ct_note_launch();
        CT_LAUNCH_CHECK(h);
        const size_t small_bytes = (size_t)(nvec * len + nvec * nvec) * sizeof(double);
        if (nvec >= 2 && small_bytes <= 200 * 1024) {
            static bool attr = false;
            if (!attr) {
                CT_CUDA(h, cudaFuncSetAttribute(svd_small_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                200 * 1024));
                attr = true;
            }
            const int cap = (h->svd_max_sweeps > 0 && h->svd_max_sweeps < SVD_MAX_SWEEPS) ? h->svd_max_sweeps
                                                                                            : SVD_MAX_SWEEPS;
            svd_small_kernel<<<1, SVD_NT, small_bytes, h->stream>>>(X, len, ldx, Q, (int)nvec, tol, cap, h->d_status,
                                                                    h->d_flags + FL_SVD_SWEEPS); ct_note_launch();
            CT_LAUNCH_CHECK(h);
            small_run = true;
        } else if (nvec >= 2) {
            // beyond the QR's shared-memory limit: the Jacobi on the vectors themselves
            double* d_frob2 = h->d_scalars + SC_TMP0;
            CT_TRY(ct_reduce_nrm2sq(h, nvec * ldx, X, d_frob2, nullptr));
            CT_TRY(ct_jacobi::run<double>(h, X, len, Q, nvec, tol, SVD_EPS2, d_frob2, nullptr));
        }
    }
    svd_norms_kernel<<<(unsigned)ct_cdiv(nv * 32, 256), 256, 0, h->stream>>>(X, len, ldx, nv, sig); ct_note_launch();
    svd_rank_kernel<<<(unsigned)ct_cdiv(nv, 256), 256, 0, h->stream>>>(sig, nv, perm); ct_note_launch();
    svd_trunc_kernel<<<1, 32, 0, h->stream>>>(sig, perm, k, chi_max, eps_trunc, h->d_scalars, h->d_flags); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    int chi = 0;
    double sums[2];
    CT_CUDA(h, cudaMemcpyAsync(&chi, h->d_flags + FL_CHI, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CT_CUDA(h, cudaMemcpyAsync(sums, h->d_scalars + SC_TMP0, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CT_CUDA(h, cudaMemcpyAsync(min_kept, h->d_scalars + SC_SVD_MINKEPT, sizeof(double), cudaMemcpyDeviceToHost,
                               h->stream));
    int small_sweeps = 0;
    if (small_run)
        CT_CUDA(h, cudaMemcpyAsync(&small_sweeps, h->d_flags + FL_SVD_SWEEPS, sizeof(int), cudaMemcpyDeviceToHost,
                                   h->stream));
    CT_CUDA(h, cudaStreamSynchronize(h->stream));
    if (small_run) {
        h->last_svd_sweeps = small_sweeps;
        h->total_svd_sweeps += small_sweeps;
    }
    int st = 0;
    CT_CUDA(h, cudaMemcpy(&st, h->d_status, sizeof(int), cudaMemcpyDeviceToHost));
    if (st != 0) {
        CT_CUDA(h, cudaMemset(h->d_status, 0, sizeof(int)));
        ct_seterr(h, "device SVD reported status %d", st);
        return st;
    }
    out->chi = chi;
    out->sum_s2_all = sums[0];
    out->sum_s2_kept = sums[1];
    if (chi > 0) {
        const int64_t tot = (m > n ? m : n) * (int64_t)chi;
        int g = (int)ct_cdiv(tot, 256);
        if (g > h->num_sms * 16) g = h->num_sms * 16;
        if (g < 1) g = 1;
        svd_gather_kernel<<<g, 256, 0, h->stream>>>(X, ldx, Qf, ldq, sig, perm, h->d_flags, m, n, cols, mode, A, B,
                                                    S); ct_note_launch();
        CT_LAUNCH_CHECK(h);
    }
    return CT_OK;
}
