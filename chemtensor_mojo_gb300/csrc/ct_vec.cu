// FP64 vector algebra of the Lanczos solver and the dense-tensor reductions.
//
// The reference reduces with one thread per 256-block summing serially and a
// single thread summing the partials, then copies one scalar to the host and
// synchronises per call (dense_tensor.mojo:142-210); its DMRG Lanczos moves
// every Krylov vector to the host per step (dmrg.mojo:640-689).  Here every
// reduction is a grid of 256-thread blocks doing warp-shuffle tree sums over
// 16-byte loads, followed by a one-block finisher that sums the partials in a
// fixed order (bitwise reproducible) and runs the scalar epilogue on the
// device (alpha, beta, the breakdown test, 1/norm), so a whole Lanczos run is
// enqueued without a host round trip.
#include "ct_common.cuh"

namespace {

constexpr int RT = 256;

__host__ __device__ __forceinline__ bool aligned16(const void* p) { return ((uintptr_t)p & 15) == 0; }

// ---- phase 1: per-block partial sums --------------------------------------
// mode 0: sum x*y, mode 1: sum x*x
template <int MODE>
__global__ void __launch_bounds__(RT) partial_kernel(int64_t n, const double* __restrict__ x,
                                                     const double* __restrict__ y, double* partials,
                                                     const int* skip) {
    if (ct_skip(skip)) return;
    __shared__ double sm[32];
    double acc = 0.0;
    const int64_t stride = (int64_t)gridDim.x * RT;
    int64_t start = (int64_t)blockIdx.x * RT + threadIdx.x;
    const bool vec = aligned16(x) && (MODE == 1 || aligned16(y));
    if (vec) {
        const int64_t n2 = n / 2;
        const double2* x2 = reinterpret_cast<const double2*>(x);
        const double2* y2 = reinterpret_cast<const double2*>(y);
        for (int64_t i = start; i < n2; i += stride) {
            const double2 a = x2[i];
            if (MODE == 0) {
                const double2 b = y2[i];
                acc = fma(a.x, b.x, acc);
                acc = fma(a.y, b.y, acc);
            } else {
                acc = fma(a.x, a.x, acc);
                acc = fma(a.y, a.y, acc);
            }
        }
        if ((n & 1) && start == 0) {
            const double a = x[n - 1];
            acc = fma(a, MODE == 0 ? y[n - 1] : a, acc);
        }
    } else {
        for (int64_t i = start; i < n; i += stride) {
            const double a = x[i];
            acc = fma(a, MODE == 0 ? y[i] : a, acc);
        }
    }
    acc = ct_block_sum<RT>(acc, sm);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

__device__ double finish_sum(const double* partials, int np, double* sm) {
    double acc = 0.0;
    for (int i = threadIdx.x; i < np; i += RT) acc += partials[i];
    return ct_block_sum<RT>(acc, sm);
}

// ---- phase 2 finishers ------------------------------------------------------
__global__ void __launch_bounds__(RT) finish_store_kernel(const double* partials, int np, double* out,
                                                          const int* skip) {
    if (ct_skip(skip)) return;
    __shared__ double sm[32];
    const double s = finish_sum(partials, np, sm);
    if (threadIdx.x == 0) *out = s;
}

int grid_for(ct_handle* h, int64_t n) {
    int64_t g = ct_cdiv(n, (int64_t)RT * 8);
    const int64_t cap = (int64_t)h->num_sms * 8;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    if (g > CT_NPARTIALS) g = CT_NPARTIALS;
    return (int)g;
}

// ---- elementwise -------------------------------------------------------------
__global__ void axpy_kernel(int64_t n, double alpha, const double* x, double* y) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = fma(alpha, x[i], y[i]);
}
__global__ void scale_kernel(int64_t n, double alpha, double* x) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] *= alpha;
}
__global__ void fill_kernel(double* x, int64_t n, double v) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = v;
}
// One FP64 reciprocal per block, shared (once per kernel: the shared slot is not reused): an
// IEEE FP64 division or square root is tens of FP64 instructions, and on this part FP64 issues
// at ~1/64 of the FP32 rate, so one per thread of an elementwise grid (~600 k threads) cost
// more FP64 time than the kernel's memory traffic.
__device__ __forceinline__ double block_reciprocal(double x) {
    __shared__ double r;
    if (threadIdx.x == 0) r = 1.0 / x;
    __syncthreads();
    return r;
}

// y = x / sqrt(*nsq); status zero_code when sqrt(nsq) < 1e-14 (dmrg.mojo:605-611)
__global__ void scale_inv_sqrt_kernel(int64_t n, const double* x, double* y, const double* nsq,
                                      const int* skip, int* status, int zero_code) {
    if (ct_skip(skip)) return;
    __shared__ double nrm_s;
    if (threadIdx.x == 0) nrm_s = sqrt(*nsq);
    __syncthreads();
    const double nrm = nrm_s;
    const bool zero = !(nrm >= 1e-14);
    if (zero) {
        if (blockIdx.x == 0 && threadIdx.x == 0 && zero_code != 0) ct_set_status(status, zero_code);
    }
    const double r = block_reciprocal(zero ? 1.0 : nrm);
    const double inv = zero ? 0.0 : r;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = x[i] * inv;
}

__global__ void check_finite_kernel(const double* x, int* status, const int* skip) {
    if (ct_skip(skip)) return;
    if (!isfinite(*x)) ct_set_status(status, CT_ERR_NONFINITE);
}

__global__ void identity_env_kernel(double* E, int64_t w, int64_t D) {
    const int64_t n = w * D * D;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = (t / D) % D, c = t % D;
        E[t] = (r == c) ? 1.0 : 0.0;
    }
}

__global__ void identity_env_rect_kernel(double* E, int64_t w, int64_t Dk, int64_t Db) {
    const int64_t n = w * Dk * Db;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = (t / Db) % Dk, c = t % Db;
        E[t] = (r == c) ? 1.0 : 0.0;
    }
}

struct PermArgs {
    int rank;
    int64_t n;
    int64_t out_shape[6];
    int64_t in_stride_of_out_axis[6];
};
__global__ void permute_kernel(const double* in, double* out, PermArgs a) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < a.n; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t rem = t, src = 0;
        for (int ax = a.rank - 1; ax >= 0; --ax) {
            const int64_t idx = rem % a.out_shape[ax];
            rem /= a.out_shape[ax];
            src += idx * a.in_stride_of_out_axis[ax];
        }
        out[t] = in[src];
    }
}

// ---- Lanczos -------------------------------------------------------------------
// w -= alpha_j v_j + beta_{j-1} v_{j-1}; partial |w|^2 when NORM (the mixed form's
// reorthogonalisation measures the norm itself, and on this part FP64 issues at 1/64 of
// the FP32 rate: the unused norm was a third of the kernel's FP64 work)
template <bool NORM>
__global__ void __launch_bounds__(RT) lanczos_update_kernel(int64_t n, double* w, const double* vj,
                                                            const double* vjm1, const double* scalars,
                                                            int j, double* partials, const int* skip) {
    if (ct_skip(skip)) return;
    __shared__ double sm[32];
    const double a = scalars[SC_ALPHA + j];
    const double b = (j > 0) ? scalars[SC_BETA + j - 1] : 0.0;
    double acc = 0.0;
    const int64_t stride = (int64_t)gridDim.x * RT;
    if (aligned16(w) && aligned16(vj) && (!vjm1 || aligned16(vjm1))) {
        // 16-byte accesses; an odd last element by one thread
        const int64_t n2 = n / 2;
        double2* w2 = reinterpret_cast<double2*>(w);
        const double2* a2 = reinterpret_cast<const double2*>(vj);
        const double2* c2 = reinterpret_cast<const double2*>(vjm1);
        for (int64_t i = (int64_t)blockIdx.x * RT + threadIdx.x; i < n2; i += stride) {
            double2 x = w2[i];
            const double2 v = a2[i];
            x.x -= a * v.x;
            x.y -= a * v.y;
            if (vjm1) {
                const double2 u = c2[i];
                x.x -= b * u.x;
                x.y -= b * u.y;
            }
            w2[i] = x;
            if (NORM) acc = fma(x.x, x.x, fma(x.y, x.y, acc));
        }
        if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
            double x = w[n - 1] - a * vj[n - 1];
            if (vjm1) x -= b * vjm1[n - 1];
            w[n - 1] = x;
            if (NORM) acc = fma(x, x, acc);
        }
    } else {
        for (int64_t i = (int64_t)blockIdx.x * RT + threadIdx.x; i < n; i += stride) {
            double x = w[i] - a * vj[i];
            if (vjm1) x -= b * vjm1[i];
            w[i] = x;
            if (NORM) acc = fma(x, x, acc);
        }
    }
    if (NORM) {
        acc = ct_block_sum<RT>(acc, sm);
        if (threadIdx.x == 0) partials[blockIdx.x] = acc;
    }
}

// beta_j = sqrt(sum); breakdown test beta < 100 n eps (dmrg.mojo:630-673)
__global__ void __launch_bounds__(RT) lanczos_beta_finish(const double* partials, int np, double* scalars,
                                                          int* flags, int j, double thr, const int* skip) {
    if (ct_skip(skip)) return;
    __shared__ double sm[32];
    const double s = finish_sum(partials, np, sm);
    if (threadIdx.x == 0) {
        const double b = sqrt(s);
        if (b < thr) {
            flags[FL_NUMITER] = j + 1;
            flags[FL_STOP] = 1;
        } else {
            scalars[SC_BETA + j] = b;
        }
    }
}

__global__ void lanczos_next_kernel(int64_t n, const double* w, double* vnext, const double* scalars, int j,
                                    const int* skip) {
    if (ct_skip(skip)) return;
    const double inv = block_reciprocal(scalars[SC_BETA + j]);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        vnext[i] = w[i] * inv;
}

// ---- reorthogonalisation pass of the Lanczos step: fused Gram-Schmidt kernels ----
// After the reference recurrence w = H v_j - alpha_j v_j - beta_{j-1} v_{j-1}, w is
// orthogonalised once more against the whole Krylov basis V[0..j] in two passes:
//   A  c_k = <V_k, w> for k <= j                 (w read once per 16 basis vectors)
//   B  w <- w - sum_k c_k V_k with |w|^2, beta_j = |w| and the breakdown test
// and the next-vector kernel scales v_{j+1} = w / beta_j.  For v_j and v_{j-1}
// this is Gram-Schmidt twice (the recurrence is the first pass), for the older
// vectors, which carry only small components, once.  (Gram-Schmidt of H v_j
// alone, with alpha_j and beta_{j-1} as two of its coefficients, reads w less
// often but was measured to break the mixed form's sweeps -- energies below the
// ground state on the Heisenberg chain, L = 20, chi = 128 -- while the FP64 form
// and isolated solves were right; it is not used.)  Each reduction finishes in
// the block that arrives last (fixed-order sums over the block partials, so the
// result is reproducible) instead of a separate one-block launch.  Loads are 16
// bytes (double2) when n is even and every vector is 16-byte aligned, which holds
// for theta = Dl d^2 Dr with d even; otherwise the scalar path runs.
constexpr int CGS_VB = 16;

// true in every thread of the block that arrives last; partials written by the
// other blocks are then visible to it (threadfence-reduction pattern)
__device__ __forceinline__ bool last_block_arrived(unsigned* counter) {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
    __syncthreads();
    if (last) __threadfence();
    return last;
}

// acc[k] += <V[k], w> over this thread's elements, k < NV.  NV is a template
// parameter so exactly NV multiply-adds issue per element: FP64 issues at 1/64 of
// the FP32 rate on this part, and a predicated-off FMA of a runtime-bounded loop
// still occupies the FP64 pipe (measured: a 16-wide group did the same FP64 work
// for one live vector as for sixteen).
template <int NV>
__device__ __forceinline__ void cgs_dots_group(int64_t n, const double* __restrict__ w, const double* __restrict__ x,
                                               int64_t ldv, int vec2, double (&acc)[CGS_VB]) {
    const int64_t stride = (int64_t)gridDim.x * RT;
    if (vec2) {
        const int64_t n2 = n / 2;
        const double2* w2 = reinterpret_cast<const double2*>(w);
        for (int64_t i = (int64_t)blockIdx.x * RT + threadIdx.x; i < n2; i += stride) {
            const double2 wi = w2[i];
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                const double2 a = reinterpret_cast<const double2*>(x + (int64_t)k * ldv)[i];
                acc[k] = fma(a.x, wi.x, fma(a.y, wi.y, acc[k]));
            }
        }
    } else {
        for (int64_t i = (int64_t)blockIdx.x * RT + threadIdx.x; i < n; i += stride) {
            const double wi = w[i];
#pragma unroll
            for (int k = 0; k < NV; ++k) acc[k] = fma(x[(int64_t)k * ldv + i], wi, acc[k]);
        }
    }
}

// pass A: coeff[v] = <V[v], w> for v < nvec
__device__ __forceinline__ void cgs_dots_dev(int64_t n, const double* __restrict__ w, const double* __restrict__ V,
                                             int64_t ldv, int nvec, int vec2, double* partials, unsigned* counter,
                                             double* coeff) {
    __shared__ double sm[CGS_VB][RT / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int v0 = 0; v0 < nvec; v0 += CGS_VB) {
        const int nv = min(CGS_VB, nvec - v0);
        double acc[CGS_VB];
#pragma unroll
        for (int k = 0; k < CGS_VB; ++k) acc[k] = 0.0;
        const double* x = V + (int64_t)v0 * ldv;
        switch (nv) {
#define CT_CGS_CASE(K) \
    case K: cgs_dots_group<K>(n, w, x, ldv, vec2, acc); break;
            CT_CGS_CASE(1) CT_CGS_CASE(2) CT_CGS_CASE(3) CT_CGS_CASE(4) CT_CGS_CASE(5) CT_CGS_CASE(6)
            CT_CGS_CASE(7) CT_CGS_CASE(8) CT_CGS_CASE(9) CT_CGS_CASE(10) CT_CGS_CASE(11) CT_CGS_CASE(12)
            CT_CGS_CASE(13) CT_CGS_CASE(14) CT_CGS_CASE(15) CT_CGS_CASE(16)
#undef CT_CGS_CASE
            default: break;
        }
#pragma unroll
        for (int k = 0; k < CGS_VB; ++k)
            if (k < nv) acc[k] = ct_warp_sum(acc[k]);
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < CGS_VB; ++k)
                if (k < nv) sm[k][wid] = acc[k];
        }
        __syncthreads();
        if (threadIdx.x < nv) {
            double r = 0.0;
            for (int q = 0; q < RT / 32; ++q) r += sm[threadIdx.x][q];
            partials[(int64_t)blockIdx.x * nvec + v0 + threadIdx.x] = r;
        }
        __syncthreads();
    }
    if (!last_block_arrived(counter)) return;
    // last block: one warp per coefficient, lanes stride over the block partials
    for (int v = wid; v < nvec; v += RT / 32) {
        double r = 0.0;
        for (int b = lane; b < (int)gridDim.x; b += 32) r += __ldcg(partials + (int64_t)b * nvec + v);
        r = ct_warp_sum(r);
        if (lane == 0) coeff[v] = r;
    }
    if (threadIdx.x == 0) *counter = 0u;
}

// pass B: w -= sum_v coeff[v] V[v] with |w|^2; the last block forms beta_j = |w|
// and makes the breakdown test beta < thr (dmrg.mojo:630-673)
__device__ __forceinline__ void cgs_update_dev(int64_t n, double* __restrict__ w, const double* __restrict__ V,
                                               int64_t ldv, int nvec, int vec2, const double* coeff, double* partials,
                                               unsigned* counter, double* scalars, int* flags, int j, double thr) {
    __shared__ double sm[32];
    __shared__ double c[CT_MAX_KRYLOV];
    for (int v = threadIdx.x; v < nvec; v += RT) c[v] = coeff[v];
    __syncthreads();
    double nn = 0.0;
    const int64_t stride = (int64_t)gridDim.x * RT;
    if (vec2) {
        const int64_t n2 = n / 2;
        double2* w2 = reinterpret_cast<double2*>(w);
        for (int64_t i = (int64_t)blockIdx.x * RT + threadIdx.x; i < n2; i += stride) {
            double2 x = w2[i];
            int v = 0;
            for (; v + 4 <= nvec; v += 4) {
                const double2 a0 = reinterpret_cast<const double2*>(V + (int64_t)v * ldv)[i];
                const double2 a1 = reinterpret_cast<const double2*>(V + (int64_t)(v + 1) * ldv)[i];
                const double2 a2 = reinterpret_cast<const double2*>(V + (int64_t)(v + 2) * ldv)[i];
                const double2 a3 = reinterpret_cast<const double2*>(V + (int64_t)(v + 3) * ldv)[i];
                x.x -= c[v] * a0.x; x.y -= c[v] * a0.y;
                x.x -= c[v + 1] * a1.x; x.y -= c[v + 1] * a1.y;
                x.x -= c[v + 2] * a2.x; x.y -= c[v + 2] * a2.y;
                x.x -= c[v + 3] * a3.x; x.y -= c[v + 3] * a3.y;
            }
            for (; v < nvec; ++v) {
                const double2 a = reinterpret_cast<const double2*>(V + (int64_t)v * ldv)[i];
                x.x -= c[v] * a.x;
                x.y -= c[v] * a.y;
            }
            w2[i] = x;
            nn = fma(x.x, x.x, fma(x.y, x.y, nn));
        }
    } else {
        for (int64_t i = (int64_t)blockIdx.x * RT + threadIdx.x; i < n; i += stride) {
            double x = w[i];
            for (int v = 0; v < nvec; ++v) x -= c[v] * V[(int64_t)v * ldv + i];
            w[i] = x;
            nn = fma(x, x, nn);
        }
    }
    nn = ct_block_sum<RT>(nn, sm);
    if (threadIdx.x == 0) partials[blockIdx.x] = nn;
    if (!last_block_arrived(counter)) return;
    double s = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += RT) s += __ldcg(partials + b);
    s = ct_block_sum<RT>(s, sm);
    if (threadIdx.x == 0) {
        const double b = sqrt(s);
        if (b < thr) {
            flags[FL_NUMITER] = j + 1;
            flags[FL_STOP] = 1;
        } else {
            scalars[SC_BETA + j] = b;
        }
        *counter = 0u;
    }
}

// ---- the same pass against an FP32 copy of the basis (mixed form) --------------------
// After the FP64 recurrence the coefficients c_k = <V_k, w> are small (the components
// that the TF32-level H_eff and rounding leave along the older vectors), so the pass
// needs them only to a small relative accuracy: the dots run on FP32 copies of the
// basis and of w (FP32 products, per-thread FP32 sums of a few dozen terms, FP64
// across threads and blocks), and the update forms the correction sum_k c_k V32_k in
// FP32 and subtracts it from w in FP64.  Errors: ~1e-7 relative on c_k and on the
// correction, i.e. residual components ~1e-7 |c| along the basis, against the 1e-8
// that semi-orthogonality asks for.  The basis is read at 4 bytes per element instead
// of 8, with FP32 multiply-adds instead of FP64 ones (1/64 of the FP32 rate here).
template <int NV>
__device__ __forceinline__ void cgs32_dots_group(int64_t n, const double* __restrict__ w, const float* __restrict__ x,
                                                 int64_t ldv, int vec4, float (&acc)[CGS_VB]) {
    const int64_t stride = (int64_t)gridDim.x * RT;
    if (vec4) {
        const int64_t n4 = n / 4;
        const double2* w2 = reinterpret_cast<const double2*>(w);
        for (int64_t i = (int64_t)blockIdx.x * RT + threadIdx.x; i < n4; i += stride) {
            const double2 wa = w2[2 * i], wb = w2[2 * i + 1];
            const float w0 = (float)wa.x, w1 = (float)wa.y, w2f = (float)wb.x, w3 = (float)wb.y;
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                const float4 a = reinterpret_cast<const float4*>(x + (int64_t)k * ldv)[i];
                acc[k] = fmaf(a.x, w0, fmaf(a.y, w1, fmaf(a.z, w2f, fmaf(a.w, w3, acc[k]))));
            }
        }
    } else {
        for (int64_t i = (int64_t)blockIdx.x * RT + threadIdx.x; i < n; i += stride) {
            const float wi = (float)w[i];
#pragma unroll
            for (int k = 0; k < NV; ++k) acc[k] = fmaf(x[(int64_t)k * ldv + i], wi, acc[k]);
        }
    }
}

__device__ __forceinline__ void cgs32_dots_dev(int64_t n, const double* __restrict__ w, const float* __restrict__ V,
                                               int64_t ldv, int nvec, int vec4, double* partials, unsigned* counter,
                                               double* coeff) {
    static_assert(RT == 256 && CGS_VB == 16, "the block reduction maps 256 threads onto 16 x 16");
    __shared__ float red[CGS_VB][RT + 1];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int v0 = 0; v0 < nvec; v0 += CGS_VB) {
        const int nv = min(CGS_VB, nvec - v0);
        float acc[CGS_VB];
#pragma unroll
        for (int k = 0; k < CGS_VB; ++k) acc[k] = 0.0f;
        const float* x = V + (int64_t)v0 * ldv;
        switch (nv) {
#define CT_CGS_CASE(K) \
    case K: cgs32_dots_group<K>(n, w, x, ldv, vec4, acc); break;
            CT_CGS_CASE(1) CT_CGS_CASE(2) CT_CGS_CASE(3) CT_CGS_CASE(4) CT_CGS_CASE(5) CT_CGS_CASE(6)
            CT_CGS_CASE(7) CT_CGS_CASE(8) CT_CGS_CASE(9) CT_CGS_CASE(10) CT_CGS_CASE(11) CT_CGS_CASE(12)
            CT_CGS_CASE(13) CT_CGS_CASE(14) CT_CGS_CASE(15) CT_CGS_CASE(16)
#undef CT_CGS_CASE
            default: break;
        }
        // block sums of the nv per-thread FP32 sums, in FP64 from the first addition on:
        // through shared memory, thread t adds 16 of coefficient t / 16's entries, then
        // 16-lane shuffles (~36 FP64 instructions per warp instead of a 5-level shuffle
        // tree per coefficient, ~80; FP64 issues at 1/64 of the FP32 rate on this part)
#pragma unroll
        for (int k = 0; k < CGS_VB; ++k)
            if (k < nv) red[k][threadIdx.x] = acc[k];
        __syncthreads();
        {
            const int k = threadIdx.x >> 4, r0 = threadIdx.x & 15;
            double r = 0.0;
            if (k < nv) {
#pragma unroll
                for (int q = 0; q < RT / 16; ++q) r += (double)red[k][r0 + 16 * q];
            }
#pragma unroll
            for (int off = 8; off > 0; off >>= 1) r += __shfl_xor_sync(0xffffffffu, r, off, 16);
            if (k < nv && r0 == 0) partials[(int64_t)blockIdx.x * nvec + v0 + k] = r;
        }
        __syncthreads();
    }
    if (!last_block_arrived(counter)) return;
    for (int v = wid; v < nvec; v += RT / 32) {
        double r = 0.0;
        for (int b = lane; b < (int)gridDim.x; b += 32) r += __ldcg(partials + (int64_t)b * nvec + v);
        r = ct_warp_sum(r);
        if (lane == 0) coeff[v] = r;
    }
    if (threadIdx.x == 0) *counter = 0u;
}

__device__ __forceinline__ void cgs32_update_dev(int64_t n, double* __restrict__ w, const float* __restrict__ V,
                                                 int64_t ldv, int nvec, int vec4, const double* coeff,
                                                 double* partials, unsigned* counter, double* scalars, int* flags,
                                                 int j, double thr, int second, double ratio64) {
    __shared__ double sm[32];
    __shared__ float c[CT_MAX_KRYLOV];
    for (int v = threadIdx.x; v < nvec; v += RT) c[v] = (float)coeff[v];
    __syncthreads();
    double nn = 0.0;
    const int64_t stride = (int64_t)gridDim.x * RT;
    if (vec4) {
        const int64_t n4 = n / 4;
        double2* w2 = reinterpret_cast<double2*>(w);
        for (int64_t i = (int64_t)blockIdx.x * RT + threadIdx.x; i < n4; i += stride) {
            float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
            for (int v = 0; v < nvec; ++v) {
                const float4 a = reinterpret_cast<const float4*>(V + (int64_t)v * ldv)[i];
                const float cv = c[v];
                s.x = fmaf(cv, a.x, s.x);
                s.y = fmaf(cv, a.y, s.y);
                s.z = fmaf(cv, a.z, s.z);
                s.w = fmaf(cv, a.w, s.w);
            }
            double2 xa = w2[2 * i], xb = w2[2 * i + 1];
            xa.x -= (double)s.x;
            xa.y -= (double)s.y;
            xb.x -= (double)s.z;
            xb.y -= (double)s.w;
            w2[2 * i] = xa;
            w2[2 * i + 1] = xb;
            nn = fma(xa.x, xa.x, fma(xa.y, xa.y, fma(xb.x, xb.x, fma(xb.y, xb.y, nn))));
        }
    } else {
        for (int64_t i = (int64_t)blockIdx.x * RT + threadIdx.x; i < n; i += stride) {
            float s = 0.f;
            for (int v = 0; v < nvec; ++v) s = fmaf(c[v], V[(int64_t)v * ldv + i], s);
            const double x = w[i] - (double)s;
            w[i] = x;
            nn = fma(x, x, nn);
        }
    }
    nn = ct_block_sum<RT>(nn, sm);
    if (threadIdx.x == 0) partials[blockIdx.x] = nn;
    if (!last_block_arrived(counter)) return;
    double s = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += RT) s += __ldcg(partials + b);
    s = ct_block_sum<RT>(s, sm);
    double cc = 0.0;   // |sum_k c_k V_k|^2 = sum_k c_k^2 (orthonormal basis)
    for (int v = threadIdx.x; v < nvec; v += RT) cc += coeff[v] * coeff[v];
    cc = ct_block_sum<RT>(cc, sm);
    if (threadIdx.x == 0) {
        // The FP32 dots of w against a basis vector it is nearly parallel to err by
        // ~1e-7 of the coefficient (the terms share a sign), so the pass leaves ~1e-7 |c|
        // along the basis: ~1e-7 |c| / beta of orthogonality loss for v_{j+1}.  Up to
        // |c| = 0.1 beta that stays near 1e-8, about the semi-orthogonality Lanczos needs.
        // Beyond it a second FP32 pass (FL_REDO) runs on the now nearly orthogonal w,
        // whose dots err at random rather than coherently; it leaves ~1e-14 |c| / beta,
        // enough up to |c| / beta = ratio64 (1e4).  Above that (a Krylov space close to
        // exhausted, |c| / beta up to 1e5 and more) the second pass is the FP64 one
        // (FL_REDO64), on the FP64 basis.  Either decides beta and breakdown again.
        if (!second) {
            const bool big = cc > 1e-2 * s;
            const bool huge = cc > ratio64 * ratio64 * s;
            flags[FL_REDO] = (big && !huge) ? 1 : 0;
            flags[FL_REDO64] = huge ? 1 : 0;
        }
        const double b = sqrt(s);
        if (b < thr) {
            flags[FL_NUMITER] = j + 1;
            flags[FL_STOP] = 1;
        } else {
            scalars[SC_BETA + j] = b;
        }
        *counter = 0u;
    }
}

// alpha_j = <v_j, w> -> scalars[SC_ALPHA + j]: block partials over 16-byte loads, then
// the block that arrives last sums them in block order (the same fixed-order sum as a
// separate one-block finisher, without its launch)
__global__ void __launch_bounds__(RT) lanczos_alpha_kernel(int64_t n, const double* __restrict__ vj,
                                                           const double* __restrict__ w, double* partials,
                                                           unsigned* counter, double* scalars, int j,
                                                           const int* skip) {
    if (ct_skip(skip)) return;
    __shared__ double sm[32];
    double acc = 0.0;
    const int64_t stride = (int64_t)gridDim.x * RT;
    const int64_t start = (int64_t)blockIdx.x * RT + threadIdx.x;
    if (aligned16(vj) && aligned16(w)) {
        const int64_t n2 = n / 2;
        const double2* x2 = reinterpret_cast<const double2*>(vj);
        const double2* y2 = reinterpret_cast<const double2*>(w);
        for (int64_t i = start; i < n2; i += stride) {
            const double2 a = x2[i], b = y2[i];
            acc = fma(a.x, b.x, acc);
            acc = fma(a.y, b.y, acc);
        }
        if ((n & 1) && start == 0) acc = fma(vj[n - 1], w[n - 1], acc);
    } else {
        for (int64_t i = start; i < n; i += stride) acc = fma(vj[i], w[i], acc);
    }
    acc = ct_block_sum<RT>(acc, sm);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
    if (!last_block_arrived(counter)) return;
    double r = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += RT) r += __ldcg(partials + b);
    r = ct_block_sum<RT>(r, sm);
    if (threadIdx.x == 0) {
        scalars[SC_ALPHA + j] = r;
        *counter = 0u;
    }
}

// FP64 pass (FP64 form, and a gated second pass of the mixed form)
__global__ void __launch_bounds__(RT) cgs_dots_kernel(int64_t n, const double* __restrict__ w,
                                                      const double* __restrict__ V, int64_t ldv, int nvec, int vec2,
                                                      double* partials, unsigned* counter, double* coeff,
                                                      const int* skip) {
    if (ct_skip(skip)) return;
    cgs_dots_dev(n, w, V, ldv, nvec, vec2, partials, counter, coeff);
}
__global__ void __launch_bounds__(RT) cgs_update_kernel(int64_t n, double* __restrict__ w,
                                                        const double* __restrict__ V, int64_t ldv, int nvec, int vec2,
                                                        const double* coeff, double* partials, unsigned* counter,
                                                        double* scalars, int* flags, int j, double thr,
                                                        const int* skip) {
    if (ct_skip(skip)) return;
    cgs_update_dev(n, w, V, ldv, nvec, vec2, coeff, partials, counter, scalars, flags, j, thr);
}

// first pass of the mixed form, against the FP32 copy of the basis
__global__ void __launch_bounds__(RT) cgs32_dots_kernel(int64_t n, const double* __restrict__ w,
                                                        const float* __restrict__ V, int64_t ldv, int nvec, int vec4,
                                                        double* partials, unsigned* counter, double* coeff,
                                                        const int* skip) {
    if (ct_skip(skip)) return;
    cgs32_dots_dev(n, w, V, ldv, nvec, vec4, partials, counter, coeff);
}
__global__ void __launch_bounds__(RT) cgs32_update_kernel(int64_t n, double* __restrict__ w,
                                                          const float* __restrict__ V, int64_t ldv, int nvec, int vec4,
                                                          const double* coeff, double* partials, unsigned* counter,
                                                          double* scalars, int* flags, int j, double thr,
                                                          const int* skip, double ratio64) {
    if (ct_skip(skip)) return;
    cgs32_update_dev(n, w, V, ldv, nvec, vec4, coeff, partials, counter, scalars, flags, j, thr, 0, ratio64);
}

// second pass of the mixed form, gated on the device by the first: against the FP64
// basis when FL_REDO64 is set, else against the FP32 copy when FL_REDO is set, else
// nothing (one launch pair either way; the gates do not change between the two)
__global__ void __launch_bounds__(RT) cgs_redo_dots_kernel(int64_t n, const double* __restrict__ w,
                                                           const double* __restrict__ V, const float* __restrict__ V32,
                                                           int64_t ldv, int nvec, int vec2, int vec4,
                                                           double* partials, unsigned* counter, double* coeff,
                                                           const int* skip, const int* flags) {
    if (ct_skip(skip)) return;
    if (*(volatile const int*)(flags + FL_REDO64))
        cgs_dots_dev(n, w, V, ldv, nvec, vec2, partials, counter, coeff);
    else if (*(volatile const int*)(flags + FL_REDO))
        cgs32_dots_dev(n, w, V32, ldv, nvec, vec4, partials, counter, coeff);
}
__global__ void __launch_bounds__(RT) cgs_redo_update_kernel(int64_t n, double* __restrict__ w,
                                                             const double* __restrict__ V,
                                                             const float* __restrict__ V32, int64_t ldv, int nvec,
                                                             int vec2, int vec4, const double* coeff,
                                                             double* partials, unsigned* counter, double* scalars,
                                                             int* flags, int j, double thr, const int* skip) {
    if (ct_skip(skip)) return;
    if (*(volatile const int*)(flags + FL_REDO64))
        cgs_update_dev(n, w, V, ldv, nvec, vec2, coeff, partials, counter, scalars, flags, j, thr);
    else if (*(volatile const int*)(flags + FL_REDO))
        cgs32_update_dev(n, w, V32, ldv, nvec, vec4, coeff, partials, counter, scalars, flags, j, thr, 1, 0.0);
}

// v_{j+1} = w / beta_j in FP64 and its FP32 copy
__global__ void lanczos_next32_kernel(int64_t n, const double* w, double* vnext, float* vnext32,
                                      const double* scalars, int j, const int* skip) {
    if (ct_skip(skip)) return;
    const double inv = block_reciprocal(scalars[SC_BETA + j]);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    if (aligned16(w) && aligned16(vnext) && ((uintptr_t)vnext32 & 7) == 0) {
        // 16-byte FP64 and 8-byte FP32 accesses; an odd last element by one thread
        const int64_t n2 = n / 2;
        const double2* w2 = reinterpret_cast<const double2*>(w);
        double2* v2 = reinterpret_cast<double2*>(vnext);
        float2* f2 = reinterpret_cast<float2*>(vnext32);
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += stride) {
            const double2 x = w2[i];
            const double2 v = make_double2(x.x * inv, x.y * inv);
            v2[i] = v;
            f2[i] = make_float2((float)v.x, (float)v.y);
        }
        if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
            const double v = w[n - 1] * inv;
            vnext[n - 1] = v;
            vnext32[n - 1] = (float)v;
        }
    } else {
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
            const double v = w[i] * inv;
            vnext[i] = v;
            vnext32[i] = (float)v;
        }
    }
}

__global__ void f64_to_f32_copy_kernel(int64_t n, const double* x, float* y, const int* skip) {
    if (ct_skip(skip)) return;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = (float)x[i];
}

// Ritz vector: out = sum_{i < numiter} c_i V[i]
__global__ void ritz_kernel(int64_t n, const double* V, int64_t ldv, const double* scalars, const int* flags,
                            double* out) {
    const int nk = flags[FL_NUMITER];
    for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int i = 0; i < nk; ++i) acc = fma(scalars[SC_RITZ + i], V[(int64_t)i * ldv + x], acc);
        out[x] = acc;
    }
}

// Classical Jacobi on the nK x nK tridiagonal matrix (dmrg.mojo:507-598),
// one warp, T and V in shared memory.  Pivot: largest |T[i][j]| (i<j) with
// the first occurrence in row-major order winning ties, like the reference's
// strict '>' scan from (0,1).
__global__ void tridiag_jacobi_kernel(double* scalars, int* flags, int* status, double tol, int max_rot,
                                      int converged_mode) {
    extern __shared__ double tsm[];
    const int n = flags[FL_NUMITER];
    const int lane = threadIdx.x;
    if (n <= 0) {
        if (lane == 0) ct_set_status(status, CT_ERR_INVALID);
        return;
    }
    // a NaN or infinite alpha / beta (non-finite environments or MPO tensors) is an
    // error, not an eigenvalue: the rotations would compare NaN with every pivot
    bool bad = false;
    for (int i = lane; i < n; i += 32)
        bad |= !isfinite(scalars[SC_ALPHA + i]) || (i + 1 < n && !isfinite(scalars[SC_BETA + i]));
    if (__any_sync(0xffffffffu, bad)) {
        if (lane == 0) {
            ct_set_status(status, CT_ERR_NONFINITE);
            scalars[SC_ENERGY] = NAN;
        }
        return;
    }
    double* A = tsm;           // n x n
    double* V = tsm + n * n;   // n x n
    for (int t = lane; t < n * n; t += 32) {
        const int i = t / n, j = t % n;
        double a = 0.0;
        if (i == j) a = scalars[SC_ALPHA + i];
        else if (j == i + 1) a = scalars[SC_BETA + i];
        else if (i == j + 1) a = scalars[SC_BETA + j];
        A[t] = a;
        V[t] = (i == j) ? 1.0 : 0.0;
    }
    __syncwarp();
    if (n == 1) {
        if (lane == 0) {
            scalars[SC_ENERGY] = A[0];
            scalars[SC_RITZ] = 1.0;
        }
        return;
    }
    bool done = false;
    for (int rot = 0; rot < max_rot; ++rot) {
        // pivot search
        double best = -1.0;
        int bidx = 0x7fffffff;
        for (int i = lane; i < n; i += 32) {
            for (int j = i + 1; j < n; ++j) {
                const double v = fabs(A[i * n + j]);
                if (v > best) { best = v; bidx = i * n + j; }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bidx, o);
            if (ob > best || (ob == best && oi < bidx)) { best = ob; bidx = oi; }
        }
        if (best < tol) { done = true; break; }
        const int p = bidx / n, q = bidx % n;
        const double app = A[p * n + p], aqq = A[q * n + q], apq = A[p * n + q];
        const double phi = 0.5 * atan2(2.0 * apq, aqq - app);
        const double c = cos(phi), s = sin(phi);
        __syncwarp();
        for (int k = lane; k < n; k += 32) {
            if (k != p && k != q) {
                const double aik = A[k * n + p], akq = A[k * n + q];
                const double nkp = c * aik - s * akq;
                const double nkq = s * aik + c * akq;
                A[k * n + p] = nkp; A[p * n + k] = nkp;
                A[k * n + q] = nkq; A[q * n + k] = nkq;
            }
            const double vip = V[k * n + p], viq = V[k * n + q];
            V[k * n + p] = c * vip - s * viq;
            V[k * n + q] = s * vip + c * viq;
        }
        __syncwarp();
        if (lane == 0) {
            A[p * n + p] = c * c * app - 2.0 * s * c * apq + s * s * aqq;
            A[q * n + q] = s * s * app + 2.0 * s * c * apq + c * c * aqq;
            A[p * n + q] = 0.0;
            A[q * n + p] = 0.0;
        }
        __syncwarp();
    }
    if (converged_mode && !done && lane == 0) ct_set_status(status, CT_ERR_NOCONV);
    if (lane == 0) {
        int mi = 0;
        double mv = A[0];
        for (int i = 1; i < n; ++i)
            if (A[i * n + i] < mv) { mv = A[i * n + i]; mi = i; }
        double nrm = 0.0;
        for (int i = 0; i < n; ++i) nrm += V[i * n + mi] * V[i * n + mi];
        nrm = sqrt(nrm);
        for (int i = 0; i < n; ++i) scalars[SC_RITZ + i] = (nrm > 0.0) ? V[i * n + mi] / nrm : V[i * n + mi];
        scalars[SC_ENERGY] = mv;
    }
}

// Converged eigensolve of the Lanczos matrix: lowest eigenvalue by Sturm-count
// multisection (32 lanes probe 32 points per step), eigenvector by two steps of
// inverse iteration on the shifted, positive definite T - (lambda - delta) I
// (Thomas algorithm, no pivoting needed).  Same result as LAPACK dstev to
// rounding; O(n) per probe instead of the O(n^2)-per-rotation Jacobi.
__device__ int sturm_below(const double* a, const double* b, int n, double x) {
    int cnt = 0;
    double q = a[0] - x;
    if (q < 0.0) ++cnt;
    for (int i = 1; i < n; ++i) {
        if (q == 0.0) q = 1e-300;
        q = (a[i] - x) - b[i - 1] * b[i - 1] / q;
        if (q < 0.0) ++cnt;
    }
    return cnt;
}

__global__ void tridiag_bisect_kernel(double* scalars, const int* flags, int* status) {
    __shared__ double a[CT_MAX_KRYLOV], b[CT_MAX_KRYLOV], x[CT_MAX_KRYLOV];
    __shared__ double lo_s, hi_s;
    const int n = flags[FL_NUMITER];
    const int lane = threadIdx.x;
    if (n <= 0 || n > CT_MAX_KRYLOV) {
        if (lane == 0) ct_set_status(status, CT_ERR_INVALID);
        return;
    }
    bool bad = false;
    for (int i = lane; i < n; i += 32) {
        a[i] = scalars[SC_ALPHA + i];
        b[i] = (i + 1 < n) ? scalars[SC_BETA + i] : 0.0;
        bad |= !isfinite(a[i]) || !isfinite(b[i]);
    }
    // non-finite alpha / beta: fmin / fmax of the Gershgorin bounds would skip the
    // NaN and the multisection would return a finite, meaningless eigenvalue
    if (__any_sync(0xffffffffu, bad)) {
        if (lane == 0) {
            ct_set_status(status, CT_ERR_NONFINITE);
            scalars[SC_ENERGY] = NAN;
        }
        return;
    }
    __syncwarp();
    if (lane == 0) {
        double lo = 1e300, hi = -1e300;
        for (int i = 0; i < n; ++i) {
            const double r = (i > 0 ? fabs(b[i - 1]) : 0.0) + (i + 1 < n ? fabs(b[i]) : 0.0);
            lo = fmin(lo, a[i] - r);
            hi = fmax(hi, a[i] + r);
        }
        const double pad = 1e-12 * fmax(1.0, fmax(fabs(lo), fabs(hi)));
        lo_s = lo - pad;
        hi_s = hi + pad;
    }
    __syncwarp();
    double lo = lo_s, hi = hi_s;
    for (int it = 0; it < 64; ++it) {
        if (hi - lo <= 4.0 * 2.2204460492503131e-16 * fmax(fabs(lo), fabs(hi)) + 1e-300) break;
        const double p = lo + (hi - lo) * (double)(lane + 1) / 33.0;
        const int below = sturm_below(a, b, n, p) >= 1 ? 1 : 0;
        const unsigned mask = __ballot_sync(0xffffffffu, below);
        // first probe with an eigenvalue below it bounds the lowest eigenvalue
        const int first = mask ? (__ffs(mask) - 1) : 32;
        const double nlo = (first == 0) ? lo : lo + (hi - lo) * (double)first / 33.0;
        const double nhi = (first == 32) ? hi : lo + (hi - lo) * (double)(first + 1) / 33.0;
        lo = nlo;
        hi = nhi;
    }
    if (lane != 0) return;
    const double lam = 0.5 * (lo + hi);
    const double sigma = lam - 1e-12 * fmax(1.0, fabs(lam));
    double* c = scalars + SC_MISC;          // scratch: Thomas coefficients
    for (int i = 0; i < n; ++i) x[i] = 1.0;
    for (int rep = 0; rep < 3; ++rep) {
        // (T - sigma I) y = x : forward elimination
        double d = a[0] - sigma;
        c[0] = d;
        for (int i = 1; i < n; ++i) {
            const double l = b[i - 1] / c[i - 1];
            c[i] = (a[i] - sigma) - l * b[i - 1];
            x[i] -= l * x[i - 1];
        }
        x[n - 1] /= c[n - 1];
        for (int i = n - 2; i >= 0; --i) x[i] = (x[i] - b[i] * x[i + 1]) / c[i];
        double nrm = 0.0;
        for (int i = 0; i < n; ++i) nrm += x[i] * x[i];
        nrm = sqrt(nrm);
        for (int i = 0; i < n; ++i) x[i] /= nrm;
    }
    for (int i = 0; i < n; ++i) scalars[SC_RITZ + i] = x[i];
    scalars[SC_ENERGY] = lam;
}

__global__ void init_lanczos_flags(int* flags, int max_iter) {
    flags[FL_STOP] = 0;
    flags[FL_NUMITER] = max_iter;
}

int elem_grid(ct_handle* h, int64_t n) {
    int64_t g = ct_cdiv(n, 256);
    const int64_t cap = (int64_t)h->num_sms * 16;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

}  // namespace

int ct_reduce_dot(ct_handle* h, int64_t n, const double* x, const double* y, double* d_out, const int* skip) {
    const int g = grid_for(h, n);
    partial_kernel<0><<<g, RT, 0, h->stream>>>(n, x, y, h->d_partials, skip); ct_note_launch();
    finish_store_kernel<<<1, RT, 0, h->stream>>>(h->d_partials, g, d_out, skip); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

int ct_reduce_nrm2sq(ct_handle* h, int64_t n, const double* x, double* d_out, const int* skip) {
    const int g = grid_for(h, n);
    partial_kernel<1><<<g, RT, 0, h->stream>>>(n, x, nullptr, h->d_partials, skip); ct_note_launch();
    finish_store_kernel<<<1, RT, 0, h->stream>>>(h->d_partials, g, d_out, skip); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

int ct_scale_by_inv_sqrt(ct_handle* h, int64_t n, const double* x, double* y, const double* d_nsq,
                         const int* skip, int zero_code) {
    scale_inv_sqrt_kernel<<<elem_grid(h, n), 256, 0, h->stream>>>(n, x, y, d_nsq, skip, h->d_status, zero_code); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

int ct_fill(ct_handle* h, double* x, int64_t n, double v) {
    if (n <= 0) return CT_OK;
    fill_kernel<<<elem_grid(h, n), 256, 0, h->stream>>>(x, n, v); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

int ct_check_finite(ct_handle* h, const double* d_x, const int* skip) {
    check_finite_kernel<<<1, 1, 0, h->stream>>>(d_x, h->d_status, skip); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

int ct_copy(ct_handle* h, double* dst, const double* src, int64_t n) {
    if (n <= 0) return CT_OK;
    CT_CUDA(h, cudaMemcpyAsync(dst, src, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    return CT_OK;
}

int ct_identity_env(ct_handle* h, double* E, int64_t w, int64_t D) {
    const int64_t n = w * D * D;
    if (n <= 0) return CT_OK;
    identity_env_kernel<<<elem_grid(h, n), 256, 0, h->stream>>>(E, w, D); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

int ct_identity_env_rect(ct_handle* h, double* E, int64_t w, int64_t Dk, int64_t Db) {
    const int64_t n = w * Dk * Db;
    if (n <= 0) return CT_OK;
    identity_env_rect_kernel<<<elem_grid(h, n), 256, 0, h->stream>>>(E, w, Dk, Db); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

int ct_permute_launch(ct_handle* h, const double* in, double* out, int rank, const int64_t* shape,
                      const int32_t* perm) {
    if (rank < 1 || rank > 6) return CT_ERR_INVALID;
    PermArgs a;
    a.rank = rank;
    int64_t in_stride[6];
    int64_t s = 1;
    for (int ax = rank - 1; ax >= 0; --ax) {
        in_stride[ax] = s;
        s *= shape[ax];
    }
    a.n = s;
    bool seen[6] = {false, false, false, false, false, false};
    for (int ax = 0; ax < rank; ++ax) {
        const int p = perm[ax];
        if (p < 0 || p >= rank || seen[p]) return CT_ERR_INVALID;
        seen[p] = true;
        a.out_shape[ax] = shape[p];
        a.in_stride_of_out_axis[ax] = in_stride[p];
    }
    if (a.n == 0) return CT_OK;
    permute_kernel<<<elem_grid(h, a.n), 256, 0, h->stream>>>(in, out, a); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

int ct_vec_axpy_launch(ct_handle* h, int64_t n, double alpha, const double* x, double* y) {
    axpy_kernel<<<elem_grid(h, n), 256, 0, h->stream>>>(n, alpha, x, y); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}
int ct_vec_scale_launch(ct_handle* h, int64_t n, double alpha, double* x) {
    scale_kernel<<<elem_grid(h, n), 256, 0, h->stream>>>(n, alpha, x); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

int ct_lanczos_init(ct_handle* h, int max_iter) {
    init_lanczos_flags<<<1, 1, 0, h->stream>>>(h->d_flags, max_iter); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

int ct_lanczos_alpha(ct_handle* h, int64_t n, const double* vj, const double* w, int j, const int* skip) {
    const int g = grid_for(h, n);
    unsigned* counter = reinterpret_cast<unsigned*>(h->d_flags + FL_CNT);
    lanczos_alpha_kernel<<<g, RT, 0, h->stream>>>(n, vj, w, h->d_partials, counter, h->d_scalars, j, skip);
    ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

int ct_lanczos_update(ct_handle* h, int64_t n, double* w, const double* vj, const double* vjm1, int j,
                      double beta_threshold, const int* skip) {
    const int g = grid_for(h, n);
    lanczos_update_kernel<true><<<g, RT, 0, h->stream>>>(n, w, vj, vjm1, h->d_scalars, j, h->d_partials, skip); ct_note_launch();
    lanczos_beta_finish<<<1, RT, 0, h->stream>>>(h->d_partials, g, h->d_scalars, h->d_flags, j,
                                                 beta_threshold, skip); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

// Reorthogonalisation pass of Lanczos step j (passes A and B above), after the
// reference recurrence has updated w; beta_j (or the breakdown stop) goes to the
// scalar slots.  The caller then forms v_{j+1} = w / beta_j.
int ct_lanczos_reorth_pass(ct_handle* h, int64_t n, double* w, const double* V, int64_t ldv, int j,
                           double beta_threshold, const int* skip) {
    const int nvec = j + 1;
    if (nvec > 64) return CT_ERR_UNSUPPORTED;
    int g = grid_for(h, n);
    if ((int64_t)g * nvec > CT_NPARTIALS) g = CT_NPARTIALS / nvec;
    const int vec2 = ((n & 1) == 0 && (ldv & 1) == 0 && aligned16(w) && aligned16(V)) ? 1 : 0;
    unsigned* counter = reinterpret_cast<unsigned*>(h->d_flags + FL_CNT);
    double* coeff = h->d_scalars + SC_MISC;
    cgs_dots_kernel<<<g, RT, 0, h->stream>>>(n, w, V, ldv, nvec, vec2, h->d_partials, counter, coeff, skip);
    ct_note_launch();
    cgs_update_kernel<<<g, RT, 0, h->stream>>>(n, w, V, ldv, nvec, vec2, coeff, h->d_partials, counter,
                                               h->d_scalars, h->d_flags, j, beta_threshold, skip);
    ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

// Reorthogonalisation pass against the FP32 copy V32 of the basis (mixed form).  It sets
// the gates of the second pass: FL_REDO (against V32) when it removed more than 0.1 beta,
// FL_REDO64 (against the FP64 basis) above ratio64 beta.
int ct_lanczos_reorth_pass32(ct_handle* h, int64_t n, double* w, const float* V32, int64_t ldv, int j,
                             double beta_threshold, const int* skip, double ratio64) {
    const int nvec = j + 1;
    if (nvec > 64) return CT_ERR_UNSUPPORTED;
    int g = grid_for(h, n);
    if ((int64_t)g * nvec > CT_NPARTIALS) g = CT_NPARTIALS / nvec;
    const int vec4 = ((n & 3) == 0 && (ldv & 3) == 0 && aligned16(w) && aligned16(V32)) ? 1 : 0;
    unsigned* counter = reinterpret_cast<unsigned*>(h->d_flags + FL_CNT);
    double* coeff = h->d_scalars + SC_MISC;
    // the dots: two blocks per SM keep ~150 KB of loads in flight per SM, and fewer blocks
    // mean fewer block reductions (FP64)
    const int gd = g < 2 * h->num_sms ? g : 2 * h->num_sms;
    cgs32_dots_kernel<<<gd, RT, 0, h->stream>>>(n, w, V32, ldv, nvec, vec4, h->d_partials, counter, coeff, skip);
    ct_note_launch();
    cgs32_update_kernel<<<g, RT, 0, h->stream>>>(n, w, V32, ldv, nvec, vec4, coeff, h->d_partials, counter,
                                                 h->d_scalars, h->d_flags, j, beta_threshold, skip, ratio64);
    ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

// The gated second pass after ct_lanczos_reorth_pass32 (V: the FP64 basis, V32 its copy,
// both with leading dimension ldv).
int ct_lanczos_reorth_redo(ct_handle* h, int64_t n, double* w, const double* V, const float* V32, int64_t ldv, int j,
                           double beta_threshold, const int* skip) {
    const int nvec = j + 1;
    if (nvec > 64) return CT_ERR_UNSUPPORTED;
    int g = grid_for(h, n);
    if ((int64_t)g * nvec > CT_NPARTIALS) g = CT_NPARTIALS / nvec;
    const int vec2 = ((n & 1) == 0 && (ldv & 1) == 0 && aligned16(w) && aligned16(V)) ? 1 : 0;
    const int vec4 = ((n & 3) == 0 && (ldv & 3) == 0 && aligned16(w) && aligned16(V32)) ? 1 : 0;
    unsigned* counter = reinterpret_cast<unsigned*>(h->d_flags + FL_CNT);
    double* coeff = h->d_scalars + SC_MISC;
    cgs_redo_dots_kernel<<<g, RT, 0, h->stream>>>(n, w, V, V32, ldv, nvec, vec2, vec4, h->d_partials, counter, coeff,
                                                  skip, h->d_flags);
    ct_note_launch();
    cgs_redo_update_kernel<<<g, RT, 0, h->stream>>>(n, w, V, V32, ldv, nvec, vec2, vec4, coeff, h->d_partials,
                                                    counter, h->d_scalars, h->d_flags, j, beta_threshold, skip);
    ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

int ct_lanczos_next32(ct_handle* h, int64_t n, const double* w, double* vnext, float* vnext32, int j,
                      const int* skip) {
    lanczos_next32_kernel<<<elem_grid(h, n), 256, 0, h->stream>>>(n, w, vnext, vnext32, h->d_scalars, j, skip);
    ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

int ct_f64_to_f32(ct_handle* h, int64_t n, const double* x, float* y, const int* skip) {
    f64_to_f32_copy_kernel<<<elem_grid(h, n), 256, 0, h->stream>>>(n, x, y, skip); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

// w -= alpha_j v_j + beta_{j-1} v_{j-1} without the norm (the reorthogonalisation
// pass measures it afterwards)
int ct_lanczos_update_nonorm(ct_handle* h, int64_t n, double* w, const double* vj, const double* vjm1, int j,
                             const int* skip) {
    const int g = grid_for(h, n);
    lanczos_update_kernel<false><<<g, RT, 0, h->stream>>>(n, w, vj, vjm1, h->d_scalars, j, h->d_partials, skip);
    ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

int ct_lanczos_next(ct_handle* h, int64_t n, const double* w, double* vnext, int j, const int* skip) {
    lanczos_next_kernel<<<elem_grid(h, n), 256, 0, h->stream>>>(n, w, vnext, h->d_scalars, j, skip); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

int ct_tridiag_eig(ct_handle* h, int max_iter, double tol, int max_rotations) {
    if (max_iter > 64) return CT_ERR_UNSUPPORTED;
    const size_t smem = 2 * (size_t)max_iter * max_iter * sizeof(double);
    static bool attr = false;
    if (!attr) {
        CT_CUDA(h, cudaFuncSetAttribute(tridiag_jacobi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        2 * 64 * 64 * 8));
        attr = true;
    }
    if (max_rotations <= 0) {
        tridiag_bisect_kernel<<<1, 32, 0, h->stream>>>(h->d_scalars, h->d_flags, h->d_status); ct_note_launch();
        CT_LAUNCH_CHECK(h);
        return CT_OK;
    }
    tridiag_jacobi_kernel<<<1, 32, smem, h->stream>>>(h->d_scalars, h->d_flags, h->d_status, tol, max_rotations, 0); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

int ct_ritz(ct_handle* h, int64_t n, const double* V, int64_t ldv, double* out) {
    ritz_kernel<<<elem_grid(h, n), 256, 0, h->stream>>>(n, V, ldv, h->d_scalars, h->d_flags, out); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}
