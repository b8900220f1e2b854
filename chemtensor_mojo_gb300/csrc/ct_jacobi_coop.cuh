// Persistent one-sided Jacobi: all round-robin rounds of all sweeps in one
// cooperative launch.  Every CTA walks the pairs of a round (k = blockIdx.x,
// += gridDim.x), then waits at a grid barrier; after each sweep every CTA reads
// the sweep's rotation count and leaves together when it is zero.  The barrier
// spins at most 2 s (then sets the status word and aborts), and cooperative
// launch refuses grids that cannot be co-resident, so no wait is unbounded.
#pragma once
#include "ct_common.cuh"

namespace ct_jacobi {

constexpr int NT = 256;
constexpr int MAX_SWEEPS = 48;

__device__ __forceinline__ unsigned long long gtime() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

struct Sync {
    unsigned* count;
    unsigned* gen;
    int* abort_flag;
    int* rot;        // [MAX_SWEEPS] rotation counts, zeroed before launch
    int* sweeps;     // out: sweeps run
    int* status;
};

__device__ __forceinline__ bool grid_barrier(const Sync& s) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        volatile unsigned* vgen = s.gen;
        volatile int* vab = s.abort_flag;
        const unsigned g0 = *vgen;
        __threadfence();
        const unsigned arrived = atomicAdd(s.count, 1u) + 1u;
        if (arrived == gridDim.x) {
            atomicExch(s.count, 0u);
            __threadfence();
            atomicAdd(s.gen, 1u);
        } else {
            const unsigned long long t0 = gtime();
            while (*vgen == g0) {
                if (*vab) { ok = 0; break; }
                if (gtime() - t0 > 2000000000ull) {
                    ok = 0;
                    atomicExch(s.abort_flag, 1);
                    ct_set_status(s.status, CT_ERR_CUDA);
                    break;
                }
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

__device__ __forceinline__ void pair_index(int P, int r, int k, int& p, int& q) {
    if (k == 0) {
        p = P - 1;
        q = r;
    } else {
        p = (r + k) % (P - 1);
        q = (r - k + (P - 1)) % (P - 1);
    }
}

template <int N>
__device__ __forceinline__ double block_sum(double v, double* sm) {
    return ct_block_sum<N>(v, sm);
}

// T = float (mixed form: FP32 data, FP64 reductions) or double (plain form)
template <typename T>
__global__ void __launch_bounds__(NT) jacobi_coop_kernel(T* X, int64_t len, T* Q, int64_t nvec, double tol,
                                                        double floor_rel, const double* frob2, int max_sweeps,
                                                        Sync s) {
    __shared__ double sm[32];
    __shared__ double rot_cs, rot_sn;
    __shared__ int do_rot;
    const int P = (int)(nvec + (nvec & 1));
    const double floor = floor_rel * (*frob2);
    int sweep = 0;
    bool ok = true;
    for (; sweep < max_sweeps && ok; ++sweep) {
        for (int r = 0; r < P - 1 && ok; ++r) {
            for (int k = blockIdx.x; k < P / 2; k += gridDim.x) {
                int p, q;
                pair_index(P, r, k, p, q);
                if (p >= nvec || q >= nvec) continue;
                T* xp = X + (int64_t)p * len;
                T* xq = X + (int64_t)q * len;
                T fa = 0, fb = 0, fc = 0;
                for (int64_t i = threadIdx.x; i < len; i += NT) {
                    const T u = xp[i], v = xq[i];
                    fa += u * u;
                    fb += v * v;
                    fc += u * v;
                }
                const double a = block_sum<NT>((double)fa, sm);
                const double b = block_sum<NT>((double)fb, sm);
                const double c = block_sum<NT>((double)fc, sm);
                if (threadIdx.x == 0) {
                    int go = 0;
                    if (a > floor && b > floor && c != 0.0 && fabs(c) > tol * sqrt(a * b)) {
                        const double zeta = (b - a) / (2.0 * c);
                        const double t = (fabs(zeta) > 1e150)
                                             ? 0.5 / zeta
                                             : copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                        const double cs = 1.0 / sqrt(1.0 + t * t);
                        rot_cs = cs;
                        rot_sn = cs * t;
                        go = 1;
                        atomicAdd(&s.rot[sweep], 1);
                    }
                    do_rot = go;
                }
                __syncthreads();
                if (do_rot) {
                    const T cs = (T)rot_cs, sn = (T)rot_sn;
                    for (int64_t i = threadIdx.x; i < len; i += NT) {
                        const T u = xp[i], v = xq[i];
                        xp[i] = cs * u - sn * v;
                        xq[i] = sn * u + cs * v;
                    }
                    T* qp = Q + (int64_t)p * nvec;
                    T* qq = Q + (int64_t)q * nvec;
                    for (int64_t i = threadIdx.x; i < nvec; i += NT) {
                        const T u = qp[i], v = qq[i];
                        qp[i] = cs * u - sn * v;
                        qq[i] = sn * u + cs * v;
                    }
                }
                __syncthreads();
            }
            ok = grid_barrier(s);
        }
        if (!ok) break;
        const int rc = *(volatile int*)&s.rot[sweep];
        if (rc == 0) {
            ++sweep;
            break;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *s.sweeps = sweep;
        if (ok && sweep >= max_sweeps && *(volatile int*)&s.rot[max_sweeps - 1] != 0)
            ct_set_status(s.status, CT_ERR_NOCONV);
    }
}

// Launches the persistent Jacobi; sync scratch comes from h->d_flags.
template <typename T>
int run(ct_handle* h, T* X, int64_t len, T* Q, int64_t nvec, double tol, double floor_rel, const double* frob2,
        int* sweeps_host) {
    if (nvec < 2) {
        if (sweeps_host) *sweeps_host = 0;
        return CT_OK;
    }
    // scratch layout in d_flags: [16] count, [17] gen, [18] abort, [19] sweeps, [32..32+MAX_SWEEPS) rot
    int* base = h->d_flags;
    CT_CUDA(h, cudaMemsetAsync(base + 16, 0, (32 + MAX_SWEEPS - 16) * sizeof(int), h->stream));
    Sync s;
    s.count = (unsigned*)(base + 16);
    s.gen = (unsigned*)(base + 17);
    s.abort_flag = base + 18;
    s.sweeps = base + 19;
    s.rot = base + 32;
    s.status = h->d_status;
    static int occ_dev = -1, occ = 0;
    if (occ_dev != h->device) {
        CT_CUDA(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, jacobi_coop_kernel<T>, NT, 0));
        occ_dev = h->device;
    }
    const int64_t pairs = (nvec + (nvec & 1)) / 2;
    int64_t grid = (int64_t)occ * h->num_sms;
    if (grid > pairs) grid = pairs;
    if (grid < 1) grid = 1;
    // the handle's sweep cap (ct_set_svd_max_sweeps) never exceeds the kernel's own
    int max_sweeps = (h->svd_max_sweeps > 0 && h->svd_max_sweeps < MAX_SWEEPS) ? h->svd_max_sweeps : MAX_SWEEPS;
    void* args[] = {&X, &len, &Q, &nvec, &tol, &floor_rel, (void*)&frob2, &max_sweeps, &s};
    CT_CUDA(h, cudaLaunchCooperativeKernel((const void*)jacobi_coop_kernel<T>, dim3((unsigned)grid), dim3(NT), args,
                                           0, h->stream));
    ct_note_launch();
    int sw = 0;
    CT_CUDA(h, cudaMemcpyAsync(&sw, s.sweeps, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CT_CUDA(h, cudaStreamSynchronize(h->stream));
    h->last_svd_sweeps = sw;
    h->total_svd_sweeps += sw;
    if (sweeps_host) *sweeps_host = sw;
    return CT_OK;
}

}  // namespace ct_jacobi
