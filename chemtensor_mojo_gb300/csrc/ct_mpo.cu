// MPO legs of the contraction chains: small-K, memory-bound contractions.
//
// The reference contracts the MPO tensors with two GEMMs plus permutes per
// H_eff apply (dmrg.mojo:326-356) and one per environment update
// (environments.mojo:158-175, :374-396).  Here W_i and W_{i+1} are first fused
// into one (d^2 wR) x (wL d^2) matrix W12 (sum over the middle MPO bond, once
// per bond) and applied in a single pass over the intermediate: each thread
// owns one column i of in(o, :, i), streams its K inputs once per chunk of 8
// outputs and keeps the weights (or a chunk of their rows) in shared memory.
#include <algorithm>

#include "ct_common.cuh"

namespace {

constexpr int MPO_NT = 128;
constexpr int MPO_JC = 8;

// Block (x, o, z) handles columns i of slab o for output rows j in chunk z
// ([z * jch, z * jch + jch) of J); shared memory holds that chunk of Wt and
// its output offsets.
__global__ void __launch_bounds__(MPO_NT) mpo_apply_f64_kernel(MpoDesc m, int64_t jch) {
    if (ct_skip(m.skip)) return;
    extern __shared__ double wsm[];
    const int64_t jbeg = (int64_t)blockIdx.z * jch;
    const int64_t jn = (m.J - jbeg) < jch ? (m.J - jbeg) : jch;
    int64_t* joff = reinterpret_cast<int64_t*>(wsm + jch * m.K);
    for (int64_t t = threadIdx.x; t < jn * m.K; t += MPO_NT) wsm[t] = m.Wt[jbeg * m.K + t];
    for (int64_t j = threadIdx.x; j < jn; j += MPO_NT) {
        const int64_t jj = jbeg + j;
        joff[j] = (jj / m.J0) * m.sOj1 + (jj % m.J0) * m.sOj0;
    }
    __syncthreads();
    const int64_t o = blockIdx.y;
    const int64_t i = (int64_t)blockIdx.x * MPO_NT + threadIdx.x;
    if (i >= m.I) return;
    const double* in = m.in + o * m.sIo + i * m.sIi;
    double* out = m.out + o * m.sOo + i * m.sOi;
    for (int64_t j0 = 0; j0 < jn; j0 += MPO_JC) {
        double acc[MPO_JC];
#pragma unroll
        for (int jj = 0; jj < MPO_JC; ++jj) acc[jj] = 0.0;
        const int nj = (int)((jn - j0) < MPO_JC ? (jn - j0) : MPO_JC);
        for (int64_t k = 0; k < m.K; ++k) {
            const double x = in[k * m.sIk];
#pragma unroll
            for (int jj = 0; jj < MPO_JC; ++jj)
                if (jj < nj) acc[jj] = fma(wsm[(j0 + jj) * m.K + k], x, acc[jj]);
        }
#pragma unroll
        for (int jj = 0; jj < MPO_JC; ++jj) {
            if (jj >= nj) break;
            out[joff[j0 + jj]] = acc[jj];
        }
    }
}

// W12t[(t1 t2 wR), (wL s1 s2)] = sum_wM W1[wL,s1,t1,wM] W2[wM,s2,t2,wR]
__global__ void build_w12_kernel(const double* W1, const double* W2, double* W12t, int64_t wL,
                                 int64_t d, int64_t wM, int64_t wR) {
    const int64_t J = d * d * wR, K = wL * d * d;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= J * K) return;
    const int64_t j = t / K, k = t % K;
    const int64_t wr = j % wR, t2 = (j / wR) % d, t1 = j / (wR * d);
    const int64_t s2 = k % d, s1 = (k / d) % d, wl = k / (d * d);
    double acc = 0.0;
    for (int64_t wm = 0; wm < wM; ++wm) {
        const double a = W1[((wl * d + s1) * d + t1) * wM + wm];
        const double b = W2[((wm * d + s2) * d + t2) * wR + wr];
        acc = fma(a, b, acc);
    }
    W12t[t] = acc;
}

// Wt[(s' wR), (wL s)] = W[wL, s, s', wR]   (left environment)
__global__ void build_wt_left_kernel(const double* W, double* Wt, int64_t wL, int64_t d, int64_t wR) {
    const int64_t J = d * wR, K = wL * d;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= J * K) return;
    const int64_t j = t / K, k = t % K;
    const int64_t sp = j / wR, wr = j % wR, wl = k / d, s = k % d;
    Wt[t] = W[((wl * d + s) * d + sp) * wR + wr];
}

// Wt[(wL s'), (wR s)] = W[wL, s, s', wR]   (right environment)
__global__ void build_wt_right_kernel(const double* W, double* Wt, int64_t wL, int64_t d, int64_t wR) {
    const int64_t J = wL * d, K = wR * d;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= J * K) return;
    const int64_t j = t / K, k = t % K;
    const int64_t wl = j / d, sp = j % d, wr = k / d, s = k % d;
    Wt[t] = W[((wl * d + s) * d + sp) * wR + wr];
}

// W[(al, bl), i, o, (ar, br)] = sum_m Wa[al, i, m, ar] Wb[bl, m, o, br]   (MPO composition)
__global__ void mpo_compose_kernel(const double* Wa, const double* Wb, double* W, int64_t wLa, int64_t d_in,
                                   int64_t d_mid, int64_t wRa, int64_t wLb, int64_t d_out, int64_t wRb) {
    const int64_t n = wLa * wLb * d_in * d_out * wRa * wRb;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t q = t;
        const int64_t br = q % wRb; q /= wRb;
        const int64_t ar = q % wRa; q /= wRa;
        const int64_t o = q % d_out; q /= d_out;
        const int64_t i = q % d_in; q /= d_in;
        const int64_t bl = q % wLb; q /= wLb;
        const int64_t al = q;
        double acc = 0.0;
        for (int64_t m = 0; m < d_mid; ++m)
            acc = fma(Wa[((al * d_in + i) * d_mid + m) * wRa + ar], Wb[((bl * d_mid + m) * d_out + o) * wRb + br], acc);
        W[t] = acc;
    }
}

// out[(w, a), t, (v, b)] = sum_s A[a, s, b] W[w, s, t, v]   (MPO applied to an MPS site).
// One block row per (w, a, t, v): threads run along b, so the reads of A and the
// writes of out are contiguous; the d weights of the row are broadcast.
__global__ void __launch_bounds__(256) apply_mpo_kernel(const double* __restrict__ A, const double* __restrict__ W,
                                                        double* __restrict__ out, int64_t Dl, int64_t d, int64_t Dr,
                                                        int64_t wL, int64_t d_out, int64_t wR) {
    const int64_t rows = wL * Dl * d_out * wR;
    for (int64_t row = blockIdx.y; row < rows; row += gridDim.y) {
        int64_t q = row;
        const int64_t v = q % wR; q /= wR;
        const int64_t t = q % d_out; q /= d_out;
        const int64_t a = q % Dl;
        const int64_t w = q / Dl;
        double* o = out + row * Dr;
        const double* Ar = A + a * d * Dr;
        for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < Dr; b += (int64_t)gridDim.x * blockDim.x) {
            double acc = 0.0;
            for (int64_t s = 0; s < d; ++s) acc = fma(Ar[s * Dr + b], __ldg(&W[((w * d + s) * d_out + t) * wR + v]), acc);
            o[b] = acc;
        }
    }
}

}  // namespace

int ct_mpo_compose_launch(ct_handle* h, const double* Wa, const double* Wb, double* Wout, int64_t wLa,
                          int64_t d_in, int64_t d_mid, int64_t wRa, int64_t wLb, int64_t d_out, int64_t wRb) {
    const int64_t n = wLa * wLb * d_in * d_out * wRa * wRb;
    if (n <= 0) return CT_OK;
    const int64_t g = std::min<int64_t>(ct_cdiv(n, 256), (int64_t)h->num_sms * 8);
    mpo_compose_kernel<<<(unsigned)g, 256, 0, h->stream>>>(Wa, Wb, Wout, wLa, d_in, d_mid, wRa, wLb, d_out, wRb);
    ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

int ct_apply_mpo_launch(ct_handle* h, const double* A, const double* W, double* out, int64_t Dl, int64_t d,
                        int64_t Dr, int64_t wL, int64_t d_out, int64_t wR) {
    const int64_t rows = wL * Dl * d_out * wR;
    if (rows <= 0 || Dr <= 0) return CT_OK;
    dim3 grid((unsigned)std::min<int64_t>(ct_cdiv(Dr, 256), 64), (unsigned)std::min<int64_t>(rows, 65535));
    apply_mpo_kernel<<<grid, 256, 0, h->stream>>>(A, W, out, Dl, d, Dr, wL, d_out, wR);
    ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

int ct_mpo_apply_f64_launch(ct_handle* h, const MpoDesc& m) {
    if (m.O <= 0 || m.I <= 0 || m.J <= 0) return CT_OK;
    // the whole of Wt in shared memory when it fits in 96 KB, else chunks of rows
    constexpr size_t kBudget = 96 * 1024;
    const size_t per_row = (size_t)m.K * sizeof(double) + sizeof(int64_t);
    int64_t jch = m.J;
    if ((size_t)m.J * per_row > kBudget) {
        jch = (int64_t)(kBudget / per_row);
        if (jch >= MPO_JC) jch -= jch % MPO_JC;
        if (jch < 1) {
            ct_seterr(h, "MPO weight row too long (K = %lld)", (long long)m.K);
            return CT_ERR_UNSUPPORTED;
        }
    }
    const size_t smem = (size_t)jch * per_row;
    const int64_t nz = ct_cdiv(m.J, jch);
    if (m.O > 65535 || nz > 65535) return CT_ERR_UNSUPPORTED;
    static int attr_dev = -1;
    if (attr_dev != h->device) {
        CT_CUDA(h, cudaFuncSetAttribute(mpo_apply_f64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)kBudget));
        attr_dev = h->device;
    }
    dim3 grid((unsigned)ct_cdiv(m.I, MPO_NT), (unsigned)m.O, (unsigned)nz);
    mpo_apply_f64_kernel<<<grid, MPO_NT, smem, h->stream>>>(m, jch); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

int ct_build_w12(ct_handle* h, const double* W1, const double* W2, double* W12t, int64_t wL,
                 int64_t d, int64_t wM, int64_t wR) {
    const int64_t n = (d * d * wR) * (wL * d * d);
    build_w12_kernel<<<(unsigned)ct_cdiv(n, 256), 256, 0, h->stream>>>(W1, W2, W12t, wL, d, wM, wR); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

int ct_build_wt_left(ct_handle* h, const double* W, double* Wt, int64_t wL, int64_t d, int64_t wR) {
    const int64_t n = (d * wR) * (wL * d);
    build_wt_left_kernel<<<(unsigned)ct_cdiv(n, 256), 256, 0, h->stream>>>(W, Wt, wL, d, wR); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}

int ct_build_wt_right(ct_handle* h, const double* W, double* Wt, int64_t wL, int64_t d, int64_t wR) {
    const int64_t n = (wL * d) * (wR * d);
    build_wt_right_kernel<<<(unsigned)ct_cdiv(n, 256), 256, 0, h->stream>>>(W, Wt, wL, d, wR); ct_note_launch();
    CT_LAUNCH_CHECK(h);
    return CT_OK;
}
