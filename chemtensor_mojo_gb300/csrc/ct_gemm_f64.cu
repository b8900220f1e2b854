// Plain-form FP64 contraction kernel: a strided, batched SIMT GEMM.
//
// C(m,n) = alpha * sum_k A(m,k) B(k,n) + beta * C(m,n) with arbitrary element
// strides for every index and a two-level batch index, so every contraction of
// the path (dense_tensor_dot, dense_tensor.mojo:963-1328, and the permute +
// GEMM chains of dmrg.mojo:254-374 / environments.mojo:99-417) is one launch
// with the permutes folded into the operand addressing -- no physical
// transposes.  FP64 on GB300 issues at a small fraction of the FP32 rate, so
// a 64x64x16 smem tile with a 4x4 register block already saturates the FP64
// pipe; the tensor-core path lives in ct_tc.cu.
#include <algorithm>

#include "ct_common.cuh"

namespace {

constexpr int BK = 16;

// One CTA computes a TBM x TBN tile of C with (TBM/4) x (TBN/4) threads, each
// holding a 4 x 4 register block.  The 64 x 64 tile is the default; the
// 32 x 32 tile gives small problems (the factorisation's panels) enough CTAs
// to occupy every SM's FP64 pipe.
template <int TBM, int TBN, bool A_K_CONTIG, bool B_N_CONTIG>
__global__ void __launch_bounds__((TBM / 4) * (TBN / 4)) gemm_f64_kernel(GemmDesc g) {
    constexpr int NT = (TBM / 4) * (TBN / 4);
    constexpr int TX = TBN / 4;
    if (ct_skip(g.skip)) return;
    __shared__ double As[BK][TBM + 1];
    __shared__ double Bs[BK][TBN + 1];

    // blockIdx.z = batch * ksplit + k-chunk
    const int64_t ks = (int64_t)blockIdx.z % g.ksplit;
    const int64_t bz = (int64_t)blockIdx.z / g.ksplit;
    const int64_t b1 = bz / g.nb0, b0 = bz % g.nb0;
    const double* A = g.A + b1 * g.sA1 + b0 * g.sA0;
    const double* B = g.B + b1 * g.sB1 + b0 * g.sB0;
    double* C = g.C + b1 * g.sC1 + b0 * g.sC0;

    const int64_t m0 = (int64_t)blockIdx.y * TBM, n0 = (int64_t)blockIdx.x * TBN;
    const int tid = threadIdx.x, tx = tid % TX, ty = tid / TX;
    if (g.tri == 1 && n0 >= m0 + TBM) return;   // tile strictly above the diagonal
    int64_t kend = (g.tri == 2 && m0 + TBM < g.K) ? m0 + TBM : g.K;
    int64_t kbeg = 0;
    if (g.ksplit > 1) {
        const int64_t chunk = ((g.K + g.ksplit - 1) / g.ksplit + BK - 1) / BK * BK;
        kbeg = ks * chunk;
        if (kbeg + chunk < kend) kend = kbeg + chunk;
    }

    double acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;

    for (int64_t k0 = kbeg; k0 < kend; k0 += BK) {
#pragma unroll
        for (int r = 0; r < (BK * TBM) / NT; ++r) {
            const int e = tid + NT * r;
            int mm, kk;
            if (A_K_CONTIG) { kk = e % BK; mm = e / BK; }
            else            { mm = e % TBM; kk = e / TBM; }
            const int64_t gm = m0 + mm, gk = k0 + kk;
            As[kk][mm] = (gm < g.M && gk < kend) ? A[gm * g.sAm + gk * g.sAk] : 0.0;
        }
#pragma unroll
        for (int r = 0; r < (BK * TBN) / NT; ++r) {
            const int e = tid + NT * r;
            int nn, kk;
            if (B_N_CONTIG) { nn = e % TBN; kk = e / TBN; }
            else            { kk = e % BK; nn = e / BK; }
            const int64_t gn = n0 + nn, gk = k0 + kk;
            Bs[kk][nn] = (gn < g.N && gk < kend) ? B[gk * g.sBk + gn * g.sBn] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            double a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + (TBM / 4) * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + (TBN / 4) * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int64_t gm = m0 + ty + (TBM / 4) * i;
        if (gm >= g.M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int64_t gn = n0 + tx + (TBN / 4) * j;
            if (gn >= g.N) continue;
            if (g.ksplit > 1) {
                g.part[(ks * g.M + gm) * g.N + gn] = acc[i][j];
                continue;
            }
            double* c = C + gm * g.sCm + gn * g.sCn;
            double v = g.alpha * acc[i][j];
            if (g.beta != 0.0) v = fma(g.beta, *c, v);
            *c = v;
        }
    }
}

// C = alpha * sum_ks part[ks] + beta * C, the partial sums added in a fixed
// order (deterministic); tiles the GEMM kernel skips (tri == 1) stay untouched.
__global__ void splitk_reduce_kernel(GemmDesc g, int tile) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < g.M * g.N;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t gm = t / g.N, gn = t % g.N;
        if (g.tri == 1 && (gn / tile) * tile >= (gm / tile) * tile + tile) continue;
        double a = 0.0;
        for (int64_t ks = 0; ks < g.ksplit; ++ks) a += g.part[(ks * g.M + gm) * g.N + gn];
        double* c = g.C + gm * g.sCm + gn * g.sCn;
        double v = g.alpha * a;
        if (g.beta != 0.0) v = fma(g.beta, *c, v);
        *c = v;
    }
}

template <int TBM, int TBN>
int launch_tiles(ct_handle* h, const GemmDesc& g, int64_t nb) {
    dim3 grid((unsigned)ct_cdiv(g.N, TBN), (unsigned)ct_cdiv(g.M, TBM), (unsigned)(nb * g.ksplit));
    if (grid.y > 65535 || grid.z > 65535) {
        ct_seterr(h, "gemm grid too large (M=%lld nb=%lld)", (long long)g.M, (long long)nb);
        return CT_ERR_UNSUPPORTED;
    }
    constexpr int nt = (TBM / 4) * (TBN / 4);
    const bool ak = (g.sAk == 1);
    const bool bn = (g.sBn == 1);
    if (ak && bn) { gemm_f64_kernel<TBM, TBN, true, true><<<grid, nt, 0, h->stream>>>(g); ct_note_launch(); }
    else if (ak) { gemm_f64_kernel<TBM, TBN, true, false><<<grid, nt, 0, h->stream>>>(g); ct_note_launch(); }
    else if (bn) { gemm_f64_kernel<TBM, TBN, false, true><<<grid, nt, 0, h->stream>>>(g); ct_note_launch(); }
    else { gemm_f64_kernel<TBM, TBN, false, false><<<grid, nt, 0, h->stream>>>(g); ct_note_launch(); }
    CT_LAUNCH_CHECK(h);
    if (g.ksplit > 1) {
        const int64_t tot = g.M * g.N;
        int64_t blocks = ct_cdiv(tot, 256);
        if (blocks > 4 * (int64_t)h->num_sms) blocks = 4 * (int64_t)h->num_sms;
        splitk_reduce_kernel<<<(unsigned)blocks, 256, 0, h->stream>>>(g, TBM); ct_note_launch();
        CT_LAUNCH_CHECK(h);
    }
    return CT_OK;
}

}  // namespace

int ct_gemm_f64_launch(ct_handle* h, const GemmDesc& g) {
    if (g.M <= 0 || g.N <= 0) return CT_OK;
    const int64_t nb = g.nb1 * g.nb0;
    if (nb <= 0) return CT_OK;
    if (g.K <= 0 && g.beta == 1.0) return CT_OK;  // C unchanged; K = 0 otherwise gives C = beta*C
    GemmDesc gg = g;
    gg.ksplit = 1;
    gg.part = nullptr;
    const int64_t sms = h->num_sms;
    // the FP64 pipe of one SM bounds a CTA here, so the launch needs at least
    // one CTA per SM: 64 x 64 tiles when there are two per SM, else 32 x 32
    // tiles, with K split over the idle SMs when even those are too few
    // tiles that do work (tri == 1 skips those strictly above the diagonal)
    auto active = [&](int64_t t) {
        const int64_t tm = ct_cdiv(g.M, t), tn = ct_cdiv(g.N, t);
        if (g.tri != 1) return tm * tn * nb;
        int64_t a = 0;
        for (int64_t i = 0; i < tm; ++i) a += std::min<int64_t>(tn, i + 1);
        return a * nb;
    };
    // (measured: 32 x 32 tiles, several CTAs per SM, beat 64 x 64 tiles with
    // split K on a 1024 x 1024 x 2048 lower-only product, 2.7 vs 3.1 ms)
    if (active(64) >= 2 * sms) return launch_tiles<64, 64>(h, gg, nb);
    const int64_t tiles = active(32);
    if (nb == 1 && tiles < sms && g.K >= 64) {
        int64_t ks = ct_cdiv(sms, tiles);
        if (ks > g.K / 32) ks = g.K / 32;
        if (h->no_alloc) {
            // partials only in the caller's fixed region, as many K pieces as it holds
            const int64_t fit = (int64_t)(h->splitk_fixed_cap / (size_t)(g.M * g.N));
            if (ks > fit) ks = fit;
            if (ks > 1) {
                gg.ksplit = ks;
                gg.part = h->splitk_fixed;
            }
        } else if (ks > 1) {
            const size_t need = (size_t)(ks * g.M * g.N);
            if (h->splitk_cap < need) {
                if (h->splitk) cudaFree(h->splitk);
                h->splitk = nullptr;
                h->splitk_cap = 0;
                CT_CUDA(h, cudaMalloc((void**)&h->splitk, need * sizeof(double)));
                h->splitk_cap = need;
            }
            gg.ksplit = ks;
            gg.part = h->splitk;
        }
    }
    return launch_tiles<32, 32>(h, gg, nb);
}
