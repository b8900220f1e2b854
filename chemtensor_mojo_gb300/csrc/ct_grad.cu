// Adjoint of the environment chain: dE/dA_i for E = <psi|H|psi> / <psi|psi>.
//
// The scalar F = <psi|H|psi> is the end of the left-environment chain
// L_{i+1} = update_left(L_i, A_i, W_i) (environments.mojo:99-201).  Its
// reverse-mode adjoint runs the chain backwards: the adjoint of L_{i+1} is the
// right environment R_{i+1} (environments.mojo:309-417), and the local
// adjoint of A_i is the one-site effective Hamiltonian applied to A_i,
//     dF/dA_i = 2 H1(L_i, W_i, R_{i+1}) A_i       (H real symmetric),
// with the same for N = <psi|psi> through identity-MPO environments, so
//     dE/dA_i = 2 (H1 A_i - E N1 A_i) / N.
// The MPS need not be canonical, nor normalised: every environment is
// divided by a power of two near its norm after each step (exact), and the
// exponents, kept on the host, enter the final factors -- the FP32 operand
// planes of the mixed form would otherwise under- or overflow along a chain of
// unnormalised tensors.  Left environments are kept only every
// k-th site (checkpoints) and recomputed one segment at a time during the
// backward sweep: memory ~ (L/k + k) environments instead of L.
#include <math.h>
#include <algorithm>
#include <vector>

#include "ct_ops.cuh"

namespace {

struct Buf {
    double* p = nullptr;
    ~Buf() {
        if (p) cudaFree(p);
    }
};

// g = fH hA - fN nA; the host folds 2/N, the energy and the environments'
// power-of-two scales into the two factors
__global__ void grad_combine_kernel(int64_t n, const double* hA, const double* nA, double fH, double fN, double* g) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        g[i] = fH * hA[i] - fN * nA[i];
}

}  // namespace

// one-site effective Hamiltonian: out[Dl', s', Dr'] = sum L[wl,Dl,Dl'] A[Dl,s,Dr] W[wl,s,s',wr] R[wr,Dr,Dr']
size_t ct_heff1_ws_bytes(int64_t Dl, int64_t d, int64_t Dr, int64_t wl, int64_t wr) {
    return ct_bytes((size_t)(Dl * wl * d * Dr), 8) + ct_bytes((size_t)(Dl * d * wr * Dr), 8) +
           ct_bytes((size_t)((d * wr) * (wl * d)), 8) + 1024;
}

int ct_heff1_run(ct_handle* h, Arena& ar, const double* L, const double* A, const double* W, const double* R,
                 double* out, int64_t Dl, int64_t d, int64_t Dr, int64_t wl, int64_t wr) {
    double* T1 = ar.take<double>((size_t)(Dl * wl * d * Dr));
    double* T2 = ar.take<double>((size_t)(Dl * d * wr * Dr));
    double* Wt = ar.take<double>((size_t)((d * wr) * (wl * d)));
    if (!T1 || !T2 || !Wt) return CT_ERR_OOM;
    CT_TRY(ct_build_wt_left(h, W, Wt, wl, d, wr));
    const int64_t n1 = d * Dr;
    {   // T1[Dl', wl, (s Dr)] = sum_Dl L[wl, Dl, Dl'] A[Dl, (s Dr)]
        GemmDesc g{};
        g.M = Dl; g.N = n1; g.K = Dl;
        g.A = L; g.sAm = 1; g.sAk = Dl;
        g.B = A; g.sBk = n1; g.sBn = 1;
        g.C = T1; g.sCm = wl * n1; g.sCn = 1;
        g.alpha = 1.0; g.beta = 0.0; g.nb1 = wl; g.nb0 = 1; g.sA1 = Dl * Dl; g.sC1 = n1;
        CT_TRY(ct_gemm_f64_launch(h, g));
    }
    {   // T2[Dl', s', wr, Dr] = sum_(wl s) W[wl,s,s',wr] T1
        MpoDesc m{};
        m.O = Dl; m.K = wl * d; m.J = d * wr; m.I = Dr;
        m.in = T1; m.sIo = wl * d * Dr; m.sIk = Dr; m.sIi = 1;
        m.out = T2; m.sOo = d * wr * Dr; m.sOi = 1; m.J0 = m.J; m.sOj1 = 0; m.sOj0 = Dr;
        m.Wt = Wt;
        CT_TRY(ct_mpo_apply_f64_launch(h, m));
    }
    {   // out[(Dl' s'), Dr'] = sum_(wr Dr) T2[(Dl' s'), (wr Dr)] R[(wr Dr), Dr']
        GemmDesc g{};
        g.M = Dl * d; g.N = Dr; g.K = wr * Dr;
        g.A = T2; g.sAm = wr * Dr; g.sAk = 1;
        g.B = R; g.sBk = Dr; g.sBn = 1;
        g.C = out; g.sCm = Dr; g.sCn = 1;
        g.alpha = 1.0; g.beta = 0.0; g.nb1 = 1; g.nb0 = 1;
        CT_TRY(ct_gemm_f64_launch(h, g));
    }
    return CT_OK;
}

extern "C" {

int ct_energy_grad(ct_handle* h, int prec, int N, int d, const int64_t* mpo_dims, const double* const* mpo_sites,
                   const int64_t* bd, const double* const* sites, double* const* grads, int checkpoint_every,
                   double* energy_host) {
    if (!h) return CT_ERR_INVALID;
    if (!mpo_dims || !mpo_sites || !bd || !sites || !grads || N < 1 || d < 1) {
        ct_seterr(h, "ct_energy_grad: bad arguments");
        return CT_ERR_INVALID;
    }
    if (prec != CT_PREC_FP64 && !(prec == CT_PREC_TF32X3 && ct_tc_available(h))) {
        ct_seterr(h, "ct_energy_grad: precision %d is not available", prec);
        return CT_ERR_UNSUPPORTED;
    }
    const bool tc = prec == CT_PREC_TF32X3;
    for (int i = 0; i < N; ++i)
        if (!sites[i] || !grads[i] || !mpo_sites[i]) return CT_ERR_INVALID;
    const int k = (checkpoint_every > 0) ? std::min(checkpoint_every, N) : N;
    // identity MPO site for the norm chain
    Buf Wid;
    CT_CUDA(h, cudaMalloc((void**)&Wid.p, (size_t)(d * d) * sizeof(double)));
    {
        std::vector<double> idh((size_t)(d * d), 0.0);
        for (int s = 0; s < d; ++s) idh[(size_t)(s * d + s)] = 1.0;
        CT_CUDA(h, cudaMemcpyAsync(Wid.p, idh.data(), idh.size() * sizeof(double), cudaMemcpyHostToDevice,
                                   h->stream));
        CT_CUDA(h, cudaStreamSynchronize(h->stream));
    }
    auto hsize = [&](int i) { return (size_t)(mpo_dims[i] * bd[i] * bd[i]); };
    auto nsize = [&](int i) { return (size_t)(bd[i] * bd[i]); };
    size_t maxh = 1, maxn = 1, maxsite = 1, ws = 1;
    for (int i = 0; i <= N; ++i) {
        maxh = std::max(maxh, hsize(i));
        maxn = std::max(maxn, nsize(i));
    }
    for (int i = 0; i < N; ++i) {
        maxsite = std::max(maxsite, (size_t)(bd[i] * d * bd[i + 1]));
        ws = std::max(ws, ct_env_ws_bytes(prec, bd[i], d, bd[i + 1], mpo_dims[i], mpo_dims[i + 1]));
        ws = std::max(ws, tc ? ct_tc_heff1_ws_bytes(bd[i], d, bd[i + 1], mpo_dims[i], mpo_dims[i + 1])
                             : ct_heff1_ws_bytes(bd[i], d, bd[i + 1], mpo_dims[i], mpo_dims[i + 1]));
    }
    CT_TRY(ct_reserve(h, ws));
    const int ncp = (N + k - 1) / k;
    std::vector<Buf> cpH(ncp), cpN(ncp), segH(k + 1), segN(k + 1);
    for (int c = 0; c < ncp; ++c) {
        CT_CUDA(h, cudaMalloc((void**)&cpH[c].p, hsize(c * k) * sizeof(double)));
        CT_CUDA(h, cudaMalloc((void**)&cpN[c].p, nsize(c * k) * sizeof(double)));
    }
    for (int j = 0; j <= k; ++j) {
        CT_CUDA(h, cudaMalloc((void**)&segH[j].p, maxh * sizeof(double)));
        CT_CUDA(h, cudaMalloc((void**)&segN[j].p, maxn * sizeof(double)));
    }
    Buf RH0, RH1, RN0, RN1, hA, nA, sc;
    CT_CUDA(h, cudaMalloc((void**)&RH0.p, maxh * sizeof(double)));
    CT_CUDA(h, cudaMalloc((void**)&RH1.p, maxh * sizeof(double)));
    CT_CUDA(h, cudaMalloc((void**)&RN0.p, maxn * sizeof(double)));
    CT_CUDA(h, cudaMalloc((void**)&RN1.p, maxn * sizeof(double)));
    CT_CUDA(h, cudaMalloc((void**)&hA.p, maxsite * sizeof(double)));
    CT_CUDA(h, cudaMalloc((void**)&nA.p, maxsite * sizeof(double)));
    CT_CUDA(h, cudaMalloc((void**)&sc.p, 2 * sizeof(double)));

    // exponent e with 2^e near the norm of E (n values); E /= 2^e
    auto renorm = [&](double* E, int64_t n, int* e_out) -> int {
        CT_TRY(ct_reduce_nrm2sq(h, n, E, h->d_scalars + SC_TMP0, nullptr));
        double v = 0.0;
        CT_CUDA(h, cudaMemcpyAsync(&v, h->d_scalars + SC_TMP0, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        CT_CUDA(h, cudaStreamSynchronize(h->stream));
        if (!std::isfinite(v)) {
            ct_seterr(h, "ct_energy_grad: environment norm is not finite");
            return CT_ERR_NONFINITE;
        }
        int e = 0;
        if (v > 0.0) e = ilogb(sqrt(v));
        if (e != 0) CT_TRY(ct_vec_scale_launch(h, n, ldexp(1.0, -e), E));
        *e_out = e;
        return CT_OK;
    };
    auto scale_by = [&](double* E, int64_t n, int e) -> int {
        return e != 0 ? ct_vec_scale_launch(h, n, ldexp(1.0, -e), E) : CT_OK;
    };
    // per-step exponents of the left chains (index = environment index) and the
    // cumulative ones of the left and right chains
    std::vector<int> stepH(N + 1, 0), stepN(N + 1, 0);
    std::vector<long long> cumHL(N + 1, 0), cumNL(N + 1, 0), cumHR(N + 1, 0), cumNR(N + 1, 0);

    auto left_step = [&](const double* Lh, const double* Ln, int i, double* outH, double* outN) -> int {
        {
            Arena ar(h);
            CT_TRY(ct_env_left_run(h, ar, prec, Lh, sites[i], mpo_sites[i], outH, bd[i], d, bd[i + 1],
                                   mpo_dims[i], mpo_dims[i + 1]));
        }
        Arena ar(h);
        return ct_env_left_run(h, ar, prec, Ln, sites[i], Wid.p, outN, bd[i], d, bd[i + 1], 1, 1);
    };

    // forward: left chain with checkpoints at multiples of k
    CT_TRY(ct_identity_env(h, segH[0].p, mpo_dims[0], bd[0]));
    CT_TRY(ct_identity_env(h, segN[0].p, 1, bd[0]));
    {
        double* ah = segH[0].p;
        double* an = segN[0].p;
        double* bh = segH[1].p;
        double* bn = segN[1].p;
        for (int i = 0; i < N; ++i) {
            if (i % k == 0) {
                CT_TRY(ct_copy(h, cpH[i / k].p, ah, (int64_t)hsize(i)));
                CT_TRY(ct_copy(h, cpN[i / k].p, an, (int64_t)nsize(i)));
            }
            CT_TRY(left_step(ah, an, i, bh, bn));
            CT_TRY(renorm(bh, (int64_t)hsize(i + 1), &stepH[i + 1]));
            CT_TRY(renorm(bn, (int64_t)nsize(i + 1), &stepN[i + 1]));
            cumHL[i + 1] = cumHL[i] + stepH[i + 1];
            cumNL[i + 1] = cumNL[i] + stepN[i + 1];
            std::swap(ah, bh);
            std::swap(an, bn);
        }
        // final environments are [w_N, D_N, D_N] = [1, 1, 1] for a closed chain: element 0
        CT_CUDA(h, cudaMemcpyAsync(sc.p, ah, sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
        CT_CUDA(h, cudaMemcpyAsync(sc.p + 1, an, sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    }
    double fn[2];
    CT_CUDA(h, cudaMemcpyAsync(fn, sc.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CT_CUDA(h, cudaStreamSynchronize(h->stream));
    if (!(fn[1] > 0.0)) {
        ct_seterr(h, "ct_energy_grad: <psi|psi> = %g", fn[1]);
        return CT_ERR_ZERO_NORM;
    }
    // F = fn[0] 2^cumHL[N], N = fn[1] 2^cumNL[N]
    const double Nsc = fn[1];
    const long long eN = cumNL[N];
    const double energy = ldexp(fn[0] / fn[1], (int)(cumHL[N] - eN));
    if (energy_host) *energy_host = energy;

    // backward: right chain (the adjoint of the left chain), segments in reverse
    double* rh = RH0.p;
    double* rn = RN0.p;
    double* rh2 = RH1.p;
    double* rn2 = RN1.p;
    CT_TRY(ct_identity_env(h, rh, mpo_dims[N], bd[N]));
    CT_TRY(ct_identity_env(h, rn, 1, bd[N]));
    for (int c = ncp - 1; c >= 0; --c) {
        const int start = c * k, end = std::min(start + k, N);
        CT_TRY(ct_copy(h, segH[0].p, cpH[c].p, (int64_t)hsize(start)));
        CT_TRY(ct_copy(h, segN[0].p, cpN[c].p, (int64_t)nsize(start)));
        for (int i = start; i < end - 1; ++i) {
            CT_TRY(left_step(segH[i - start].p, segN[i - start].p, i, segH[i - start + 1].p, segN[i - start + 1].p));
            CT_TRY(scale_by(segH[i - start + 1].p, (int64_t)hsize(i + 1), stepH[i + 1]));
            CT_TRY(scale_by(segN[i - start + 1].p, (int64_t)nsize(i + 1), stepN[i + 1]));
        }
        for (int i = end - 1; i >= start; --i) {
            const int64_t Dl = bd[i], Dr = bd[i + 1], wl = mpo_dims[i], wr = mpo_dims[i + 1];
            {
                Arena ar(h);
                CT_TRY((tc ? ct_tc_heff1_run : ct_heff1_run)(h, ar, segH[i - start].p, sites[i], mpo_sites[i], rh,
                                                             hA.p, Dl, d, Dr, wl, wr));
            }
            {
                Arena ar(h);
                CT_TRY((tc ? ct_tc_heff1_run : ct_heff1_run)(h, ar, segN[i - start].p, sites[i], Wid.p, rn, nA.p, Dl,
                                                             d, Dr, 1, 1));
            }
            const int64_t ns = Dl * d * Dr;
            int g = (int)ct_cdiv(ns, 256);
            if (g > h->num_sms * 16) g = h->num_sms * 16;
            if (g < 1) g = 1;
            // g = 2 (hA_true - E nA_true) / N_true with X_true = X 2^(left + right exponents)
            const double fH = ldexp(2.0 / Nsc, (int)(cumHL[i] + cumHR[i + 1] - eN));
            const double fNn = ldexp(2.0 * energy / Nsc, (int)(cumNL[i] + cumNR[i + 1] - eN));
            grad_combine_kernel<<<g, 256, 0, h->stream>>>(ns, hA.p, nA.p, fH, fNn, grads[i]); ct_note_launch();
            CT_LAUNCH_CHECK(h);
            if (i > 0) {
                {
                    Arena ar(h);
                    CT_TRY(ct_env_right_run(h, ar, prec, rh, sites[i], mpo_sites[i], rh2, Dl, d, Dr, wl, wr));
                }
                Arena ar(h);
                CT_TRY(ct_env_right_run(h, ar, prec, rn, sites[i], Wid.p, rn2, Dl, d, Dr, 1, 1));
                int eh = 0, en = 0;
                CT_TRY(renorm(rh2, (int64_t)hsize(i), &eh));
                CT_TRY(renorm(rn2, (int64_t)nsize(i), &en));
                cumHR[i] = cumHR[i + 1] + eh;
                cumNR[i] = cumNR[i + 1] + en;
                std::swap(rh, rh2);
                std::swap(rn, rn2);
            }
        }
    }
    CT_CUDA(h, cudaStreamSynchronize(h->stream));
    int st = 0;
    CT_CUDA(h, cudaMemcpy(&st, h->d_status, sizeof(int), cudaMemcpyDeviceToHost));
    if (st) {
        cudaMemset(h->d_status, 0, sizeof(int));
        return st;
    }
    return CT_OK;
}

}  // extern "C"
