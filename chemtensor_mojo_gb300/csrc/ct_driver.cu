// Native sweep driver (dmrg_two_site, dmrg.mojo:377-483 and
// dmrg_local_update_two_site, dmrg.mojo:759-844), MPS utilities and the
// seeded initial state (rng_c_compat.mojo:14-231).
//
// The sweep runs entirely on the device: theta build, Lanczos (with the
// tridiagonal eigensolve), SVD split and environment update per bond; the
// host reads back only the local energy and the kept bond dimension per bond
// (one 16-byte copy), which it needs to size the next launches.
#include <math.h>
#include <chrono>
#include <vector>

#include "ct_ops.cuh"

namespace {

struct DevBuf {
    double* p = nullptr;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
};

struct EventTimer {
    cudaEvent_t a = nullptr, b = nullptr;
    EventTimer() {
        cudaEventCreate(&a);
        cudaEventCreate(&b);
    }
    ~EventTimer() {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
};

double heff_flops_general(int64_t Dl, int64_t d, int64_t Dr, int64_t wL, int64_t wM, int64_t wR) {
    const double s1 = 2.0 * (double)(Dl * wL) * (double)(d * d * Dr) * (double)Dl;
    const double s2 = 2.0 * (double)(Dl * d * Dr) * (double)(wL * d) * (double)(d * wM);
    const double s3 = 2.0 * (double)(Dl * Dr * d) * (double)(wM * d) * (double)(d * wR);
    const double s4 = 2.0 * (double)(Dl * d * d) * (double)Dr * (double)(wR * Dr);
    return s1 + s2 + s3 + s4;
}

double env_flops_general(int64_t Dl, int64_t d, int64_t Dr, int64_t wL, int64_t wR) {
    const double s1 = 2.0 * (double)(Dl * wL) * (double)(d * Dr) * (double)Dl;
    const double s2 = 2.0 * (double)(Dl * Dr) * (double)(wL * d) * (double)(d * wR);
    const double s3 = 2.0 * (double)(wR * Dr) * (double)Dr * (double)(Dl * d);
    return s1 + s2 + s3;
}

int64_t sat_mul(int64_t a, int64_t b, int64_t cap) {
    if (a >= cap || b >= cap) return cap;
    const int64_t r = a * b;
    return r > cap ? cap : r;
}

}  // namespace

extern "C" {

int ct_dmrg_two_site(ct_handle* h, const ct_dmrg_params* P, int N, int d, const int64_t* mpo_dims,
                     const double* const* mpo_sites, int64_t* bd, double* const* mps_sites,
                     const int64_t* site_capacity, double* energy_host, double* sweep_energies_host,
                     int* sweeps_done_host, double* discarded_host, ct_dmrg_stats* stats_host) {
    if (!h) return CT_ERR_INVALID;
    if (!P || !mpo_dims || !mpo_sites || !bd || !mps_sites || !site_capacity || !energy_host) {
        ct_seterr(h, "ct_dmrg_two_site: null argument");
        return CT_ERR_INVALID;
    }
    if (!P->two_site) {
        ct_seterr(h, "Only two-site DMRG is currently implemented");
        return CT_ERR_UNSUPPORTED;
    }
    if (N < 2) {
        ct_seterr(h, "DMRG requires at least 2 sites");
        return CT_ERR_INVALID;
    }
    if (d < 1 || P->chi_max < 1 || P->max_krylov_iter < 1 || P->max_krylov_iter > 64 || P->num_sweeps < 0) {
        ct_seterr(h, "ct_dmrg_two_site: bad parameters");
        return CT_ERR_INVALID;
    }
    if (P->prec != CT_PREC_FP64 && !(P->prec == CT_PREC_TF32X3 && ct_tc_available(h))) {
        ct_seterr(h, "precision %d not available", P->prec);
        return CT_ERR_UNSUPPORTED;
    }
    for (int i = 0; i <= N; ++i)
        if (bd[i] < 1 || mpo_dims[i] < 1) return CT_ERR_SHAPE;
    for (int i = 0; i < N; ++i) {
        if (!mps_sites[i] || !mpo_sites[i]) return CT_ERR_INVALID;
        if (bd[i] * d * bd[i + 1] > site_capacity[i]) {
            ct_seterr(h, "site %d holds more elements than its capacity", i);
            return CT_ERR_SHAPE;
        }
    }
    auto t_start = std::chrono::steady_clock::now();
    const int prec = P->prec;

    // capacities of every bond under two-site growth
    std::vector<int64_t> cap(N + 1);
    {
        std::vector<int64_t> lc(N + 1), rc(N + 1);
        const int64_t big = (int64_t)1 << 40;
        lc[0] = bd[0];
        for (int k = 1; k <= N; ++k) lc[k] = sat_mul(lc[k - 1], d, big);
        rc[N] = bd[N];
        for (int k = N - 1; k >= 0; --k) rc[k] = sat_mul(rc[k + 1], d, big);
        for (int k = 0; k <= N; ++k) {
            int64_t c = std::min<int64_t>(P->chi_max, std::min(lc[k], rc[k]));
            if (k == 0 || k == N) c = bd[k];
            cap[k] = std::max(c, bd[k]);
        }
    }
    // environments
    std::vector<DevBuf> Lenv(N + 1), Renv(N + 1);
    for (int k = 0; k <= N; ++k) {
        const size_t n = (size_t)(mpo_dims[k] * cap[k] * cap[k]);
        CT_CUDA(h, cudaMalloc((void**)&Lenv[k].p, n * sizeof(double)));
        CT_CUDA(h, cudaMalloc((void**)&Renv[k].p, n * sizeof(double)));
    }
    int64_t th_cap = 1;
    for (int i = 0; i + 2 <= N; ++i) th_cap = std::max<int64_t>(th_cap, cap[i] * d * d * cap[i + 2]);
    DevBuf th, th_opt;
    CT_CUDA(h, cudaMalloc((void**)&th.p, (size_t)th_cap * sizeof(double)));
    CT_CUDA(h, cudaMalloc((void**)&th_opt.p, (size_t)th_cap * sizeof(double)));

    // mixed form: rotations of the last split per (bond, direction), FP32, to
    // warm-start the next sweep's Jacobi at the same bond
    struct QCache {
        float* p = nullptr;
        int64_t cap = 0;     // elements
        int64_t m = -1, n = -1;
        ~QCache() {
            if (p) cudaFree(p);
        }
    };
    std::vector<QCache> qcache((size_t)(2 * N));
    if (h->basis_cache.size() < (size_t)(2 * N)) h->basis_cache.resize((size_t)(2 * N));
    if (!P->keep_bases)
        for (auto& b : h->basis_cache) b.len = b.c = -1;

    EventTimer ev_l, ev_s, ev_e;
    uint64_t cold_seq = 0;   // seeds of the random start rows of first-visit splits
    ct_dmrg_stats st{};
    std::vector<double> disc_all;
    const int64_t handovers0 = h->mixed_fp64_splits;

    // build_right_environments (environments.mojo:420-472)
    CT_TRY(ct_identity_env(h, Renv[N].p, mpo_dims[N], bd[N]));
    CT_CUDA(h, cudaEventRecord(ev_e.a, h->stream));
    for (int i = N - 1; i >= 0; --i) {
        CT_TRY(ct_reserve(h, ct_env_ws_bytes(prec, bd[i], d, bd[i + 1], mpo_dims[i], mpo_dims[i + 1])));
        Arena ar(h);
        CT_TRY(ct_env_right_run(h, ar, prec, Renv[i + 1].p, mps_sites[i], mpo_sites[i], Renv[i].p, bd[i], d,
                                bd[i + 1], mpo_dims[i], mpo_dims[i + 1]));
        st.env_flops += env_flops_general(bd[i], d, bd[i + 1], mpo_dims[i], mpo_dims[i + 1]);
    }
    CT_CUDA(h, cudaEventRecord(ev_e.b, h->stream));
    CT_TRY(ct_identity_env(h, Lenv[0].p, mpo_dims[0], bd[0]));
    CT_CUDA(h, cudaStreamSynchronize(h->stream));
    {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev_e.a, ev_e.b);
        st.seconds_env += ms * 1e-3;
    }

    auto local_update = [&](int i, bool l2r, double* E_out) -> int {
        const int64_t Dl = bd[i], Dm = bd[i + 1], Dr = bd[i + 2];
        const int64_t wL = mpo_dims[i], wM = mpo_dims[i + 1], wR = mpo_dims[i + 2];
        const int64_t m = Dl * d, n = d * Dr;
        size_t need = ct_lanczos_ws_bytes(prec, Dl, d, Dr, wL, wM, wR, P->max_krylov_iter);
        need = std::max(need, ct_theta_ws_bytes(prec, Dl, d, Dm, Dr));
        need = std::max(need, ct_split_ws_bytes(prec, m, n, P->chi_max, l2r ? 0 : 1));
        // mixed form, large bonds: the warm subspace split when the other
        // direction kept a basis of this bond -- where chi_max binds, and with
        // eps_trunc = 0 also where every state is kept (then any orthonormal
        // basis of the whole space will do); the bases are kept on every large
        // bond, so a bond that starts binding has one
        const bool mixed_large = (prec == CT_PREC_TF32X3) && P->split_power_steps >= 0 &&
                                 !ct_svd_is_small(m, n, l2r ? 0 : 1);
        const bool binding = (int64_t)P->chi_max < std::min(m, n);
        const bool use_subspace = mixed_large && (binding || P->eps_trunc <= 0.0);
        const int64_t c_sub = std::min<int64_t>(P->chi_max, std::min(m, n));
        if (mixed_large) {
            need = std::max(need, ct_split_subspace_ws_bytes(m, n, c_sub));
            // short-side Jacobi + gauge move: the basis rows next to the subspace split's workspace
            need = std::max(need, ct_split_subspace_ws_bytes(m, n, c_sub) + ct_bytes(c_sub * std::max(m, n), 8));
            need = std::max(need, ct_split_ws_bytes(prec, m, n, P->chi_max, l2r ? 1 : 0));
        }
        const int64_t chi_ub = std::min<int64_t>(std::min(m, n), P->chi_max);
        need = std::max(need, l2r ? ct_env_ws_bytes(prec, Dl, d, chi_ub, wL, wM)
                                  : ct_env_ws_bytes(prec, chi_ub, d, Dr, wM, wR));
        CT_TRY(ct_reserve(h, need));
        // The mixed form always reorthogonalises its Krylov basis: with TF32-level
        // H_eff rounding the plain recursion of the reference loses orthogonality on
        // some bonds and returns a poorer Ritz vector (measured on the XXZ chain at
        // chi = 256: single sweeps 1e-8 to 3.5e-5 above the FP64 form without it, all
        // within 5.7e-10 with it).  The FP64 form keeps the reference's plain Lanczos.
        // theta (dmrg.mojo:93-140)
        CT_CUDA(h, cudaEventRecord(ev_l.a, h->stream));
        CT_TRY(ct_theta_run(h, prec, mps_sites[i], mps_sites[i + 1], th.p, Dl, d, Dm, Dr));
        {
            Arena ar(h);
            LanczosResult lr;
            CT_TRY(ct_lanczos_run(h, ar, prec, th.p, th_opt.p, Lenv[i].p, Renv[i + 2].p, mpo_sites[i],
                                  mpo_sites[i + 1], Dl, d, Dr, wL, wM, wR, P->max_krylov_iter, P->krylov_tol,
                                  P->max_rotations, (P->reorth || prec == CT_PREC_TF32X3) ? 1 : 0, &lr));
        }
        CT_CUDA(h, cudaEventRecord(ev_l.b, h->stream));
        // split (dmrg.mojo:143-252): |theta|^2 then SVD
        CT_TRY(ct_reduce_nrm2sq(h, m * n, th_opt.p, h->d_scalars + SC_THETA_NSQ, nullptr));
        CT_TRY(ct_check_finite(h, h->d_scalars + SC_THETA_NSQ, nullptr));
        struct {
            double e;
            double tn;
            int nk;
        } hb{};
        CT_CUDA(h, cudaMemcpyAsync(&hb.e, h->d_scalars + SC_ENERGY, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        CT_CUDA(h, cudaMemcpyAsync(&hb.tn, h->d_scalars + SC_THETA_NSQ, sizeof(double), cudaMemcpyDeviceToHost,
                                   h->stream));
        CT_CUDA(h, cudaMemcpyAsync(&hb.nk, h->d_flags + FL_NUMITER, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
        const int64_t chi_bound = std::min<int64_t>(std::min(m, n), P->chi_max);
        if (Dl * d * chi_bound > site_capacity[i] || chi_bound * d * Dr > site_capacity[i + 1] ||
            chi_bound > cap[i + 1]) {
            ct_seterr(h, "bond %d: bond dimension bound %lld exceeds the site capacity", i, (long long)chi_bound);
            return CT_ERR_SHAPE;
        }
        CT_CUDA(h, cudaEventRecord(ev_s.a, h->stream));
        SvdOut so;
        bool last_split_subspace = false;
        {
            Arena ar(h);
            // kept bond bound by the capacity of the sites it is written into
            bool done_split = false;
            ct_handle::BasisCache* bc = nullptr;
            if (mixed_large) {
                // this split keeps its far-side basis in `own`; it starts from the
                // basis the last split of the bond in the other direction kept
                const int64_t c = c_sub, own_len = l2r ? m : n, src_len = l2r ? n : m;
                ct_handle::BasisCache& own = h->basis_cache[(size_t)(2 * i + (l2r ? 0 : 1))];
                const ct_handle::BasisCache& src = h->basis_cache[(size_t)(2 * i + (l2r ? 1 : 0))];
                bc = &own;
                if (own.cap < c * own_len) {
                    if (own.p) cudaFree(own.p);
                    own.p = nullptr;
                    own.cap = 0;
                    CT_CUDA(h, cudaMalloc((void**)&own.p, (size_t)(c * own_len) * sizeof(double)));
                    own.cap = c * own_len;
                }
                own.len = own.c = -1;
                if (use_subspace && src.p && src.len == src_len && src.c == c) {
                    // accepted when it loses at most 1.5x the weight of the bond's previous
                    // truncating visit (+1e-12); otherwise one retry with a power step more,
                    // accepted within 4x + 1e-8, before the Jacobi SVD
                    bool ok = false;
                    CT_TRY(ct_split_subspace(h, ar, th_opt.p, m, n, c, l2r ? 0 : 1, src.p, own.p,
                                             mps_sites[i], mps_sites[i + 1], h->d_scalars + SC_THETA_NSQ,
                                             P->eps_trunc, src.disc, 1.5, 1e-12, P->split_power_steps, false, 0,
                                             &so, &ok));
                    if (!ok && so.stale) {
                        if (P->verbose >= 2)
                            fprintf(stderr, "bond %d %s: subspace split stale (kept %.12g of %.12g), retrying\n", i,
                                    l2r ? "L->R" : "R->L", so.sum_s2_kept, so.sum_s2_all);
                        CT_TRY(ct_split_subspace(h, ar, th_opt.p, m, n, c, l2r ? 0 : 1, src.p, own.p,
                                                 mps_sites[i], mps_sites[i + 1], h->d_scalars + SC_THETA_NSQ,
                                                 P->eps_trunc, src.disc, 4.0, 1e-8, P->split_power_steps + 1, false,
                                                 0, &so, &ok));
                        st.stale_retries++;
                    }
                    done_split = ok;
                    last_split_subspace = ok;
                    if (P->verbose >= 2)
                        fprintf(stderr,
                                "bond %d %s: subspace split %s (pivot %.3g, pass-2 deviation %.2g%s, kept %.12g of "
                                "%.12g)\n",
                                i, l2r ? "L->R" : "R->L", ok ? "accepted" : "refused", so.min_pivot,
                                1.0 - so.min_pivot2,
                                so.chol_fail ? ", Cholesky failed" : "", so.sum_s2_kept, so.sum_s2_all);
                    if (ok) {
                        st.subspace_splits++;
                        own.len = own_len;
                        own.c = c;
                        own.disc = binding && so.sum_s2_all > 0.0 ? 1.0 - so.sum_s2_kept / so.sum_s2_all : -1.0;
                    }
                }
                if (!done_split && use_subspace && P->cold_power_steps >= 0) {
                    // first visit: rows the bond kept at a smaller chi (same length), then random rows
                    const size_t mark = ar.off;
                    double* X = ar.take<double>(c * src_len);
                    if (!X) return CT_ERR_OOM;
                    const bool reuse = src.p && src.len == src_len && src.c > 0 && src.c < c;
                    const uint64_t seed = 0x5DEECE66Dull * (uint64_t)(2 * i + (l2r ? 0 : 1)) + (uint64_t)(++cold_seq);
                    CT_TRY(ct_cold_basis(h, reuse ? src.p : nullptr, reuse ? src.c : 0, c, src_len, seed, X));
                    bool ok = false;
                    CT_TRY(ct_split_subspace(h, ar, th_opt.p, m, n, c, l2r ? 0 : 1, X, own.p, mps_sites[i],
                                             mps_sites[i + 1], h->d_scalars + SC_THETA_NSQ, P->eps_trunc, -1.0, 0.0,
                                             0.0, P->cold_power_steps, true, seed, &so, &ok));
                    ar.off = mark;
                    done_split = ok;
                    last_split_subspace = ok;
                    if (P->verbose >= 2)
                        fprintf(stderr, "bond %d %s: cold subspace split %s (%lld kept rows reused, %d rows completed)\n",
                                i, l2r ? "L->R" : "R->L", ok ? "accepted" : "refused", reuse ? (long long)src.c : 0ll,
                                so.replaced);
                    if (ok) {
                        st.subspace_splits++;
                        st.cold_splits++;
                        st.completed_rows += so.replaced;
                        own.len = own_len;
                        own.c = c;
                        own.disc = -1.0;   // no reference: the next visit must not be judged against it
                    }
                }
            }
            float* qc = nullptr;
            int warm = 0;
            if (!done_split && prec == CT_PREC_TF32X3 && !ct_svd_is_small(m, n, l2r ? 0 : 1)) {
                QCache& c = qcache[(size_t)(2 * i + (l2r ? 0 : 1))];
                const int64_t nv = l2r ? m : n;
                if (c.cap < nv * nv) {
                    if (c.p) cudaFree(c.p);
                    c.p = nullptr;
                    CT_CUDA(h, cudaMalloc((void**)&c.p, (size_t)(nv * nv) * sizeof(float)));
                    c.cap = nv * nv;
                    c.m = c.n = -1;
                }
                warm = (c.m == m && c.n == n) ? 1 : 0;
                qc = c.p;
                c.m = m;
                c.n = n;
            }
            if (!done_split && bc && (l2r ? m > n : m < n)) {
                // the canonical factor is on the long side: run the Jacobi on the
                // short side (the other direction), then move the gauge with the
                // subspace split started from that exact basis
                Arena ar2(h);
                SvdOut s0;
                CT_TRY(ct_split_run(h, ar2, prec, th_opt.p, m, n, P->chi_max, P->eps_trunc, l2r ? 1 : 0,
                                    mps_sites[i], mps_sites[i + 1], nullptr, h->d_scalars + SC_THETA_NSQ, &s0,
                                    nullptr, 0));
                if (s0.chi > 0) {
                    Arena ar3(h);
                    const int64_t c0 = s0.chi;
                    double* basis = ar3.take<double>(c0 * (l2r ? n : m));
                    if (!basis) return CT_ERR_OOM;
                    CT_TRY(ct_basis_from_split(h, l2r ? 1 : 0, mps_sites[i], mps_sites[i + 1], m, n, c0, basis));
                    SvdOut s1;
                    bool ok = false;
                    CT_TRY(ct_split_subspace(h, ar3, th_opt.p, m, n, c0, l2r ? 0 : 1, basis, bc->p,
                                             mps_sites[i], mps_sites[i + 1], h->d_scalars + SC_THETA_NSQ, 0.0,
                                             -1.0, 0.0, 0.0, 0, false, 0, &s1, &ok));
                    if (ok) {
                        so = s0;
                        done_split = true;
                        st.exact_splits++;
                        bc->len = l2r ? m : n;
                        bc->c = c0;
                        bc->disc = binding && so.sum_s2_all > 0.0 ? 1.0 - so.sum_s2_kept / so.sum_s2_all : -1.0;
                    }
                }
            }
            if (!done_split) {
                Arena ar2(h);
                CT_TRY(ct_split_run(h, ar2, prec, th_opt.p, m, n, P->chi_max, P->eps_trunc, l2r ? 0 : 1,
                                    mps_sites[i], mps_sites[i + 1], nullptr, h->d_scalars + SC_THETA_NSQ, &so, qc,
                                    warm));
                st.exact_splits++;
                if (bc && so.chi == c_sub) {
                    CT_TRY(ct_basis_from_split(h, l2r ? 0 : 1, mps_sites[i], mps_sites[i + 1], m, n, so.chi, bc->p));
                    bc->len = l2r ? m : n;
                    bc->c = so.chi;
                    // a split that truncated nothing is no reference for the loss of one that does
                    bc->disc = binding && so.sum_s2_all > 0.0 ? 1.0 - so.sum_s2_kept / so.sum_s2_all : -1.0;
                }
            }
        }
        CT_CUDA(h, cudaEventRecord(ev_s.b, h->stream));
        const int64_t chi = so.chi;
        if (chi <= 0) {
            // a device error (a non-finite theta, say) takes precedence over the empty truncation
            int dst0 = 0;
            CT_CUDA(h, cudaStreamSynchronize(h->stream));
            CT_CUDA(h, cudaMemcpy(&dst0, h->d_status, sizeof(int), cudaMemcpyDeviceToHost));
            if (dst0 != 0) {
                cudaMemset(h->d_status, 0, sizeof(int));
                ct_seterr(h, "bond %d: device status %d", i, dst0);
                return dst0;
            }
            ct_seterr(h, "bond %d: truncation kept no singular values", i);
            return CT_ERR_EMPTY;
        }
        bd[i + 1] = chi;
        CT_CUDA(h, cudaEventRecord(ev_e.a, h->stream));
        {
            Arena ar(h);
            if (l2r) {
                CT_TRY(ct_env_left_run(h, ar, prec, Lenv[i].p, mps_sites[i], mpo_sites[i], Lenv[i + 1].p, Dl, d, chi,
                                       wL, wM));
                st.env_flops += env_flops_general(Dl, d, chi, wL, wM);
            } else {
                CT_TRY(ct_env_right_run(h, ar, prec, Renv[i + 2].p, mps_sites[i + 1], mpo_sites[i + 1],
                                        Renv[i + 1].p, chi, d, Dr, wM, wR));
                st.env_flops += env_flops_general(chi, d, Dr, wM, wR);
            }
        }
        CT_CUDA(h, cudaEventRecord(ev_e.b, h->stream));
        CT_CUDA(h, cudaStreamSynchronize(h->stream));
        int dst = 0;
        CT_CUDA(h, cudaMemcpy(&dst, h->d_status, sizeof(int), cudaMemcpyDeviceToHost));
        if (dst != 0) {
            cudaMemset(h->d_status, 0, sizeof(int));
            ct_seterr(h, "bond %d: device status %d", i, dst);
            return dst;
        }
        float ms = 0.f, ms_l = 0.f;
        cudaEventElapsedTime(&ms_l, ev_l.a, ev_l.b);
        st.seconds_lanczos += ms_l * 1e-3;
        cudaEventElapsedTime(&ms, ev_s.a, ev_s.b);
        st.seconds_svd += ms * 1e-3;
        if (last_split_subspace) st.seconds_subspace += ms * 1e-3;
        if (P->verbose >= 2)
            fprintf(stderr, "bond %d %s: %lld x %lld -> chi %lld, lanczos %.3f ms (%d applies), %s split %.3f ms\n",
                    i, l2r ? "L->R" : "R->L", (long long)m, (long long)n, (long long)so.chi, (double)ms_l, hb.nk,
                    last_split_subspace ? "subspace" : "exact", (double)ms);
        cudaEventElapsedTime(&ms, ev_e.a, ev_e.b);
        st.seconds_env += ms * 1e-3;
        st.heff_applies += hb.nk;
        st.heff_flops += (double)hb.nk * heff_flops_general(Dl, d, Dr, wL, wM, wR);
        st.local_updates += 1;
        const double disc = (hb.tn > 0.0) ? (hb.tn - so.sum_s2_kept) / hb.tn : 0.0;
        st.max_discarded = std::max(st.max_discarded, disc);
        disc_all.push_back(disc);
        *E_out = hb.e;
        return CT_OK;
    };

    double energy = 0.0, prev = 0.0;
    int sweeps_done = 0;
    for (int sweep = 0; sweep < P->num_sweeps; ++sweep) {
        for (int i = 0; i <= N - 2; ++i) CT_TRY(local_update(i, true, &energy));
        for (int i = N - 2; i >= 0; --i) CT_TRY(local_update(i, false, &energy));
        if (sweep_energies_host) sweep_energies_host[sweep] = energy;
        sweeps_done = sweep + 1;
        if (P->verbose) {
            printf("[ctdmrg] sweep %d/%d energy %.15f\n", sweep + 1, P->num_sweeps, energy);
            fflush(stdout);
        }
        if (sweep > 0 && fabs(energy - prev) < P->energy_tol) break;
        prev = energy;
    }
    *energy_host = energy;
    st.energy_rayleigh = NAN;
    if (P->final_rayleigh) {
        const auto t_rq = std::chrono::steady_clock::now();
        double e = 0.0, nsq = 0.0;
        // the mixed form's FP64 energy with its products on the BF16 tensor cores (FP64-accurate
        // slicing); the FP64 form keeps its SIMT GEMMs
        const int rprec = (prec == CT_PREC_TF32X3) ? CT_PREC_FP64_TC : CT_PREC_FP64;
        CT_TRY(ct_mps_expectation(h, rprec, N, d, mpo_dims, mpo_sites, bd, (const double* const*)mps_sites,
                                  &e, &nsq));
        st.energy_rayleigh = e / nsq;
        st.seconds_rayleigh = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_rq).count();
    }
    if (sweeps_done_host) *sweeps_done_host = sweeps_done;
    if (discarded_host)
        for (size_t k = 0; k < disc_all.size(); ++k) discarded_host[k] = disc_all[k];
    st.seconds_total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    st.fp64_handovers = h->mixed_fp64_splits - handovers0;
    if (stats_host) *stats_host = st;
    return CT_OK;
}

int ct_mps_right_normalize(ct_handle* h, int N, int d, int64_t* bd, double* const* sites) {
    if (!h || !bd || !sites || N < 1 || d < 1) return CT_ERR_INVALID;
    int64_t maxel = 1, maxm = 1;
    for (int i = 0; i < N; ++i) {
        maxel = std::max<int64_t>(maxel, bd[i] * d * bd[i + 1]);
        maxm = std::max<int64_t>(maxm, bd[i]);
    }
    DevBuf US, tmp;
    CT_CUDA(h, cudaMalloc((void**)&US.p, (size_t)(maxm * maxm) * sizeof(double)));
    CT_CUDA(h, cudaMalloc((void**)&tmp.p, (size_t)maxel * sizeof(double)));
    for (int i = N - 1; i >= 1; --i) {
        const int64_t Dl = bd[i], Dr = bd[i + 1];
        const int64_t m = Dl, n = d * Dr;
        if (n < m) {
            ct_seterr(h, "site %d: left bond %lld exceeds d*right bond %lld; cannot right-normalise", i,
                      (long long)m, (long long)n);
            return CT_ERR_SHAPE;
        }
        CT_TRY(ct_reserve(h, ct_svd_ws_bytes(m, n, 1)));
        Arena ar(h);
        SvdOut so;
        // A_i = (U S) Vt ; A_i <- Vt, A_{i-1} <- A_{i-1} (U S); no truncation
        CT_TRY(ct_svd_run(h, ar, sites[i], m, n, m, 0.0, 1, US.p, tmp.p, nullptr, &so));
        if (so.chi != m) return CT_ERR_SHAPE;
        CT_TRY(ct_copy(h, sites[i], tmp.p, m * n));
        const int64_t Dp = bd[i - 1];
        GemmDesc g{};
        g.M = Dp * d; g.N = m; g.K = m;
        g.A = sites[i - 1]; g.sAm = m; g.sAk = 1;
        g.B = US.p; g.sBk = m; g.sBn = 1;
        g.C = tmp.p; g.sCm = m; g.sCn = 1;
        g.alpha = 1.0; g.beta = 0.0; g.nb1 = 1; g.nb0 = 1;
        CT_TRY(ct_gemm_f64_launch(h, g));
        // keep the running norm O(1): a long random chain's norm under- or overflows
        CT_TRY(ct_reduce_nrm2sq(h, Dp * d * m, tmp.p, h->d_scalars + SC_NORM, nullptr));
        CT_TRY(ct_scale_by_inv_sqrt(h, Dp * d * m, tmp.p, sites[i - 1], h->d_scalars + SC_NORM, nullptr,
                                    CT_ERR_ZERO_NORM));
    }
    const int64_t n0 = bd[0] * d * bd[1];
    CT_TRY(ct_reduce_nrm2sq(h, n0, sites[0], h->d_scalars + SC_NORM, nullptr));
    CT_TRY(ct_scale_by_inv_sqrt(h, n0, sites[0], sites[0], h->d_scalars + SC_NORM, nullptr, CT_ERR_ZERO_NORM));
    CT_CUDA(h, cudaStreamSynchronize(h->stream));
    int dst = 0;
    CT_CUDA(h, cudaMemcpy(&dst, h->d_status, sizeof(int), cudaMemcpyDeviceToHost));
    if (dst) {
        cudaMemset(h->d_status, 0, sizeof(int));
        return dst;
    }
    return CT_OK;
}

int ct_mps_expectation(ct_handle* h, int prec, int N, int d, const int64_t* mpo_dims, const double* const* mpo_sites,
                       const int64_t* bd, const double* const* sites, double* energy_host, double* norm_sq_host) {
    if (!h || !mpo_dims || !mpo_sites || !bd || !sites || N < 1 || d < 1) return CT_ERR_INVALID;
    if (prec != CT_PREC_FP64 && !((prec == CT_PREC_TF32X3 || prec == CT_PREC_FP64_TC) && ct_tc_available(h)))
        return CT_ERR_UNSUPPORTED;
    // CT_PREC_FP64_TC: FP64-accurate products on the BF16 tensor cores; TF32X3 as FP64
    const int eprec = (prec == CT_PREC_FP64_TC) ? CT_PREC_FP64_TC : CT_PREC_FP64;
    int64_t cap = 1;
    for (int k = 0; k <= N; ++k) cap = std::max<int64_t>(cap, std::max<int64_t>(mpo_dims[k], 1) * bd[k] * bd[k]);
    DevBuf e0, e1, Wid;
    CT_CUDA(h, cudaMalloc((void**)&e0.p, (size_t)cap * sizeof(double)));
    CT_CUDA(h, cudaMalloc((void**)&e1.p, (size_t)cap * sizeof(double)));
    CT_CUDA(h, cudaMalloc((void**)&Wid.p, (size_t)(d * d) * sizeof(double)));
    std::vector<double> idh((size_t)(d * d), 0.0);
    for (int s = 0; s < d; ++s) idh[(size_t)(s * d + s)] = 1.0;
    CT_CUDA(h, cudaMemcpyAsync(Wid.p, idh.data(), idh.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    double res[2] = {0.0, 0.0};
    for (int pass = 0; pass < 2; ++pass) {
        if (pass == 0 && !energy_host) continue;
        if (pass == 1 && !norm_sq_host) continue;
        double* a = e0.p;
        double* b = e1.p;
        const int64_t w0 = (pass == 0) ? mpo_dims[0] : 1;
        CT_TRY(ct_identity_env(h, a, w0, bd[0]));
        for (int i = 0; i < N; ++i) {
            const int64_t wl = (pass == 0) ? mpo_dims[i] : 1, wr = (pass == 0) ? mpo_dims[i + 1] : 1;
            CT_TRY(ct_reserve(h, ct_env_ws_bytes(CT_PREC_FP64, bd[i], d, bd[i + 1], wl, wr)));
            Arena ar(h);
            CT_TRY(ct_env_left_run(h, ar, eprec, a, sites[i], pass == 0 ? mpo_sites[i] : Wid.p, b, bd[i], d,
                                   bd[i + 1], wl, wr));
            std::swap(a, b);
        }
        // final env [w_N, D_N, D_N]: the reference reads element 0 (w=0, D=0)
        CT_CUDA(h, cudaMemcpyAsync(&res[pass], a, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        CT_CUDA(h, cudaStreamSynchronize(h->stream));
    }
    if (energy_host) *energy_host = res[0];
    if (norm_sq_host) *norm_sq_host = res[1];
    return CT_OK;
}

// <bra|mpo|ket> (expectation_value_two_mps, environments.mojo:698-730) or, with
// mpo_sites == NULL, <bra|ket> (mps_vdot_direct, environments.mojo:971-1016),
// through left environments L[w, D_ket, D_bra] in FP64.
int ct_mps_expectation2(ct_handle* h, int prec, int N, int d, const int64_t* mpo_dims,
                        const double* const* mpo_sites, const int64_t* bra_dims, const double* const* bra_sites,
                        const int64_t* ket_dims, const double* const* ket_sites, double* value_host) {
    if (!h || !bra_dims || !bra_sites || !ket_dims || !ket_sites || !value_host || N < 1 || d < 1)
        return CT_ERR_INVALID;
    if (mpo_sites && !mpo_dims) return CT_ERR_INVALID;
    if (prec != CT_PREC_FP64) {
        ct_seterr(h, "ct_mps_expectation2: only the FP64 form takes a bra different from the ket");
        return CT_ERR_UNSUPPORTED;
    }
    for (int k = 0; k <= N; ++k)
        if (bra_dims[k] < 1 || ket_dims[k] < 1 || (mpo_sites && mpo_dims[k] < 1)) return CT_ERR_SHAPE;
    if (mpo_sites && bra_dims[0] != ket_dims[0]) {
        ct_seterr(h, "ct_mps_expectation2: bra and ket left bonds differ");
        return CT_ERR_SHAPE;
    }
    int64_t cap = 1;
    for (int k = 0; k <= N; ++k)
        cap = std::max<int64_t>(cap, (mpo_sites ? mpo_dims[k] : 1) * bra_dims[k] * ket_dims[k]);
    DevBuf e0, e1;
    CT_CUDA(h, cudaMalloc((void**)&e0.p, (size_t)cap * sizeof(double)));
    CT_CUDA(h, cudaMalloc((void**)&e1.p, (size_t)cap * sizeof(double)));
    double* a = e0.p;
    double* b = e1.p;
    const int64_t w0 = mpo_sites ? mpo_dims[0] : 1;
    CT_TRY(ct_identity_env_rect(h, a, w0, ket_dims[0], bra_dims[0]));
    for (int i = 0; i < N; ++i) {
        const int64_t wl = mpo_sites ? mpo_dims[i] : 1, wr = mpo_sites ? mpo_dims[i + 1] : 1;
        CT_TRY(ct_reserve(h, ct_env2_ws_bytes(ket_dims[i], bra_dims[i], d, ket_dims[i + 1], bra_dims[i + 1], wl, wr)));
        Arena ar(h);
        CT_TRY(ct_env_left2_run(h, ar, a, ket_sites[i], bra_sites[i], mpo_sites ? mpo_sites[i] : nullptr, b,
                                ket_dims[i], bra_dims[i], d, ket_dims[i + 1], bra_dims[i + 1], wl, wr));
        std::swap(a, b);
    }
    if ((mpo_sites ? mpo_dims[N] : 1) * bra_dims[N] * ket_dims[N] != 1) {
        ct_seterr(h, "ct_mps_expectation2: final environment is not a scalar");
        return CT_ERR_SHAPE;
    }
    CT_CUDA(h, cudaMemcpyAsync(value_host, a, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CT_CUDA(h, cudaStreamSynchronize(h->stream));
    return CT_OK;
}

// ---------------------------------------------------------------------------
// seeded initial state: PCG32 (O'Neill) + Box-Muller in float32
// ---------------------------------------------------------------------------
}  // extern "C"

namespace {
struct Pcg {
    uint64_t state, inc;
    uint32_t next() {
        const uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        const uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        const uint32_t rot = (uint32_t)(old >> 59u);
        return (xs >> rot) | (xs << ((-rot) & 31u));
    }
};
Pcg pcg_seed(uint64_t initstate, uint64_t initseq) {
    Pcg g{0u, (initseq << 1u) | 1u};
    g.next();
    g.state += initstate;
    g.next();
    return g;
}
struct Rng2 {
    Pcg g0, g1;
    uint64_t u64() {
        const uint64_t a = g0.next();
        const uint64_t b = g1.next();
        return (a << 32) | b;
    }
    uint64_t bounded(uint64_t bound) {
        const uint64_t thr = (0 - bound) % bound;
        for (;;) {
            const uint64_t r = u64();
            if (r >= thr) return r % bound;
        }
    }
    void choice_advance(int64_t bound, int64_t nsamp) {
        for (int64_t i = 0; i < nsamp; ++i) bounded((uint64_t)(bound - nsamp + 1 + i));
    }
    float randnf() {
        const float inv = 2.32830644e-10f;
        float u1 = (float)g0.next() * inv;
        const float u2 = (float)g0.next() * inv;
        if (u1 == 0.0f) u1 = 1.0f;
        const float r = sqrtf(-2.0f * logf(u1));
        return r * sinf(6.2831853071795864769f * u2);
    }
};
Rng2 seed_state(uint64_t seed) {
    const uint64_t mult = 6364136223846793005ULL, inc = 1442695040888963407ULL;
    Pcg g = pcg_seed(seed, mult * seed + inc);
    uint32_t v[8];
    for (int i = 0; i < 8; ++i) v[i] = g.next();
    const uint64_t seed1 = ((uint64_t)v[0] << 32) | v[1];
    const uint64_t seed2 = ((uint64_t)v[2] << 32) | v[3];
    const uint64_t seq1 = ((uint64_t)v[4] << 32) | v[5];
    uint64_t seq2 = ((uint64_t)v[6] << 32) | v[7];
    const uint64_t mask = 0x7FFFFFFFFFFFFFFFULL;
    if ((seq1 & mask) == (seq2 & mask)) seq2 = ~seq2;
    return Rng2{pcg_seed(seed1, seq1), pcg_seed(seed2, seq2)};
}
}  // namespace

extern "C" {

int ct_rng_randnf_host(uint64_t seed, int64_t n, float* out) {
    if (!out || n < 0) return CT_ERR_INVALID;
    Rng2 r = seed_state(seed);
    for (int64_t i = 0; i < n; ++i) out[i] = r.randnf();
    return CT_OK;
}

int ct_random_mps_host(int N, int d, int chi_max, uint64_t seed, int64_t* dims, double* const* sites) {
    if (N < 1 || d < 1 || chi_max < 1 || !dims) return CT_ERR_INVALID;
    Rng2 rng = seed_state(seed);
    for (int i = 0; i <= N; ++i) dims[i] = 0;
    dims[0] = 1;
    dims[N] = 1;
    const int mid = (N + 1) / 2;
    for (int l = 1; l < mid; ++l) {
        const int64_t full = dims[l - 1] * d;
        dims[l] = std::min<int64_t>(full, chi_max);
        if (full > chi_max) rng.choice_advance(full, chi_max);
    }
    for (int l = N - 1; l >= mid; --l) {
        const int64_t full = dims[l + 1] * d;
        dims[l] = std::min<int64_t>(full, chi_max);
        if (full > chi_max) rng.choice_advance(full, chi_max);
    }
    if (!sites) return CT_OK;
    for (int i = 0; i < N; ++i) {
        const int64_t nel = dims[i] * d * dims[i + 1];
        const float scale = (float)(1.0 / sqrt((double)nel));
        double* s = sites[i];
        if (!s) return CT_ERR_INVALID;
        for (int64_t k = 0; k < nel; ++k) s[k] = (double)(rng.randnf() * scale);
    }
    return CT_OK;
}

}  // extern "C"

