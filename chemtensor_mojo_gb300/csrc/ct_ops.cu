// Contraction chains of the two-site DMRG path, built from the strided GEMM
// (ct_gemm_f64.cu), the MPO apply (ct_mpo.cu) and, for the mixed form, the
// tcgen05 GEMM (ct_tc.cu).  Layouts of the intermediates are chosen so that
// every permute of the reference chains becomes operand addressing:
//
//   H_eff (dmrg.mojo:254-374)
//     T1[Dl', wL, s1, s2, Dr] = sum_Dl L[wL,Dl,Dl'] th[Dl,(s1 s2 Dr)]      GEMM, batch wL
//     T3[Dl', t1, t2, wR, Dr] = sum_(wL s1 s2) W12[..] T1[Dl',(wL s1 s2),Dr] MPO apply
//     out[(Dl' t1 t2), Dr']   = sum_(wR Dr) T3[..,(wR Dr)] R[(wR Dr), Dr'] GEMM
//   left env (environments.mojo:99-201)
//     T1[Dl', wL, s, Dr] = sum_Dl L[wL,Dl,Dl'] A[Dl,(s Dr)]                GEMM, batch wL
//     T2[Dl', s', wR, Dr] = sum_(wL s) W[wL,s,s',wR] T1                    MPO apply
//     Ln[(wR Dr), Dr'] = sum_(Dl' s') T2[(Dl' s'),(wR Dr)] A[(Dl' s'),Dr'] GEMM
//   right env (environments.mojo:309-417)
//     T1[Dr', wR, s, Dl] = sum_Dr R[wR,Dr,Dr'] A[Dl,s,Dr]                  GEMM, batch (wR,s)
//     T2[wL, Dl, s', Dr'] = sum_(wR s) W[wL,s,s',wR] T1                    MPO apply
//     Rp[wL, Dl, Dl'] = sum_(s' Dr') T2[wL,Dl,(s' Dr')] A[Dl',(s' Dr')]    GEMM, batch wL
#include <stdlib.h>

#include "ct_ops.cuh"

size_t ct_heff_ws_bytes(int prec, int64_t Dl, int64_t d, int64_t Dr, int64_t wL, int64_t wM, int64_t wR) {
    (void)wM;
    if (prec == CT_PREC_TF32X3) return ct_tc_heff_ws_bytes(Dl, d, Dr, wL, wM, wR);
    const int64_t t1 = Dl * wL * d * d * Dr;
    const int64_t t3 = Dl * d * d * wR * Dr;
    const int64_t w12 = (d * d * wR) * (wL * d * d);
    return ct_bytes(t1, 8) + ct_bytes(t3, 8) + ct_bytes(w12, 8);
}

// Per-bond preparation (W12) is separated so that a Lanczos run builds it once.
int ct_heff_prepare(ct_handle* h, Arena& ar, HeffPlan& p, int prec, const double* L, const double* R,
                    const double* W1, const double* W2, int64_t Dl, int64_t d, int64_t Dr, int64_t wL,
                    int64_t wM, int64_t wR) {
    p.prec = prec;
    p.L = L; p.R = R; p.W1 = W1; p.W2 = W2;
    p.Dl = Dl; p.d = d; p.Dr = Dr; p.wL = wL; p.wM = wM; p.wR = wR;
    if (prec == CT_PREC_TF32X3) return ct_tc_heff_prepare(h, ar, p);
    p.T1 = ar.take<double>(Dl * wL * d * d * Dr);
    p.T3 = ar.take<double>(Dl * d * d * wR * Dr);
    p.W12 = ar.take<double>((d * d * wR) * (wL * d * d));
    if (!p.T1 || !p.T3 || !p.W12) return CT_ERR_OOM;
    return ct_build_w12(h, W1, W2, p.W12, wL, d, wM, wR);
}

int ct_heff_run(ct_handle* h, const HeffPlan& p, const double* theta, double* out, const int* skip) {
    if (p.prec == CT_PREC_TF32X3) return ct_tc_heff_run(h, p, theta, out, skip);
    const int64_t Dl = p.Dl, d = p.d, Dr = p.Dr, wL = p.wL, wR = p.wR;
    const int64_t n1 = d * d * Dr;
    {   // T1[Dl', wL, n1] = sum_Dl L[wL, Dl, Dl'] theta[Dl, n1]
        GemmDesc g{};
        g.M = Dl; g.N = n1; g.K = Dl;
        g.A = p.L; g.sAm = 1; g.sAk = Dl;
        g.B = theta; g.sBk = n1; g.sBn = 1;
        g.C = p.T1; g.sCm = wL * n1; g.sCn = 1;
        g.alpha = 1.0; g.beta = 0.0;
        g.nb1 = wL; g.nb0 = 1;
        g.sA1 = Dl * Dl; g.sB1 = 0; g.sC1 = n1;
        g.skip = skip;
        CT_TRY(ct_gemm_f64_launch(h, g));
    }
    {   // T3[Dl', (t1 t2 wR), Dr] = sum_k W12t[j, k] T1[Dl', k, Dr]
        MpoDesc m{};
        m.O = Dl; m.K = wL * d * d; m.J = d * d * wR; m.I = Dr;
        m.in = p.T1; m.sIo = wL * d * d * Dr; m.sIk = Dr; m.sIi = 1;
        m.out = p.T3; m.sOo = d * d * wR * Dr; m.sOi = 1; m.J0 = m.J; m.sOj1 = 0; m.sOj0 = Dr;
        m.Wt = p.W12; m.skip = skip;
        CT_TRY(ct_mpo_apply_f64_launch(h, m));
    }
    {   // out[(Dl' t1 t2), Dr'] = sum_(wR Dr) T3[.., (wR Dr)] R[(wR Dr), Dr']
        GemmDesc g{};
        g.M = Dl * d * d; g.N = Dr; g.K = wR * Dr;
        g.A = p.T3; g.sAm = wR * Dr; g.sAk = 1;
        g.B = p.R; g.sBk = Dr; g.sBn = 1;
        g.C = out; g.sCm = Dr; g.sCn = 1;
        g.alpha = 1.0; g.beta = 0.0; g.nb1 = 1; g.nb0 = 1;
        g.skip = skip;
        CT_TRY(ct_gemm_f64_launch(h, g));
    }
    return CT_OK;
}

size_t ct_env_ws_bytes(int prec, int64_t Dl, int64_t d, int64_t Dr, int64_t wL, int64_t wR) {
    if (prec == CT_PREC_TF32X3) return ct_tc_env_ws_bytes(Dl, d, Dr, wL, wR);
    const int64_t t1 = Dl * d * Dr * (wL > wR ? wL : wR);
    const int64_t wt = (wL * d) * (wR * d);
    return 2 * ct_bytes(t1, 8) + ct_bytes(wt, 8);
}

size_t ct_env2_ws_bytes(int64_t Dlk, int64_t Dlb, int64_t d, int64_t Drk, int64_t Drb, int64_t wL, int64_t wR) {
    (void)Dlk;
    (void)Drb;
    return ct_bytes(Dlb * wL * d * Drk, 8) + ct_bytes(Dlb * d * wR * Drk, 8) + ct_bytes((wL * d) * (wR * d), 8);
}

// Left environment with different bra and ket (environments.mojo:535-590), FP64:
//   Ln[wR, Drk, Drb] = sum L[wL, Dlk, Dlb] Ak[Dlk, s, Drk] W[wL, s, s', wR] Ab[Dlb, s', Drb]
// With W == null (wL = wR = 1) the MPO step drops out and this is the overlap
// transfer step L[Dlk, Dlb] -> L[Drk, Drb] of environments.mojo:767-862.
bool ct_fp64_tc_enabled(ct_handle* h, int64_t M, int64_t N, int64_t K) {
    static const int mode = [] {
        const char* e = getenv("CTDMRG_FP64_TC");
        return e ? atoi(e) : 1;
    }();
    return mode != 0 && !h->no_alloc && M * N * K >= ((int64_t)1 << 21) && ct_tc_available(h);
}

int ct_env_left2_run(ct_handle* h, Arena& ar, const double* Lp, const double* Ak, const double* Ab,
                     const double* W, double* Ln, int64_t Dlk, int64_t Dlb, int64_t d, int64_t Drk, int64_t Drb,
                     int64_t wL, int64_t wR, bool fp64_tc) {
    if (!W && (wL != 1 || wR != 1)) return CT_ERR_SHAPE;
    const int64_t n1 = d * Drk;
    double* T1 = ar.take<double>(Dlb * wL * n1);
    if (!T1) return CT_ERR_OOM;
    if (fp64_tc && ct_fp64_tc_enabled(h, wL * Dlb, n1, Dlk)) {
        // the same product as one GEMM over rows (wL, Dlb): A(r, k) = L[wL][k][Dlb],
        // B(n, k) = Ak[k][n], C row (wL, Dlb) at T1[Dlb][wL][.]
        const OzMat a{Lp, Dlb, Dlk * Dlb, 1, Dlb};
        const OzMat b{Ak, n1, 0, 1, n1};
        const OzOut c{T1, Dlb, n1, wL * n1};
        CT_TRY(ct_oz_gemm_ex(h, wL * Dlb, n1, Dlk, a, b, 1.0, 0.0, c));
    } else {   // T1[Dlb, wL, (s Drk)] = sum_Dlk L[wL, Dlk, Dlb] Ak[Dlk, (s Drk)]; batch wL
        GemmDesc g{};
        g.M = Dlb; g.N = n1; g.K = Dlk;
        g.A = Lp; g.sAm = 1; g.sAk = Dlb;
        g.B = Ak; g.sBk = n1; g.sBn = 1;
        g.C = T1; g.sCm = wL * n1; g.sCn = 1;
        g.alpha = 1.0; g.beta = 0.0; g.nb1 = wL; g.nb0 = 1;
        g.sA1 = Dlk * Dlb; g.sC1 = n1;
        CT_TRY(ct_gemm_f64_launch(h, g));
    }
    const double* T2 = T1;   // [(Dlb s'), (wR Drk)]
    if (W) {
        double* T2w = ar.take<double>(Dlb * d * wR * Drk);
        double* Wt = ar.take<double>((d * wR) * (wL * d));
        if (!T2w || !Wt) return CT_ERR_OOM;
        CT_TRY(ct_build_wt_left(h, W, Wt, wL, d, wR));
        MpoDesc m{};
        m.O = Dlb; m.K = wL * d; m.J = d * wR; m.I = Drk;
        m.in = T1; m.sIo = wL * d * Drk; m.sIk = Drk; m.sIi = 1;
        m.out = T2w; m.sOo = d * wR * Drk; m.sOi = 1; m.J0 = m.J; m.sOj1 = 0; m.sOj0 = Drk;
        m.Wt = Wt;
        CT_TRY(ct_mpo_apply_f64_launch(h, m));
        T2 = T2w;
    }
    if (fp64_tc && ct_fp64_tc_enabled(h, wR * Drk, Drb, Dlb * d)) {
        const int64_t M2 = wR * Drk;
        const OzMat a{T2, M2, 0, 1, M2};      // A(m, k) = T2[k][m]
        const OzMat b{Ab, Drb, 0, 1, Drb};    // B(n, k) = Ab[k][n]
        const OzOut c{Ln, M2, 0, Drb};
        CT_TRY(ct_oz_gemm_ex(h, M2, Drb, Dlb * d, a, b, 1.0, 0.0, c));
    } else {   // Ln[(wR Drk), Drb] = sum_(Dlb s') T2[(Dlb s'), (wR Drk)] Ab[(Dlb s'), Drb]
        GemmDesc g{};
        g.M = wR * Drk; g.N = Drb; g.K = Dlb * d;
        g.A = T2; g.sAm = 1; g.sAk = wR * Drk;
        g.B = Ab; g.sBk = Drb; g.sBn = 1;
        g.C = Ln; g.sCm = Drb; g.sCn = 1;
        g.alpha = 1.0; g.beta = 0.0; g.nb1 = 1; g.nb0 = 1;
        CT_TRY(ct_gemm_f64_launch(h, g));
    }
    return CT_OK;
}

int ct_env_left_run(ct_handle* h, Arena& ar, int prec, const double* Lp, const double* A, const double* W,
                    double* Ln, int64_t Dl, int64_t d, int64_t Dr, int64_t wL, int64_t wR) {
    if (prec == CT_PREC_TF32X3) return ct_tc_env_left_run(h, ar, Lp, A, W, Ln, Dl, d, Dr, wL, wR);
    return ct_env_left2_run(h, ar, Lp, A, A, W, Ln, Dl, Dl, d, Dr, Dr, wL, wR, prec == CT_PREC_FP64_TC);
}

int ct_env_right_run(ct_handle* h, Arena& ar, int prec, const double* Rn, const double* A, const double* W,
                     double* Rp, int64_t Dl, int64_t d, int64_t Dr, int64_t wL, int64_t wR) {
    if (prec == CT_PREC_TF32X3) return ct_tc_env_right_run(h, ar, Rn, A, W, Rp, Dl, d, Dr, wL, wR);
    double* T1 = ar.take<double>(Dr * wR * d * Dl);
    double* T2 = ar.take<double>(wL * Dl * d * Dr);
    double* Wt = ar.take<double>((wL * d) * (wR * d));
    if (!T1 || !T2 || !Wt) return CT_ERR_OOM;
    CT_TRY(ct_build_wt_right(h, W, Wt, wL, d, wR));
    {   // T1[Dr', wR, s, Dl] = sum_Dr R[wR, Dr, Dr'] A[Dl, s, Dr]; batch (wR, s)
        GemmDesc g{};
        g.M = Dr; g.N = Dl; g.K = Dr;
        g.A = Rn; g.sAm = 1; g.sAk = Dr;
        g.B = A; g.sBk = 1; g.sBn = d * Dr;
        g.C = T1; g.sCm = wR * d * Dl; g.sCn = 1;
        g.alpha = 1.0; g.beta = 0.0;
        g.nb1 = wR; g.nb0 = d;
        g.sA1 = Dr * Dr; g.sA0 = 0;
        g.sB1 = 0; g.sB0 = Dr;
        g.sC1 = d * Dl; g.sC0 = Dl;
        CT_TRY(ct_gemm_f64_launch(h, g));
    }
    {   // T2[wL, Dl, s', Dr'] = sum_(wR s) Wt[(wL s'), (wR s)] T1[Dr', (wR s), Dl]
        MpoDesc m{};
        m.O = Dr; m.K = wR * d; m.J = wL * d; m.I = Dl;
        m.in = T1; m.sIo = wR * d * Dl; m.sIk = Dl; m.sIi = 1;
        m.out = T2; m.sOo = 1; m.sOi = d * Dr; m.J0 = d; m.sOj1 = Dl * d * Dr; m.sOj0 = Dr;
        m.Wt = Wt;
        CT_TRY(ct_mpo_apply_f64_launch(h, m));
    }
    {   // Rp[wL, Dl, Dl'] = sum_(s' Dr') T2[wL, Dl, (s' Dr')] A[Dl', (s' Dr')]; batch wL
        GemmDesc g{};
        g.M = Dl; g.N = Dl; g.K = d * Dr;
        g.A = T2; g.sAm = d * Dr; g.sAk = 1;
        g.B = A; g.sBk = 1; g.sBn = d * Dr;
        g.C = Rp; g.sCm = Dl; g.sCn = 1;
        g.alpha = 1.0; g.beta = 0.0; g.nb1 = wL; g.nb0 = 1;
        g.sA1 = Dl * d * Dr; g.sC1 = Dl * Dl;
        CT_TRY(ct_gemm_f64_launch(h, g));
    }
    return CT_OK;
}

size_t ct_theta_ws_bytes(int prec, int64_t Dl, int64_t d, int64_t Dm, int64_t Dr) {
    return prec == CT_PREC_TF32X3 ? ct_tc_gemm_ws_bytes(Dl * d, d * Dr, Dm) : 0;
}

// theta = A_i . A_{i+1}.  In the mixed form the product runs on the tensor
// cores: theta is only the Lanczos start vector, and an FP64 GEMM of this size
// (8.6 GFLOP at chi = 1024) costs ~7 ms at this part's FP64 rate.  The
// workspace must hold ct_theta_ws_bytes (the caller reserves it).
int ct_theta_run(ct_handle* h, int prec, const double* Ai, const double* Aj, double* theta, int64_t Dl,
                 int64_t d, int64_t Dm, int64_t Dr) {
    if (prec == CT_PREC_TF32X3 && ct_tc_available(h)) {
        Arena ar(h);
        return ct_tc_gemm(h, ar, 0, 0, Dl * d, d * Dr, Dm, 1.0, Ai, Dm, Aj, d * Dr, 0.0, theta, d * Dr);
    }
    GemmDesc g{};
    g.M = Dl * d; g.N = d * Dr; g.K = Dm;
    g.A = Ai; g.sAm = Dm; g.sAk = 1;
    g.B = Aj; g.sBk = d * Dr; g.sBn = 1;
    g.C = theta; g.sCm = d * Dr; g.sCn = 1;
    g.alpha = 1.0; g.beta = 0.0; g.nb1 = 1; g.nb0 = 1;
    return ct_gemm_f64_launch(h, g);
}

// ---------------------------------------------------------------------------
// Lanczos (dmrg.mojo:486-756), everything device resident
// ---------------------------------------------------------------------------
size_t ct_lanczos_ws_bytes(int prec, int64_t Dl, int64_t d, int64_t Dr, int64_t wL, int64_t wM, int64_t wR,
                           int max_iter) {
    const int64_t N = Dl * d * d * Dr;
    // (the mixed form also keeps an FP32 copy of the basis for the reorthogonalisation)
    return ct_bytes(N * (int64_t)max_iter, 8) + ct_bytes(N, 8) + ct_heff_ws_bytes(prec, Dl, d, Dr, wL, wM, wR) +
           (prec == CT_PREC_TF32X3 ? ct_bytes(N * (int64_t)max_iter, 4) : 0);
}

// Second FP32 reorthogonalisation pass in place of most FP64 passes (CTDMRG_LANCZOS_REDO32=0
// restores the FP64 pass after every FP32 pass that removed more than 0.1 beta); read on
// every Lanczos run so that a test can compare both in one process.
static bool ct_lanczos_redo32() {
    const char* e = getenv("CTDMRG_LANCZOS_REDO32");
    return !(e && e[0] == '0');
}

int ct_lanczos_run(ct_handle* h, Arena& ar, int prec, const double* theta_in, double* theta_out, const double* L,
                   const double* R, const double* W1, const double* W2, int64_t Dl, int64_t d, int64_t Dr,
                   int64_t wL, int64_t wM, int64_t wR, int max_iter, double tol, int max_rotations, int reorth,
                   LanczosResult* res) {
    if (max_iter < 1 || max_iter > 64) {
        ct_seterr(h, "max_krylov_iter must be in [1, 64], got %d", max_iter);
        return CT_ERR_UNSUPPORTED;
    }
    const int64_t N = Dl * d * d * Dr;
    double* V = ar.take<double>(N * (int64_t)max_iter);
    double* w = ar.take<double>(N);
    if (!V || !w) return CT_ERR_OOM;
    // mixed form: FP32 copy of the basis for the reorthogonalisation pass (CTDMRG_LANCZOS_FP32=0: FP64 basis)
    static const bool fp32_basis = [] {
        const char* e = getenv("CTDMRG_LANCZOS_FP32");
        return !(e && e[0] == '0');
    }();
    float* V32 = nullptr;
    if (reorth && prec == CT_PREC_TF32X3 && fp32_basis) {
        V32 = ar.take<float>(N * (int64_t)max_iter);
        if (!V32) return CT_ERR_OOM;
    }
    HeffPlan plan;
    CT_TRY(ct_heff_prepare(h, ar, plan, prec, L, R, W1, W2, Dl, d, Dr, wL, wM, wR));
    const int* stop = h->d_flags + FL_STOP;
    CT_TRY(ct_lanczos_init(h, max_iter));
    // v0 = theta / |theta|  (zero norm -> CT_ERR_ZERO_NORM, dmrg.mojo:605-611; a NaN
    // or infinite norm -> CT_ERR_NONFINITE, where the reference would carry NaN on)
    CT_TRY(ct_reduce_nrm2sq(h, N, theta_in, h->d_scalars + SC_NORM, nullptr));
    CT_TRY(ct_check_finite(h, h->d_scalars + SC_NORM, nullptr));
    CT_TRY(ct_scale_by_inv_sqrt(h, N, theta_in, V, h->d_scalars + SC_NORM, nullptr, CT_ERR_ZERO_NORM));
    if (V32) CT_TRY(ct_f64_to_f32(h, N, V, V32, nullptr));
    const double thr = 100.0 * (double)N * 2.2204460492503131e-16;
    // algorithmic FLOPs of one apply (the reference's four contractions)
    const double heff_flops = 2.0 * (double)Dl * wL * d * d * Dr * Dl + 2.0 * (double)Dl * d * Dr * wL * d * d * wM +
                              2.0 * (double)Dl * Dr * d * wM * d * d * wR + 2.0 * (double)Dl * d * d * Dr * wR * Dr;
    for (int j = 0; j < max_iter - 1; ++j) {
        double* vj = V + (int64_t)j * N;
        const double* vjm1 = (j > 0) ? V + (int64_t)(j - 1) * N : nullptr;
        int ks = -1;
        CT_TRY(ct_ktime_begin(h, KT_HEFF_APPLY, heff_flops, &ks));
        CT_TRY(ct_heff_run(h, plan, vj, w, stop));
        CT_TRY(ct_ktime_end(h, ks));
        if (reorth) {
            // the reference recurrence, then one Gram-Schmidt pass against the whole
            // Krylov basis (ct_lanczos_reorth_pass), then v_{j+1} = w / beta_j.
            // Algorithmic bytes of the vector work: alpha reads v_j and w, the
            // recurrence reads w, v_j, v_{j-1} and writes w, the pass reads w and j + 1
            // vectors twice and writes w, the next vector reads w and writes v_{j+1}.
            // With the FP32 copy (mixed form) the pass reads 4-byte basis vectors and the
            // next-vector kernel also writes the copy.
            const double nb = (double)(j + 1);
            const double bytes = V32 ? (double)N * (8.0 * (2 + (j > 0 ? 4 : 3)) + (8.0 + 4.0 * nb) +
                                                    (16.0 + 4.0 * nb) + 20.0)
                                     : 8.0 * (double)N * (double)(2 + (j > 0 ? 4 : 3) + (j + 2) + (j + 3) + 2);
            int kv = -1;
            CT_TRY(ct_ktime_begin(h, KT_LANCZOS_VEC, bytes, &kv));
            CT_TRY(ct_lanczos_alpha(h, N, vj, w, j, stop));
            CT_TRY(ct_lanczos_update_nonorm(h, N, w, vj, vjm1, j, stop));
            if (V32) {
                // the FP32 pass, then a second pass gated on the device: against the FP32 copy
                // when the first removed more than 0.1 beta, against the FP64 basis above 1e4 beta
                // (CTDMRG_LANCZOS_REDO32=0: the FP64 basis whenever above 0.1 beta)
                CT_TRY(ct_lanczos_reorth_pass32(h, N, w, V32, N, j, thr, stop, ct_lanczos_redo32() ? 1e4 : 0.1));
                CT_TRY(ct_lanczos_reorth_redo(h, N, w, V, V32, N, j, thr, stop));
                CT_TRY(ct_lanczos_next32(h, N, w, V + (int64_t)(j + 1) * N, V32 + (int64_t)(j + 1) * N, j, stop));
            } else {
                CT_TRY(ct_lanczos_reorth_pass(h, N, w, V, N, j, thr, stop));
                CT_TRY(ct_lanczos_next(h, N, w, V + (int64_t)(j + 1) * N, j, stop));
            }
            CT_TRY(ct_ktime_end(h, kv));
            continue;
        }
        // the reference's recurrence (dmrg.mojo:612-689): alpha, w -= alpha v_j + beta v_{j-1},
        // beta = |w|, v_{j+1} = w / beta
        CT_TRY(ct_lanczos_alpha(h, N, vj, w, j, stop));
        CT_TRY(ct_lanczos_update(h, N, w, vj, vjm1, j, thr, stop));
        CT_TRY(ct_lanczos_next(h, N, w, V + (int64_t)(j + 1) * N, j, stop));
    }
    {   // final alpha-only iteration, only when no breakdown (dmrg.mojo:691-703)
        const int j = max_iter - 1;
        double* vj = V + (int64_t)j * N;
        int ks = -1;
        CT_TRY(ct_ktime_begin(h, KT_HEFF_APPLY, heff_flops, &ks));
        CT_TRY(ct_heff_run(h, plan, vj, w, stop));
        CT_TRY(ct_ktime_end(h, ks));
        CT_TRY(ct_lanczos_alpha(h, N, vj, w, j, stop));
    }
    CT_TRY(ct_tridiag_eig(h, max_iter, tol, max_rotations));
    // non-finite environments or MPO tensors surface here, in the eigenvalue
    CT_TRY(ct_check_finite(h, h->d_scalars + SC_ENERGY, nullptr));
    CT_TRY(ct_ritz(h, N, V, N, w));
    CT_TRY(ct_reduce_nrm2sq(h, N, w, h->d_scalars + SC_NORM, nullptr));
    CT_TRY(ct_scale_by_inv_sqrt(h, N, w, theta_out, h->d_scalars + SC_NORM, nullptr, 0));
    if (res) {
        res->d_energy = h->d_scalars + SC_ENERGY;
        res->d_numiter = h->d_flags + FL_NUMITER;
        res->applies_upper = max_iter;
    }
    return CT_OK;
}
