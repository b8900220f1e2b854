// Mixed-precision (TF32x3) tensor-core path: placeholder until the tcgen05
// kernels land; every entry reports CT_ERR_UNSUPPORTED.
#include "ct_ops.cuh"

int ct_tc_available(ct_handle* h) { (void)h; return 0; }
size_t ct_tc_heff_ws_bytes(int64_t, int64_t, int64_t, int64_t, int64_t, int64_t) { return 0; }
int ct_tc_heff_prepare(ct_handle*, Arena&, HeffPlan&) { return CT_ERR_UNSUPPORTED; }
int ct_tc_heff_run(ct_handle*, const HeffPlan&, const double*, double*, const int*) { return CT_ERR_UNSUPPORTED; }
size_t ct_tc_env_ws_bytes(int64_t, int64_t, int64_t, int64_t, int64_t) { return 0; }
int ct_tc_env_left_run(ct_handle*, Arena&, const double*, const double*, const double*, double*, int64_t, int64_t,
                       int64_t, int64_t, int64_t) { return CT_ERR_UNSUPPORTED; }
int ct_tc_env_right_run(ct_handle*, Arena&, const double*, const double*, const double*, double*, int64_t, int64_t,
                        int64_t, int64_t, int64_t) { return CT_ERR_UNSUPPORTED; }
int ct_tc_gemm(ct_handle*, Arena&, int, int, int64_t, int64_t, int64_t, double, const double*, int64_t,
               const double*, int64_t, double, double*, int64_t) { return CT_ERR_UNSUPPORTED; }
size_t ct_tc_gemm_ws_bytes(int64_t, int64_t, int64_t) { return 0; }
