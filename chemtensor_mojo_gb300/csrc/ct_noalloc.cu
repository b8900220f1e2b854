// H_eff apply that allocates nothing.
//
// Some callers cannot let a library allocate device memory: a Mojo/MAX host
// whose DeviceContext allocator owns every device buffer, or a caller running
// under a fixed device-memory budget that has handed all of it out already.
// ct_heff2_apply_noalloc gives them the FP64 H_eff apply (the same kernels as
// ct_heff2_apply) with its intermediates (T1, T3 and the fused MPO matrix) in
// a file-scope __device__ array of CT_NOALLOC_SCRATCH_DOUBLES doubles that every
// GPU which loads the library holds until the process exits.
//
// Set-up: the first call on a device looks up the array's device address with
// cudaGetSymbolAddress while that device is current (host code cannot use the
// symbol itself as a device pointer).  Make that first call before any stream
// capture.  All calls share the one array, so calls whose kernels overlap on
// the GPU race on it.  Every element a call reads is written earlier in the
// same call (the split-K partial sums included: each K piece writes its whole
// M x N slice before the reduction reads it), so no part of the array needs
// clearing between calls.  No allocation happens anywhere on this path: the
// handle below is flagged no-alloc, so the FP64 GEMM launcher takes its split-K
// scratch from the array instead of growing a handle-owned buffer.
#include <mutex>

#include "ct_ops.cuh"

static __device__ __align__(256) double g_heff_scratch[CT_NOALLOC_SCRATCH_DOUBLES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
double* g_scratch_ptr[kMaxDevices] = {};

int64_t round_up_256b(int64_t n) { return (n + 31) / 32 * 32; }   // doubles, 256-byte pieces

}  // namespace

extern "C" int ct_heff2_apply_noalloc(void* stream, const double* theta, const double* L, const double* R,
                                      const double* W1, const double* W2, double* out, int64_t Dl, int64_t d,
                                      int64_t Dr, int64_t wL, int64_t wM, int64_t wR) {
    if (!theta || !L || !R || !W1 || !W2 || !out) return CT_ERR_INVALID;
    if (Dl <= 0 || d <= 0 || Dr <= 0 || wL <= 0 || wM <= 0 || wR <= 0) return CT_ERR_SHAPE;
    const int64_t n_t1 = round_up_256b(Dl * wL * d * d * Dr);
    const int64_t n_t3 = round_up_256b(Dl * d * d * wR * Dr);
    const int64_t n_w12 = round_up_256b((d * d * wR) * (wL * d * d));
    if (n_t1 + n_t3 + n_w12 > (int64_t)CT_NOALLOC_SCRATCH_DOUBLES) return CT_ERR_TOO_LARGE;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        (void)cudaGetLastError();
        return CT_ERR_CUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) return CT_ERR_UNSUPPORTED;
    double* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_scratch_mu);
        if (!g_scratch_ptr[dev]) {
            void* p = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&p, g_heff_scratch);
            if (e != cudaSuccess || p == nullptr) {
                (void)cudaGetLastError();
                return CT_ERR_CUDA;
            }
            g_scratch_ptr[dev] = static_cast<double*>(p);
        }
        base = g_scratch_ptr[dev];
    }
    // a handle on the stack: it carries the stream and the SM count, owns nothing,
    // and its no-alloc mode keeps the GEMM launcher away from cudaMalloc: the FP64
    // GEMM's split-K partial sums go to the part of the array past W12, and K is
    // split only as far as that part holds (not at all when it is too small)
    ct_handle h;
    h.device = dev;
    h.stream = static_cast<cudaStream_t>(stream);
    h.no_alloc = true;
    h.splitk_fixed = base + n_t1 + n_t3 + n_w12;
    h.splitk_fixed_cap = (size_t)((int64_t)CT_NOALLOC_SCRATCH_DOUBLES - (n_t1 + n_t3 + n_w12));
    if (cudaDeviceGetAttribute(&h.num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        (void)cudaGetLastError();
        return CT_ERR_CUDA;
    }
    HeffPlan p;
    p.prec = CT_PREC_FP64;
    p.L = L; p.R = R; p.W1 = W1; p.W2 = W2;
    p.Dl = Dl; p.d = d; p.Dr = Dr; p.wL = wL; p.wM = wM; p.wR = wR;
    p.T1 = base;
    p.T3 = base + n_t1;
    p.W12 = base + n_t1 + n_t3;
    CT_TRY(ct_build_w12(&h, W1, W2, p.W12, wL, d, wM, wR));
    return ct_heff_run(&h, p, theta, out, nullptr);
}
