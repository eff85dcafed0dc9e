// Objective of caller-owned device buffers, computed without allocating any device
// memory: the per-sequence partial sums live in a file-scope __device__ array.
//
// Who needs it: a caller that owns its device memory through its own allocator and
// must not have a library call cudaMalloc behind it -- e.g. a Julia process whose
// CUDA.jl memory pool holds (almost) all free device memory, so that a foreign
// cudaMalloc fails or forces the pool to release and re-grow, or a serving loop
// that has pinned its memory budget and treats any new allocation as a fault.
// Such a caller passes its own X, DX and S (device pointers) and gets the value of
// objective(c, S) (src/SETUP/CDL_setup.jl:286) back in host memory.
//
// Limits and sharing:
//   * N <= CDLGB_NOALLOC_MAX_SEQ (65536) sequences: the scratch holds two float64
//     partial sums per sequence (1 MiB per device, held by every device that loads
//     the library until the process exits).  Larger N is rejected with
//     CDLGB_EINVAL before any GPU work.
//   * The scratch is shared by every call in the process: calls that overlap on
//     the GPU (different streams, or different host threads on one device) race on
//     it and must be serialised by the caller.
//   * The first call on a device looks up the scratch's device address
//     (cudaGetSymbolAddress) with that device current and caches it; that first
//     call should come before any stream capture.  cdlgb_create does the same
//     lookup for its device, as a warm-up.
//   * With CUDA's lazy module loading (the default since CUDA 12.2) the driver
//     loads this module, and backs the 1 MiB array, only at that lookup.  A caller
//     whose pool later takes (almost) all free memory must therefore make the
//     first call, or create a context, on each device before the pool grows, or
//     set CUDA_MODULE_LOADING=EAGER; otherwise that first lookup can fail for lack
//     of memory (reported as CDLGB_ECUDA, nothing else is affected).
#include "cdlgb_internal.h"

#include <mutex>

#define CDLGB_NOALLOC_MAX_SEQ 65536

namespace {

constexpr int kMaxDevices = 64;
constexpr int kThreads = 256;

// [0, 2N): per-sequence (sum |X|, sum over the data window of (DX - S)^2);
// [2*MAX, 2*MAX+1): the objective.  Every call rewrites the slots it reads.
__device__ __align__(256) double g_noalloc_scratch[2 * CDLGB_NOALLOC_MAX_SEQ + 8];

double* g_scratch_addr[kMaxDevices];
std::mutex g_scratch_mu;

__device__ __forceinline__ double block_sum(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double t = 0.0;
    if (w == 0) {
        t = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    __syncthreads();
    return t;
}

// one block per sequence n: sum |X[n,:,:]| and sum_j (DX[n, gamma+j] - S[n, j])^2
__global__ void k_obj_per_seq(const float* __restrict__ X, const float* __restrict__ DX,
                              const float* __restrict__ S, int L4, int Lg, int M, int gamma,
                              double* __restrict__ part) {
    __shared__ double sh[32];
    const size_t n = blockIdx.x;
    const size_t cols = (size_t)M * Lg;
    const float* x = X + n * cols;
    double a = 0.0;
    for (size_t i = threadIdx.x; i < cols; i += blockDim.x) a += (double)fabsf(x[i]);
    double r = 0.0;
    for (int j = threadIdx.x; j < L4; j += blockDim.x) {
        const double d = (double)DX[n * Lg + gamma + j] - (double)S[n * L4 + j];
        r += d * d;
    }
    a = block_sum(a, sh);
    r = block_sum(r, sh);
    if (threadIdx.x == 0) {
        part[2 * n] = a;
        part[2 * n + 1] = r;
    }
}

// sums the N per-sequence partials in a fixed order: 0.5 * fit + lambda * |X|_1
__global__ void k_obj_total(const double* __restrict__ part, int N, double lam,
                            double* __restrict__ out) {
    __shared__ double sh[32];
    double a = 0.0, r = 0.0;
    for (int n = threadIdx.x; n < N; n += blockDim.x) {
        a += part[2 * n];
        r += part[2 * n + 1];
    }
    a = block_sum(a, sh);
    r = block_sum(r, sh);
    if (threadIdx.x == 0) out[0] = 0.5 * r + lam * a;
}

// device address of the scratch on the current device, looked up once per device
cudaError_t scratch_for_current_device(double** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        if (!p) return cudaErrorInvalidSymbol;
        g_scratch_addr[dev] = (double*)p;
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

}  // namespace

// Warm-up for cdlgb_create: the scratch address of the current device, looked up
// (and the module loaded) while the caller's memory is still free.
int noalloc_warm_current_device() {
    double* p = nullptr;
    return scratch_for_current_device(&p) == cudaSuccess ? CDLGB_OK : CDLGB_ECUDA;
}

extern "C" int cdlgb_objective_noalloc(const float* X, const float* DX, const float* S,
                                       int32_t L4, int32_t N, int32_t M, int32_t gamma,
                                       float lambda, double* obj, void* stream) {
    if (!X || !DX || !S || !obj || L4 <= 0 || N <= 0 || M <= 0 || gamma < 0 || (L4 % 4))
        return noctx_seterr(CDLGB_EINVAL, "cdlgb_objective_noalloc: invalid argument");
    if (N > CDLGB_NOALLOC_MAX_SEQ)
        return noctx_seterr(CDLGB_EINVAL,
                            "cdlgb_objective_noalloc: N=%d sequences exceeds the fixed scratch of %d "
                            "sequences; use cdlgb_objective on a context instead",
                            N, CDLGB_NOALLOC_MAX_SEQ);
    double* scratch = nullptr;
    cudaError_t se = scratch_for_current_device(&scratch);
    if (se != cudaSuccess)
        return noctx_seterr(CDLGB_ECUDA, "cdlgb_objective_noalloc: scratch lookup: %s",
                            cudaGetErrorString(se));
    cudaStream_t s = (cudaStream_t)stream;
    const int Lg = L4 + 2 * gamma;
    k_obj_per_seq<<<N, kThreads, 0, s>>>(X, DX, S, L4, Lg, M, gamma, scratch);
    double* res = scratch + 2 * CDLGB_NOALLOC_MAX_SEQ;
    k_obj_total<<<1, kThreads, 0, s>>>(scratch, N, (double)lambda, res);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(obj, res, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess)
        return noctx_seterr(CDLGB_ECUDA, "cdlgb_objective_noalloc: %s", cudaGetErrorString(e));
    return CDLGB_OK;
}
