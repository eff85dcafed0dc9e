// Reference-structured CUDA baseline: the reference's CDL ADMM (CUDA.jl path) restated
// statement by statement in CUDA C++, to stand in for the reference GPU path, which
// cannot run here (Julia is absent; CUDA.jl 3.9 cannot target sm_103 / CUDA 13).
// This is a measurement comparator, not part of the product: it keeps the reference's
// decomposition and its costs --
//   * full-spectrum complex FFTs of real arrays promoted to complex (cuFFT C2C, the
//     plans of src/SETUP/CDL_setup.jl:195-204), an allocation per transform result,
//     the inverse scaled by a separate pass and `real.` by another;
//   * one kernel per Julia broadcast statement (CUDA.jl fuses each statement);
//   * the custom kernels with the reference's launch shapes, 10x10x10 threads for 3-D
//     and 32x32 for 2-D (src/SETUP/GPU_setup.jl:2-11), each followed by a stream sync
//     (CUDA.@sync);
//   * the per-iteration allocations of RHS_csc / alpha_csc (src/CDL/train.jl:21-22) and
//     of every re-assigned array (stream-ordered pool, as CUDA.jl's pool allocator);
//   * the dense W*DX product (train.jl:28), whose result is unused.
// Statement order follows src/CDL/train.jl:1-98 (code_update!, dict_update!,
// update_best!) and src/WRAPPER/wrap.jl:6-11 (the outer loop).
// Layout: Julia's column-major (Lg, M, N) == C-order (N, M, Lg).
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <cufft.h>

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <vector>

namespace {

typedef float2 cplx;

struct RS {
    int N, M, Lg, L4, gamma, flen;
    float rho, sigma, lam, kcsc, kcdl;
    cudaStream_t s;
    cublasHandle_t blas;
    cufftHandle pLMN, pLN, pLM;
    // real (N, M, Lg)
    float *X, *Y2, *Y3, *y2, *y3, *d, *g1, *g3, *X_best;
    // real (N, Lg)
    float *DX, *Y1, *y1, *Td, *G2, *g2, *WtS, *WDX;
    // real (M, Lg), (Lg, Lg), (Lg, 4L), (N, 4L)
    float *G1, *G3, *P_D, *D_best, *WtW, *W, *dat;
    // complex
    cplx *Xh, *Y2h, *y2h, *Y3h, *y3h, *dh, *g1h, *g3h;          // (N, M, Lg)
    cplx *RHS_csc, *dots_cdl, *X_cdl, *RHS_cdl;
    cplx *Y1h, *y1h, *G2h, *g2h, *alpha_csc, *ifft_elem_mult, *beta_cdl;   // (N, Lg)
    cplx *G1h, *G3h, *dots_csc, *A_csc;                           // (M, Lg)
    cplx *sum_dots_csc;                                           // (Lg)
    cplx *sum_dots_cdl;                                           // (N, Lg)
    float *v_avg_1, *v_avg_2;                                     // (M, Lg)
    double obj_best;
    char err[256];
};

#define RS_TRY(x)                                                                       \
    do {                                                                                \
        cudaError_t e_ = (x);                                                           \
        if (e_ != cudaSuccess) {                                                        \
            snprintf(r->err, sizeof r->err, "%s: %s", #x, cudaGetErrorString(e_));      \
            return -1;                                                                  \
        }                                                                               \
    } while (0)
#define FFT_TRY(x)                                                                      \
    do {                                                                                \
        cufftResult e_ = (x);                                                           \
        if (e_ != CUFFT_SUCCESS) {                                                      \
            snprintf(r->err, sizeof r->err, "%s: cufft %d", #x, (int)e_);              \
            return -1;                                                                  \
        }                                                                               \
    } while (0)

__device__ __forceinline__ cplx cmul(cplx a, cplx b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ cplx conjf2(cplx a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ cplx csub(cplx a, cplx b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ cplx cadd(cplx a, cplx b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ cplx cdiv(cplx a, cplx b) {
    float den = b.x * b.x + b.y * b.y;
    return make_float2((a.x * b.x + a.y * b.y) / den, (a.y * b.x - a.x * b.y) / den);
}

#define GRID_STRIDE(i, n) for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (n); i += (size_t)gridDim.x * blockDim.x)

// ---- broadcasts (one kernel per Julia statement)
__global__ void b_promote(const float* a, cplx* o, size_t n) { GRID_STRIDE(i, n) o[i] = make_float2(a[i], 0.f); }
__global__ void b_scale(cplx* a, float s, size_t n) { GRID_STRIDE(i, n) a[i] = make_float2(a[i].x * s, a[i].y * s); }
__global__ void b_real(const cplx* a, float* o, size_t n) { GRID_STRIDE(i, n) o[i] = a[i].x; }
__global__ void b_dual(float* y, const float* a, const float* b, size_t n) { GRID_STRIDE(i, n) y[i] = y[i] + a[i] - b[i]; }
// o = a + b - C broadcast over n (C has period per)
__global__ void b_dual_bc(const float* a, const float* b, const float* C, float* o, size_t n, size_t per) {
    GRID_STRIDE(i, n) o[i] = a[i] + b[i] - C[i % per];
}
__global__ void b_abs2(const cplx* a, cplx* o, size_t n) { GRID_STRIDE(i, n) o[i] = cmul(a[i], conjf2(a[i])); }
__global__ void b_addc(const cplx* a, cplx* o, float k, size_t n) { GRID_STRIDE(i, n) o[i] = make_float2(a[i].x + k, a[i].y); }
// o[i] = a[i] / b[i % ... per the broadcast of (Lg) over M, or (Lg,1,N) over M]
__global__ void b_div_csc(const cplx* a, const cplx* b, cplx* o, size_t n, int Lg) {
    GRID_STRIDE(i, n) o[i] = cdiv(a[i], b[i % Lg]);
}
__global__ void b_div_cdl(const cplx* a, const cplx* b, cplx* o, size_t n, int Lg, int M) {
    GRID_STRIDE(i, n) {
        size_t l = i % Lg, nn = i / ((size_t)Lg * M);
        o[i] = cdiv(a[i], b[nn * Lg + l]);
    }
}
// o = A .* B with A (M, Lg) broadcast over N
__global__ void b_mul_bcast(const cplx* A, const cplx* B, cplx* o, size_t n, size_t per) {
    GRID_STRIDE(i, n) o[i] = cmul(A[i % per], B[i]);
}
__global__ void b_mul(const cplx* A, const cplx* B, cplx* o, size_t n) { GRID_STRIDE(i, n) o[i] = cmul(A[i], B[i]); }
__global__ void b_add_real(const float* a, const float* b, float* o, size_t n) { GRID_STRIDE(i, n) o[i] = a[i] + b[i]; }
__global__ void b_divN(const float* a, float* o, float N, size_t n) { GRID_STRIDE(i, n) o[i] = a[i] / N; }
__global__ void b_sub_real(const float* a, const float* b, float* o, size_t n) { GRID_STRIDE(i, n) o[i] = a[i] - b[i]; }
__global__ void b_abs(const float* a, float* o, size_t n) { GRID_STRIDE(i, n) o[i] = fabsf(a[i]); }

// ---- reductions (mapreducedim: one output element per thread)
// sum over the middle dimension of (outer, M, Lg) -> (outer, Lg)
__global__ void r_sum_m_c(const cplx* a, cplx* o, int M, int Lg, size_t outer) {
    GRID_STRIDE(i, outer * Lg) {
        size_t nn = i / Lg, l = i % Lg;
        cplx s = make_float2(0.f, 0.f);
        for (int m = 0; m < M; ++m) s = cadd(s, a[(nn * M + m) * Lg + l]);
        o[i] = s;
    }
}
// sum over the outer dimension of (N, ML) -> (ML)
__global__ void r_sum_n(const float* a, float* o, int N, size_t ML) {
    GRID_STRIDE(i, ML) {
        float s = 0.f;
        for (int nn = 0; nn < N; ++nn) s += a[(size_t)nn * ML + i];
        o[i] = s;
    }
}
__global__ void r_sum_all(const float* a, size_t n, double* out) {
    // block partial sums in float (as a GPU mapreduce), combined by one atomic per block
    __shared__ float sh[256];
    float s = 0.f;
    GRID_STRIDE(i, n) s += a[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(out, (double)sh[0]);
}

// ---- the reference's custom kernels (src/CDL/csc_kernels.jl, cdl_kernels.jl), 3-D
// (10,10,10) or 2-D (32,32) shapes, l fastest
__global__ void k_shrink(float* Y2, const float* X, const float* y2, float lam, int Lg, int M, int N) {
    int l = blockIdx.x * blockDim.x + threadIdx.x, m = blockIdx.y * blockDim.y + threadIdx.y,
        n = blockIdx.z * blockDim.z + threadIdx.z;
    if (l < Lg && m < M && n < N) {
        size_t i = ((size_t)n * M + m) * Lg + l;
        float t = X[i] + y2[i];
        float sg = t > 0.f ? 1.f : (t < 0.f ? -1.f : 0.f);
        Y2[i] = sg * fmaxf(fabsf(t) - lam, 0.f);
    }
}
__global__ void k_csc_rhs(cplx* R, const cplx* Dh, const cplx* Y1, const cplx* y1, const cplx* Y2,
                          const cplx* y2, const cplx* Y3, const cplx* y3, int Lg, int M, int N) {
    int l = blockIdx.x * blockDim.x + threadIdx.x, m = blockIdx.y * blockDim.y + threadIdx.y,
        n = blockIdx.z * blockDim.z + threadIdx.z;
    if (l < Lg && m < M && n < N) {
        size_t i = ((size_t)n * M + m) * Lg + l, j = (size_t)n * Lg + l;
        R[i] = cadd(cadd(cmul(conjf2(Dh[(size_t)m * Lg + l]), csub(Y1[j], y1[j])), csub(Y2[i], y2[i])),
                    csub(Y3[i], y3[i]));
    }
}
__global__ void k_csc_dot(cplx* re, const cplx* left, const cplx* right, int Lg, int M, int N) {
    int l = blockIdx.x * blockDim.x + threadIdx.x, n = blockIdx.y * blockDim.y + threadIdx.y;
    if (l < Lg && n < N) {
        size_t j = (size_t)n * Lg + l;
        re[j] = make_float2(0.f, 0.f);
        for (int m = 0; m < M; ++m)
            re[j] = cadd(re[j], cmul(left[(size_t)m * Lg + l], right[((size_t)n * M + m) * Lg + l]));
    }
}
__global__ void k_csc_combine(cplx* sol, const cplx* dots, const cplx* Dh, const cplx* right, float k,
                              int Lg, int M, int N) {
    int l = blockIdx.x * blockDim.x + threadIdx.x, m = blockIdx.y * blockDim.y + threadIdx.y,
        n = blockIdx.z * blockDim.z + threadIdx.z;
    if (l < Lg && m < M && n < N) {
        size_t i = ((size_t)n * M + m) * Lg + l;
        cplx t = csub(right[i], cmul(dots[(size_t)n * Lg + l], conjf2(Dh[(size_t)m * Lg + l])));
        sol[i] = make_float2(t.x / k, t.y / k);
    }
}
__global__ void k_update_Y1(float* Y1, const float* WtW, const float* WtS, const float* DX, const float* y1,
                            float rho, int Lg, int N) {
    int l = blockIdx.x * blockDim.x + threadIdx.x, n = blockIdx.y * blockDim.y + threadIdx.y;
    if (l < Lg && n < N) {
        size_t j = (size_t)n * Lg + l;
        Y1[j] = (WtS[j] + rho * (DX[j] + y1[j])) / (WtW[(size_t)l * Lg + l] + rho);
    }
}
__global__ void k_projectionX(float* Y3, const float* X, const float* y3, int Lg, int M, int N) {
    int l = blockIdx.x * blockDim.x + threadIdx.x, m = blockIdx.y * blockDim.y + threadIdx.y,
        n = blockIdx.z * blockDim.z + threadIdx.z;
    if (l < Lg && m < M && n < N) {
        size_t i = ((size_t)n * M + m) * Lg + l;
        Y3[i] = (l % 4 != 0) ? 0.f : X[i] + y3[i];
    }
}
__global__ void k_cdl_rhs(cplx* R, const cplx* Xh, const cplx* G1, const cplx* g1, const cplx* G2,
                          const cplx* g2, const cplx* G3, const cplx* g3, int Lg, int M, int N) {
    int l = blockIdx.x * blockDim.x + threadIdx.x, m = blockIdx.y * blockDim.y + threadIdx.y,
        n = blockIdx.z * blockDim.z + threadIdx.z;
    if (l < Lg && m < M && n < N) {
        size_t i = ((size_t)n * M + m) * Lg + l, j = (size_t)n * Lg + l, p = (size_t)m * Lg + l;
        R[i] = cadd(cadd(cmul(conjf2(Xh[i]), csub(G2[j], g2[j])), csub(G1[p], g1[i])), csub(G3[p], g3[i]));
    }
}
__global__ void k_cdl_combine(cplx* dt, const cplx* R, const cplx* beta, const cplx* X, int Lg, int M, int N) {
    int l = blockIdx.x * blockDim.x + threadIdx.x, m = blockIdx.y * blockDim.y + threadIdx.y,
        n = blockIdx.z * blockDim.z + threadIdx.z;
    if (l < Lg && m < M && n < N) {
        size_t i = ((size_t)n * M + m) * Lg + l;
        dt[i] = csub(R[i], cmul(beta[(size_t)n * Lg + l], conjf2(X[i])));
    }
}
__global__ void k_update_g2(float* G2, const float* WtW, const float* WtS, const float* Td, const float* g2,
                            float sigma, int Lg, int N) {
    int l = blockIdx.x * blockDim.x + threadIdx.x, n = blockIdx.y * blockDim.y + threadIdx.y;
    if (l < Lg && n < N) {
        size_t j = (size_t)n * Lg + l;
        G2[j] = (WtS[j] + sigma * (Td[j] + g2[j])) / (WtW[(size_t)l * Lg + l] + sigma);
    }
}
__global__ void k_box(float* G3, const float* v, const float* PD, int Lg, int M) {
    int l = blockIdx.x * blockDim.x + threadIdx.x, m = blockIdx.y * blockDim.y + threadIdx.y;
    if (l < Lg && m < M) {
        size_t p = (size_t)m * Lg + l;
        if (v[p] >= 1.f) G3[p] = PD[p] != 0.f ? 1.f : 0.f;
        else if (v[p] <= 0.f) G3[p] = 0.f;
        else G3[p] = PD[p] != 0.f ? v[p] : 0.f;
    }
}
__global__ void k_prox(float* G1, const float* v, const float* PD, int Lg, int M) {
    int l = blockIdx.x * blockDim.x + threadIdx.x, m = blockIdx.y * blockDim.y + threadIdx.y;
    if (l < Lg && m < M) {
        size_t p = (size_t)m * Lg + l;
        if (PD[p] != 0.f) {
            int i = 4 * ((l + 1) / 4);      // 1-based i = 4 floor(l/4); rows i+1..i+4 (1-based)
            const float* vm = v + (size_t)m * Lg;
            G1[p] = (float)((double)v[p] - 0.25 * (double)(vm[i] + vm[i + 1] + vm[i + 2] + vm[i + 3] - 1.f));
        } else {
            G1[p] = 0.f;
        }
    }
}

// ---- plumbing
template <class T>
int alloc(RS* r, T** p, size_t n) {
    RS_TRY(cudaMallocAsync((void**)p, n * sizeof(T), r->s));
    return 0;
}
template <class T>
void release(RS* r, T*& p) {
    if (p) cudaFreeAsync(p, r->s);
    p = nullptr;
}
dim3 g1d(size_t n) {
    size_t b = (n + 255) / 256;
    if (b > 152 * 64) b = 152 * 64;
    return dim3((unsigned)b);
}
dim3 g3d(int Lg, int M, int N) { return dim3((Lg + 9) / 10, (M + 9) / 10, (N + 9) / 10); }
dim3 g2d(int a, int b) { return dim3((a + 31) / 32, (b + 31) / 32); }
const dim3 kT3(10, 10, 10), kT2(32, 32);
int sync(RS* r) {
    RS_TRY(cudaStreamSynchronize(r->s));
    return 0;
}

// out = fft(real array) along Lg: promotion, then C2C into a new array (the old result freed)
int fft_real(RS* r, cufftHandle plan, const float* a, size_t n, cplx** out) {
    cplx* tmp;
    if (alloc(r, &tmp, n)) return -1;
    b_promote<<<g1d(n), 256, 0, r->s>>>(a, tmp, n);
    cplx* o;
    if (alloc(r, &o, n)) return -1;
    FFT_TRY(cufftExecC2C(plan, (cufftComplex*)tmp, (cufftComplex*)o, CUFFT_FORWARD));
    release(r, tmp);
    release(r, *out);
    *out = o;
    return 0;
}
// out = fft(complex array)
int fft_c(RS* r, cufftHandle plan, const cplx* a, size_t n, cplx** out) {
    cplx* o;
    if (alloc(r, &o, n)) return -1;
    FFT_TRY(cufftExecC2C(plan, (cufftComplex*)a, (cufftComplex*)o, CUFFT_FORWARD));
    release(r, *out);
    *out = o;
    return 0;
}
// out = real.(ifft(a)): C2C inverse into a new array, the 1/Lg scaling pass, real.
int ifft_real(RS* r, cufftHandle plan, const cplx* a, size_t n, float** out) {
    cplx* tmp;
    if (alloc(r, &tmp, n)) return -1;
    FFT_TRY(cufftExecC2C(plan, (cufftComplex*)a, (cufftComplex*)tmp, CUFFT_INVERSE));
    b_scale<<<g1d(n), 256, 0, r->s>>>(tmp, 1.f / (float)r->Lg, n);
    float* o;
    if (alloc(r, &o, n)) return -1;
    b_real<<<g1d(n), 256, 0, r->s>>>(tmp, o, n);
    release(r, tmp);
    release(r, *out);
    *out = o;
    return 0;
}

int code_update(RS* r, int iters) {
    const int Lg = r->Lg, M = r->M, N = r->N;
    const size_t LMN = (size_t)Lg * M * N, LN = (size_t)Lg * N, LM = (size_t)Lg * M;
    for (int it = 0; it < iters; ++it) {
        k_shrink<<<g3d(Lg, M, N), kT3, 0, r->s>>>(r->Y2, r->X, r->y2, r->lam, Lg, M, N);
        if (sync(r)) return -1;
        if (fft_real(r, r->pLMN, r->Y2, LMN, &r->Y2h)) return -1;
        b_dual<<<g1d(LN), 256, 0, r->s>>>(r->y1, r->DX, r->Y1, LN);
        if (fft_real(r, r->pLN, r->y1, LN, &r->y1h)) return -1;
        b_dual<<<g1d(LMN), 256, 0, r->s>>>(r->y2, r->X, r->Y2, LMN);
        if (fft_real(r, r->pLMN, r->y2, LMN, &r->y2h)) return -1;
        b_dual<<<g1d(LMN), 256, 0, r->s>>>(r->y3, r->X, r->Y3, LMN);
        if (fft_real(r, r->pLMN, r->y3, LMN, &r->y3h)) return -1;
        // Sherman-Morrison prep (train.jl:18-20)
        cplx* t;
        if (alloc(r, &t, LM)) return -1;
        b_abs2<<<g1d(LM), 256, 0, r->s>>>(r->G1h, t, LM);
        release(r, r->dots_csc); r->dots_csc = t;
        cplx* red;
        if (alloc(r, &red, (size_t)Lg)) return -1;
        r_sum_m_c<<<g1d(Lg), 256, 0, r->s>>>(r->dots_csc, red, M, Lg, 1);
        if (alloc(r, &t, (size_t)Lg)) return -1;
        b_addc<<<g1d(Lg), 256, 0, r->s>>>(red, t, r->kcsc, Lg);
        release(r, red);
        release(r, r->sum_dots_csc); r->sum_dots_csc = t;
        if (alloc(r, &t, LM)) return -1;
        b_div_csc<<<g1d(LM), 256, 0, r->s>>>(r->G1h, r->sum_dots_csc, t, LM, Lg);
        release(r, r->A_csc); r->A_csc = t;
        // per-iteration allocations (train.jl:21-22)
        release(r, r->RHS_csc);
        if (alloc(r, &r->RHS_csc, LMN)) return -1;
        release(r, r->alpha_csc);
        if (alloc(r, &r->alpha_csc, LN)) return -1;
        k_csc_rhs<<<g3d(Lg, M, N), kT3, 0, r->s>>>(r->RHS_csc, r->G1h, r->Y1h, r->y1h, r->Y2h, r->y2h,
                                                     r->Y3h, r->y3h, Lg, M, N);
        if (sync(r)) return -1;
        k_csc_dot<<<g2d(Lg, N), kT2, 0, r->s>>>(r->alpha_csc, r->A_csc, r->RHS_csc, Lg, M, N);
        if (sync(r)) return -1;
        k_csc_combine<<<g3d(Lg, M, N), kT3, 0, r->s>>>(r->Xh, r->alpha_csc, r->G1h, r->RHS_csc, r->kcsc,
                                                         Lg, M, N);
        if (sync(r)) return -1;
        if (ifft_real(r, r->pLMN, r->Xh, LMN, &r->X)) return -1;
        // DX = real(ifft(sum(G1h .* Xh, dims=2)))
        if (alloc(r, &t, LMN)) return -1;
        b_mul_bcast<<<g1d(LMN), 256, 0, r->s>>>(r->G1h, r->Xh, t, LMN, LM);
        if (alloc(r, &red, LN)) return -1;
        r_sum_m_c<<<g1d(LN), 256, 0, r->s>>>(t, red, M, Lg, N);
        release(r, t);
        if (ifft_real(r, r->pLN, red, LN, &r->DX)) return -1;
        release(r, red);
        // WDX = W * DX (unused): (N, 4L) = DX (N, Lg) * W^T
        float* wdx;
        if (alloc(r, &wdx, (size_t)r->L4 * N)) return -1;
        const float one = 1.f, zero = 0.f;
        if (cublasSgemm(r->blas, CUBLAS_OP_T, CUBLAS_OP_N, r->L4, N, Lg, &one, r->W, Lg, r->DX, Lg, &zero,
                        wdx, r->L4) != CUBLAS_STATUS_SUCCESS) {
            snprintf(r->err, sizeof r->err, "cublasSgemm failed");
            return -1;
        }
        release(r, r->WDX); r->WDX = wdx;
        k_update_Y1<<<g2d(Lg, N), kT2, 0, r->s>>>(r->Y1, r->WtW, r->WtS, r->DX, r->y1, r->rho, Lg, N);
        if (sync(r)) return -1;
        if (fft_real(r, r->pLN, r->Y1, LN, &r->Y1h)) return -1;
        k_projectionX<<<g3d(Lg, M, N), kT3, 0, r->s>>>(r->Y3, r->X, r->y3, Lg, M, N);
        if (sync(r)) return -1;
        if (fft_real(r, r->pLMN, r->Y3, LMN, &r->Y3h)) return -1;
    }
    return 0;
}

int dict_update(RS* r, int iters) {
    const int Lg = r->Lg, M = r->M, N = r->N;
    const size_t LMN = (size_t)Lg * M * N, LN = (size_t)Lg * N, LM = (size_t)Lg * M;
    for (int it = 0; it < iters; ++it) {
        cplx *t, *red;
        if (alloc(r, &t, LMN)) return -1;
        b_abs2<<<g1d(LMN), 256, 0, r->s>>>(r->Y3h, t, LMN);
        release(r, r->dots_cdl); r->dots_cdl = t;
        if (alloc(r, &red, LN)) return -1;
        r_sum_m_c<<<g1d(LN), 256, 0, r->s>>>(r->dots_cdl, red, M, Lg, N);
        if (alloc(r, &t, LN)) return -1;
        b_addc<<<g1d(LN), 256, 0, r->s>>>(red, t, r->kcdl, LN);
        release(r, red);
        release(r, r->sum_dots_cdl); r->sum_dots_cdl = t;
        if (alloc(r, &t, LMN)) return -1;
        b_div_cdl<<<g1d(LMN), 256, 0, r->s>>>(r->Y3h, r->sum_dots_cdl, t, LMN, Lg, M);
        release(r, r->X_cdl); r->X_cdl = t;
        release(r, r->RHS_cdl);
        if (alloc(r, &r->RHS_cdl, LMN)) return -1;
        RS_TRY(cudaMemsetAsync(r->RHS_cdl, 0, LMN * sizeof(cplx), r->s));
        // ifft_elem_mult = ifft(sum(Y3h .* dh, dims=2)); Td = real.(...)
        if (alloc(r, &t, LMN)) return -1;
        b_mul<<<g1d(LMN), 256, 0, r->s>>>(r->Y3h, r->dh, t, LMN);
        if (alloc(r, &red, LN)) return -1;
        r_sum_m_c<<<g1d(LN), 256, 0, r->s>>>(t, red, M, Lg, N);
        release(r, t);
        cplx* iem;
        if (alloc(r, &iem, LN)) return -1;
        FFT_TRY(cufftExecC2C(r->pLN, (cufftComplex*)red, (cufftComplex*)iem, CUFFT_INVERSE));
        b_scale<<<g1d(LN), 256, 0, r->s>>>(iem, 1.f / (float)Lg, LN);
        release(r, red);
        release(r, r->ifft_elem_mult); r->ifft_elem_mult = iem;
        float* td;
        if (alloc(r, &td, LN)) return -1;
        b_real<<<g1d(LN), 256, 0, r->s>>>(r->ifft_elem_mult, td, LN);
        release(r, r->Td); r->Td = td;
        k_cdl_rhs<<<g3d(Lg, M, N), kT3, 0, r->s>>>(r->RHS_cdl, r->Y3h, r->G1h, r->g1h, r->G2h, r->g2h, r->G3h,
                                                     r->g3h, Lg, M, N);
        if (sync(r)) return -1;
        // beta = sum(X_cdl .* RHS_cdl, dims=2)
        if (alloc(r, &t, LMN)) return -1;
        b_mul<<<g1d(LMN), 256, 0, r->s>>>(r->X_cdl, r->RHS_cdl, t, LMN);
        if (alloc(r, &red, LN)) return -1;
        r_sum_m_c<<<g1d(LN), 256, 0, r->s>>>(t, red, M, Lg, N);
        release(r, t);
        release(r, r->beta_cdl); r->beta_cdl = red;
        k_cdl_combine<<<g3d(Lg, M, N), kT3, 0, r->s>>>(r->dh, r->RHS_cdl, r->beta_cdl, r->Y3h, Lg, M, N);
        if (sync(r)) return -1;
        if (ifft_real(r, r->pLMN, r->dh, LMN, &r->d)) return -1;
        k_update_g2<<<g2d(Lg, N), kT2, 0, r->s>>>(r->G2, r->WtW, r->WtS, r->Td, r->g2, r->sigma, Lg, N);
        if (sync(r)) return -1;
        if (fft_real(r, r->pLN, r->G2, LN, &r->G2h)) return -1;
        float* nv;
        if (alloc(r, &nv, LMN)) return -1;
        b_dual_bc<<<g1d(LMN), 256, 0, r->s>>>(r->g1, r->d, r->G1, nv, LMN, LM);
        release(r, r->g1); r->g1 = nv;
        if (fft_real(r, r->pLMN, r->g1, LMN, &r->g1h)) return -1;
        if (alloc(r, &nv, LN)) return -1;
        b_dual_bc<<<g1d(LN), 256, 0, r->s>>>(r->g2, r->Td, r->G2, nv, LN, LN);
        release(r, r->g2); r->g2 = nv;
        if (fft_real(r, r->pLN, r->g2, LN, &r->g2h)) return -1;
        if (alloc(r, &nv, LMN)) return -1;
        b_dual_bc<<<g1d(LMN), 256, 0, r->s>>>(r->g3, r->d, r->G3, nv, LMN, LM);
        release(r, r->g3); r->g3 = nv;
        if (fft_real(r, r->pLMN, r->g3, LMN, &r->g3h)) return -1;
        // v_avg_2 = sum(d .+ g3, dims=3) ./ N; projection2box!
        for (int which = 0; which < 2; ++which) {
            float *s1, *s2, *va;
            if (alloc(r, &s1, LMN)) return -1;
            b_add_real<<<g1d(LMN), 256, 0, r->s>>>(r->d, which == 0 ? r->g3 : r->g1, s1, LMN);
            if (alloc(r, &s2, LM)) return -1;
            r_sum_n<<<g1d(LM), 256, 0, r->s>>>(s1, s2, N, LM);
            release(r, s1);
            if (alloc(r, &va, LM)) return -1;
            b_divN<<<g1d(LM), 256, 0, r->s>>>(s2, va, (float)N, LM);
            release(r, s2);
            if (which == 0) {
                release(r, r->v_avg_2); r->v_avg_2 = va;
                k_box<<<g2d(Lg, M), kT2, 0, r->s>>>(r->G3, r->v_avg_2, r->P_D, Lg, M);
                if (sync(r)) return -1;
                if (fft_real(r, r->pLM, r->G3, LM, &r->G3h)) return -1;
            } else {
                release(r, r->v_avg_1); r->v_avg_1 = va;
                k_prox<<<g2d(Lg, M), kT2, 0, r->s>>>(r->G1, r->v_avg_1, r->P_D, Lg, M);
                if (sync(r)) return -1;
                if (fft_real(r, r->pLM, r->G1, LM, &r->G1h)) return -1;
            }
        }
    }
    return 0;
}

// 0.5 ||W DX - dat||^2 + lambda sum |X|  (src/SETUP/CDL_setup.jl:286)
int objective(RS* r, double* obj) {
    const int Lg = r->Lg, N = r->N;
    const size_t LMN = (size_t)Lg * r->M * N, n4 = (size_t)r->L4 * N;
    float *wdx, *res;
    if (alloc(r, &wdx, n4)) return -1;
    const float one = 1.f, zero = 0.f;
    if (cublasSgemm(r->blas, CUBLAS_OP_T, CUBLAS_OP_N, r->L4, N, Lg, &one, r->W, Lg, r->DX, Lg, &zero, wdx,
                    r->L4) != CUBLAS_STATUS_SUCCESS) {
        snprintf(r->err, sizeof r->err, "cublasSgemm failed");
        return -1;
    }
    if (alloc(r, &res, n4)) return -1;
    b_sub_real<<<g1d(n4), 256, 0, r->s>>>(wdx, r->dat, res, n4);
    float nrm = 0.f;
    if (cublasSnrm2(r->blas, (int)n4, res, 1, &nrm) != CUBLAS_STATUS_SUCCESS) {
        snprintf(r->err, sizeof r->err, "cublasSnrm2 failed");
        return -1;
    }
    release(r, wdx);
    release(r, res);
    float* ab;
    if (alloc(r, &ab, LMN)) return -1;
    b_abs<<<g1d(LMN), 256, 0, r->s>>>(r->X, ab, LMN);
    double* acc;
    if (alloc(r, &acc, 1)) return -1;
    RS_TRY(cudaMemsetAsync(acc, 0, sizeof(double), r->s));
    r_sum_all<<<g1d(LMN), 256, 0, r->s>>>(ab, LMN, acc);
    double sabs = 0;
    RS_TRY(cudaMemcpyAsync(&sabs, acc, sizeof(double), cudaMemcpyDeviceToHost, r->s));
    if (sync(r)) return -1;
    release(r, ab);
    release(r, acc);
    *obj = 0.5 * (double)(nrm * nrm) + (double)(r->lam * (float)sabs);
    return 0;
}

int update_best(RS* r, double* obj) {
    if (objective(r, obj)) return -1;
    if (*obj < r->obj_best) {
        r->obj_best = *obj;
        const size_t LM = (size_t)r->Lg * r->M, LMN = LM * r->N;
        float* s2;
        if (alloc(r, &s2, LM)) return -1;
        r_sum_n<<<g1d(LM), 256, 0, r->s>>>(r->d, s2, r->N, LM);
        float* db;
        if (alloc(r, &db, LM)) return -1;
        b_divN<<<g1d(LM), 256, 0, r->s>>>(s2, db, (float)r->N, LM);
        release(r, s2);
        release(r, r->D_best); r->D_best = db;
        float* xb;
        if (alloc(r, &xb, LMN)) return -1;
        RS_TRY(cudaMemcpyAsync(xb, r->X, LMN * sizeof(float), cudaMemcpyDeviceToDevice, r->s));
        release(r, r->X_best); r->X_best = xb;
    }
    return 0;
}

void destroy(RS* r) {
    float** fs[] = {&r->X, &r->Y2, &r->Y3, &r->y2, &r->y3, &r->d, &r->g1, &r->g3, &r->X_best, &r->DX, &r->Y1,
                    &r->y1, &r->Td, &r->G2, &r->g2, &r->WtS, &r->WDX, &r->G1, &r->G3, &r->P_D, &r->D_best,
                    &r->WtW, &r->W, &r->dat, &r->v_avg_1, &r->v_avg_2};
    for (float** p : fs) release(r, *p);
    cplx** cs[] = {&r->Xh, &r->Y2h, &r->y2h, &r->Y3h, &r->y3h, &r->dh, &r->g1h, &r->g3h, &r->RHS_csc,
                   &r->dots_cdl, &r->X_cdl, &r->RHS_cdl, &r->Y1h, &r->y1h, &r->G2h, &r->g2h, &r->alpha_csc,
                   &r->ifft_elem_mult, &r->beta_cdl, &r->G1h, &r->G3h, &r->dots_csc, &r->A_csc,
                   &r->sum_dots_csc, &r->sum_dots_cdl};
    for (cplx** p : cs) release(r, *p);
    cudaStreamSynchronize(r->s);
    if (r->pLMN) cufftDestroy(r->pLMN);
    if (r->pLN) cufftDestroy(r->pLN);
    if (r->pLM) cufftDestroy(r->pLM);
    if (r->blas) cublasDestroy(r->blas);
    if (r->s) cudaStreamDestroy(r->s);
}

}  // namespace

extern "C" {

const char* rs_last_error(void* h) { return h ? ((RS*)h)->err : "null handle"; }

// The cdl constructor (src/SETUP/CDL_setup.jl:165-270) from given X0 (N, M, Lg) and D0
// (M, Lg), masked as there; S is the one-hot data (N, 4L).  Returns 0 or -1 (see
// rs_last_error; *out is set in both cases unless allocation of the handle failed).
int rs_create(int L4, int N, int M, int filter_size, float rho, float sigma, float lam, const float* S,
              const float* X0, const float* D0, void** out) {
    RS* r = (RS*)calloc(1, sizeof(RS));
    if (!r) return -1;
    *out = r;
    r->N = N; r->M = M; r->L4 = L4; r->flen = 4 * filter_size; r->gamma = r->flen;
    r->Lg = L4 + 2 * r->gamma;
    r->rho = rho; r->sigma = sigma; r->lam = lam; r->kcsc = 2.f; r->kcdl = 2.f;
    const int Lg = r->Lg;
    const size_t LMN = (size_t)Lg * M * N, LN = (size_t)Lg * N, LM = (size_t)Lg * M;
    RS_TRY(cudaStreamCreateWithFlags(&r->s, cudaStreamNonBlocking));
    {
        // keep freed blocks in the stream-ordered pool, as CUDA.jl's pool allocator does
        int dev = 0;
        cudaMemPool_t pool;
        RS_TRY(cudaGetDevice(&dev));
        RS_TRY(cudaDeviceGetDefaultMemPool(&pool, dev));
        uint64_t thr = ~0ull;
        RS_TRY(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
    }
    if (cublasCreate(&r->blas) != CUBLAS_STATUS_SUCCESS) { snprintf(r->err, sizeof r->err, "cublasCreate"); return -1; }
    cublasSetStream(r->blas, r->s);
    int nl[1] = {Lg};
    FFT_TRY(cufftPlanMany(&r->pLMN, 1, nl, nullptr, 1, Lg, nullptr, 1, Lg, CUFFT_C2C, M * N));
    FFT_TRY(cufftPlanMany(&r->pLN, 1, nl, nullptr, 1, Lg, nullptr, 1, Lg, CUFFT_C2C, N));
    FFT_TRY(cufftPlanMany(&r->pLM, 1, nl, nullptr, 1, Lg, nullptr, 1, Lg, CUFFT_C2C, M));
    cufftSetStream(r->pLMN, r->s); cufftSetStream(r->pLN, r->s); cufftSetStream(r->pLM, r->s);
    // host-side masks and matrices
    std::vector<float> X((size_t)LMN), D(LM), PD(LM, 0.f), W((size_t)L4 * Lg, 0.f), WtW((size_t)Lg * Lg, 0.f),
        WtS(LN, 0.f);
    for (size_t i = 0; i < LMN; ++i) X[i] = (i % Lg) % 4 == 0 ? X0[i] : 0.f;   // enforce_dummy_code_constraint!
    for (int m = 0; m < M; ++m)
        for (int l = 0; l < Lg; ++l) {
            PD[(size_t)m * Lg + l] = l < r->flen ? 1.f : 0.f;                   // make_D_projector
            D[(size_t)m * Lg + l] = PD[(size_t)m * Lg + l] * D0[(size_t)m * Lg + l];
        }
    for (int k = 0; k < L4; ++k) W[(size_t)k * Lg + r->gamma + k] = 1.f;        // W[:, gamma+1:gamma+L] = I
    for (int l = r->gamma; l < r->gamma + L4; ++l) WtW[(size_t)l * Lg + l] = 1.f;
    for (int n = 0; n < N; ++n)
        for (int k = 0; k < L4; ++k) WtS[(size_t)n * Lg + r->gamma + k] = S[(size_t)n * L4 + k];
    if (alloc(r, &r->X, LMN) || alloc(r, &r->G1, LM) || alloc(r, &r->P_D, LM) || alloc(r, &r->W, (size_t)L4 * Lg) ||
        alloc(r, &r->WtW, (size_t)Lg * Lg) || alloc(r, &r->WtS, LN) || alloc(r, &r->dat, (size_t)L4 * N))
        return -1;
    RS_TRY(cudaMemcpyAsync(r->X, X.data(), LMN * 4, cudaMemcpyHostToDevice, r->s));
    RS_TRY(cudaMemcpyAsync(r->G1, D.data(), LM * 4, cudaMemcpyHostToDevice, r->s));
    RS_TRY(cudaMemcpyAsync(r->P_D, PD.data(), LM * 4, cudaMemcpyHostToDevice, r->s));
    RS_TRY(cudaMemcpyAsync(r->W, W.data(), W.size() * 4, cudaMemcpyHostToDevice, r->s));
    RS_TRY(cudaMemcpyAsync(r->WtW, WtW.data(), WtW.size() * 4, cudaMemcpyHostToDevice, r->s));
    RS_TRY(cudaMemcpyAsync(r->WtS, WtS.data(), LN * 4, cudaMemcpyHostToDevice, r->s));
    RS_TRY(cudaMemcpyAsync(r->dat, S, (size_t)L4 * N * 4, cudaMemcpyHostToDevice, r->s));
    // D-hat, X-hat, DX, d-hat = D-hat broadcast, d, Td = 0
    if (fft_real(r, r->pLM, r->G1, LM, &r->G1h)) return -1;
    if (fft_real(r, r->pLMN, r->X, LMN, &r->Xh)) return -1;
    cplx *t, *red;
    if (alloc(r, &t, LMN)) return -1;
    b_mul_bcast<<<g1d(LMN), 256, 0, r->s>>>(r->G1h, r->Xh, t, LMN, LM);
    if (alloc(r, &red, LN)) return -1;
    r_sum_m_c<<<g1d(LN), 256, 0, r->s>>>(t, red, M, Lg, N);
    release(r, t);
    if (ifft_real(r, r->pLN, red, LN, &r->DX)) return -1;
    release(r, red);
    if (alloc(r, &r->dh, LMN)) return -1;
    for (int n = 0; n < N; ++n)
        RS_TRY(cudaMemcpyAsync(r->dh + (size_t)n * LM, r->G1h, LM * sizeof(cplx), cudaMemcpyDeviceToDevice, r->s));
    if (ifft_real(r, r->pLMN, r->dh, LMN, &r->d)) return -1;
    if (alloc(r, &r->Td, LN)) return -1;
    RS_TRY(cudaMemsetAsync(r->Td, 0, LN * 4, r->s));
    // auxiliaries: Y1 = 0, Y2 = Y3 = X, y1 = y2 = y3 = 0, G1 = G3 = D, G2 = DX, g = 0
    if (alloc(r, &r->Y1, LN) || alloc(r, &r->y1, LN) || alloc(r, &r->Y2, LMN) || alloc(r, &r->Y3, LMN) ||
        alloc(r, &r->y2, LMN) || alloc(r, &r->y3, LMN) || alloc(r, &r->G3, LM) || alloc(r, &r->G2, LN) ||
        alloc(r, &r->g1, LMN) || alloc(r, &r->g3, LMN) || alloc(r, &r->g2, LN))
        return -1;
    RS_TRY(cudaMemsetAsync(r->Y1, 0, LN * 4, r->s));
    RS_TRY(cudaMemsetAsync(r->y1, 0, LN * 4, r->s));
    RS_TRY(cudaMemcpyAsync(r->Y2, r->X, LMN * 4, cudaMemcpyDeviceToDevice, r->s));
    RS_TRY(cudaMemcpyAsync(r->Y3, r->X, LMN * 4, cudaMemcpyDeviceToDevice, r->s));
    RS_TRY(cudaMemsetAsync(r->y2, 0, LMN * 4, r->s));
    RS_TRY(cudaMemsetAsync(r->y3, 0, LMN * 4, r->s));
    RS_TRY(cudaMemcpyAsync(r->G3, r->G1, LM * 4, cudaMemcpyDeviceToDevice, r->s));
    RS_TRY(cudaMemcpyAsync(r->G2, r->DX, LN * 4, cudaMemcpyDeviceToDevice, r->s));
    RS_TRY(cudaMemsetAsync(r->g1, 0, LMN * 4, r->s));
    RS_TRY(cudaMemsetAsync(r->g3, 0, LMN * 4, r->s));
    RS_TRY(cudaMemsetAsync(r->g2, 0, LN * 4, r->s));
    if (fft_real(r, r->pLN, r->Y1, LN, &r->Y1h) || fft_real(r, r->pLMN, r->Y2, LMN, &r->Y2h) ||
        fft_real(r, r->pLN, r->y1, LN, &r->y1h) || fft_real(r, r->pLMN, r->y2, LMN, &r->y2h) ||
        fft_real(r, r->pLN, r->G2, LN, &r->G2h))
        return -1;
    if (alloc(r, &r->Y3h, LMN) || alloc(r, &r->y3h, LMN) || alloc(r, &r->G3h, LM) || alloc(r, &r->g1h, LMN) ||
        alloc(r, &r->g3h, LMN) || alloc(r, &r->g2h, LN))
        return -1;
    RS_TRY(cudaMemcpyAsync(r->Y3h, r->Y2h, LMN * 8, cudaMemcpyDeviceToDevice, r->s));
    RS_TRY(cudaMemcpyAsync(r->y3h, r->y2h, LMN * 8, cudaMemcpyDeviceToDevice, r->s));
    RS_TRY(cudaMemcpyAsync(r->G3h, r->G1h, LM * 8, cudaMemcpyDeviceToDevice, r->s));
    RS_TRY(cudaMemcpyAsync(r->g1h, r->y2h, LMN * 8, cudaMemcpyDeviceToDevice, r->s));
    RS_TRY(cudaMemcpyAsync(r->g3h, r->y2h, LMN * 8, cudaMemcpyDeviceToDevice, r->s));
    RS_TRY(cudaMemcpyAsync(r->g2h, r->Y1h, LN * 8, cudaMemcpyDeviceToDevice, r->s));
    if (alloc(r, &r->D_best, LM) || alloc(r, &r->X_best, LMN)) return -1;
    RS_TRY(cudaMemcpyAsync(r->D_best, r->G1, LM * 4, cudaMemcpyDeviceToDevice, r->s));
    RS_TRY(cudaMemcpyAsync(r->X_best, r->Y3, LMN * 4, cudaMemcpyDeviceToDevice, r->s));
    double obj = 0;
    if (objective(r, &obj)) return -1;
    r->obj_best = obj;
    return sync(r);
}

// `iters` outer iterations of cdl_optimize (src/WRAPPER/wrap.jl:6-11): code_update!(csc),
// update_best!, dict_update!(cdl); objs[i] = the objective update_best! computed.
int rs_run_outer(void* h, int iters, int csc, int cdl, double* objs) {
    RS* r = (RS*)h;
    for (int i = 0; i < iters; ++i) {
        if (code_update(r, csc)) return -1;
        double o = 0;
        if (update_best(r, &o)) return -1;
        if (objs) objs[i] = o;
        if (dict_update(r, cdl)) return -1;
    }
    return sync(r);
}

// 0 X, 1 d, 2 G1, 3 D_best, 4 DX, 5 X_best: copied to host (sizes as the fields)
int rs_get(void* h, int field, float* dst) {
    RS* r = (RS*)h;
    const size_t LMN = (size_t)r->Lg * r->M * r->N, LM = (size_t)r->Lg * r->M, LN = (size_t)r->Lg * r->N;
    const float* src = nullptr;
    size_t n = 0;
    switch (field) {
        case 0: src = r->X; n = LMN; break;
        case 1: src = r->d; n = LMN; break;
        case 2: src = r->G1; n = LM; break;
        case 3: src = r->D_best; n = LM; break;
        case 4: src = r->DX; n = LN; break;
        case 5: src = r->X_best; n = LMN; break;
        default: snprintf(r->err, sizeof r->err, "unknown field %d", field); return -1;
    }
    RS_TRY(cudaMemcpyAsync(dst, src, n * 4, cudaMemcpyDeviceToHost, r->s));
    return sync(r);
}

void rs_destroy(void* h) {
    if (!h) return;
    destroy((RS*)h);
    free(h);
}

}  // extern "C"
