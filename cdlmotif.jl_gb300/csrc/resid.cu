// Residual norms of the ADMM and the stopping test, accumulated in float64.
//
// The reference runs a fixed number of iterations (cdl_optimize, src/WRAPPER/wrap.jl:6-11)
// and computes no residual.  The record kept here (RESIDUAL_* below, 19 float64 values)
// holds, after each code update, the primal residuals of its final iterate -- the
// vectors the next dual updates of code_update! (src/CDL/train.jl:12-14) would add:
//     X - shrink(X + y2), X - projectionX(X + y3), DX - Y1
// and, after each D-step, the increments its dual updates (train.jl:70-72) added,
//     d - G1_old, d - G3_old, Td - G2,
// with the change of the consensus dictionary (G1, G3) as the D-step's dual residual,
// plus the norms the relative residuals are taken against.  The fused kernels produce
// the X-step sums in their store pass (k_xiter) and the D-step sums in their solve pass
// (k_dspec, through Parseval's relation on the half-spectra); the kernels below cover
// the other paths and the small reductions.  Every sum is split into per-thread
// partials that are combined in float64 in a fixed order, so the record is
// deterministic for a given size and device.
#include "cdlgb_internal.h"

namespace {

constexpr int kRB = 256;       // threads per block of the partial-sum kernels
constexpr int kRGrid = 304;    // blocks of the partial-sum kernels

__device__ __forceinline__ double warp_sum_d(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// block-wide sums of NV values; thread 0 writes part[blockIdx.x * NV + k]
template <int NV>
__device__ __forceinline__ void block_partials(double (&v)[NV], double* part) {
    __shared__ double sh[NV][32];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        v[k] = warp_sum_d(v[k]);
        if (lane == 0) sh[k][w] = v[k];
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        double t = 0.0;
        for (int i = 0; i < nw; ++i) t += sh[threadIdx.x][i];
        part[(size_t)blockIdx.x * NV + threadIdx.x] = t;
    }
}

// X-step residuals from the arrays in memory (paths other than the multi-iteration
// kernel): per block sums of (X - shrink(X + y2))^2, (X - projectionX(X + y3))^2, X^2
// over (Lg, M, N) and of (DX - Y1)^2, DX^2 over (Lg, N).  Lg % 4 == 0, so the rows kept
// by projectionX! are the .x components of the float4s.
__global__ void k_xresid(const float4* __restrict__ X, const float4* __restrict__ y2,
                         const float4* __restrict__ y3, const float* __restrict__ DX,
                         const float* __restrict__ Y1, size_t n4, size_t ln, float lam,
                         double* __restrict__ part) {
    double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4; i += stride) {
        const float4 x = X[i], a = y2[i], b = y3[i];
        const float xs[4] = {x.x, x.y, x.z, x.w}, as[4] = {a.x, a.y, a.z, a.w};
        const float bs[4] = {b.x, b.y, b.z, b.w};
        float q2 = 0.f, q3 = 0.f, qx = 0.f;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float t = xs[k] + as[k];
            const float Y2 = t - fminf(fmaxf(t, -lam), lam);
            const float r2 = xs[k] - Y2;
            const float r3 = k == 0 ? xs[k] - (xs[k] + bs[k]) : xs[k];
            q2 = fmaf(r2, r2, q2);
            q3 = fmaf(r3, r3, q3);
            qx = fmaf(xs[k], xs[k], qx);
        }
        v[0] += (double)q2;
        v[1] += (double)q3;
        v[2] += (double)qx;
    }
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < ln; i += stride) {
        const float dx = DX[i], r = dx - Y1[i];
        v[3] += (double)(r * r);
        v[4] += (double)(dx * dx);
    }
    block_partials<5>(v, part);
}

// (Td - G2)^2 and Td^2 over (Lg, N) -- the g2 increment of the D-step
__global__ void k_tdresid(const float* __restrict__ Td, const float* __restrict__ G2, size_t ln,
                          double* __restrict__ part) {
    double v[2] = {0.0, 0.0};
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < ln;
         i += (size_t)gridDim.x * blockDim.x) {
        const float t = Td[i], r = t - G2[i];
        v[0] += (double)(r * r);
        v[1] += (double)(t * t);
    }
    block_partials<2>(v, part);
}

// the time-domain D-step's increments: (d - G1)^2, (d - G3)^2 and d^2 over (Lg, M, N),
// G1 and G3 (before their update) broadcast over the sequences
__global__ void k_dresid_time(const float4* __restrict__ d, const float4* __restrict__ G1,
                              const float4* __restrict__ G3, size_t n4, size_t lm4,
                              double* __restrict__ part) {
    double v[3] = {0.0, 0.0, 0.0};
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4;
         i += (size_t)gridDim.x * blockDim.x) {
        const float4 x = d[i], a = G1[i % lm4], b = G3[i % lm4];
        const float r1[4] = {x.x - a.x, x.y - a.y, x.z - a.z, x.w - a.w};
        const float r3[4] = {x.x - b.x, x.y - b.y, x.z - b.z, x.w - b.w};
        const float xs[4] = {x.x, x.y, x.z, x.w};
        float q1 = 0.f, q3 = 0.f, qd = 0.f;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            q1 = fmaf(r1[k], r1[k], q1);
            q3 = fmaf(r3[k], r3[k], q3);
            qd = fmaf(xs[k], xs[k], qd);
        }
        v[0] += (double)q1;
        v[1] += (double)q3;
        v[2] += (double)qd;
    }
    block_partials<3>(v, part);
}

// out[map[k]] = scale * sum over nb blocks of part[b * nv + k], k < nv; one warp per
// value, lanes over blocks in a fixed order
struct ResMap { int idx[5]; };
__global__ void k_res_sum(const double* __restrict__ part, int nb, int nv, double scale, ResMap map,
                          double* __restrict__ out) {
    const int k = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (k >= nv) return;
    double t = 0.0;
    for (int b = lane; b < nb; b += 32) t += part[(size_t)b * nv + k];
    t = warp_sum_d(t);
    if (lane == 0) out[map.idx[k]] = scale * t;
}

// the D-step's dual residual: N sum (G1 - G1_old)^2, N sum (G3 - G3_old)^2 and
// N (sum G1^2 + sum G3^2); one block, fixed order
__global__ void k_gdual(const float* __restrict__ G1, const float* __restrict__ G3,
                        const float* __restrict__ Gprev, size_t lm, int N, double* __restrict__ out) {
    double v[3] = {0.0, 0.0, 0.0};
    for (size_t i = threadIdx.x; i < lm; i += blockDim.x) {
        const float a = G1[i], b = G3[i];
        const double e1 = (double)a - (double)Gprev[i], e3 = (double)b - (double)Gprev[lm + i];
        v[0] += e1 * e1;
        v[1] += e3 * e3;
        v[2] += (double)a * a + (double)b * b;
    }
    __shared__ double sh[3][32];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        v[k] = warp_sum_d(v[k]);
        if (lane == 0) sh[k][w] = v[k];
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += sh[threadIdx.x][i];
        out[RESIDUAL_DUAL_G1 + threadIdx.x] = (double)N * t;
    }
}

// the stopping test's relative residuals and their maximum, from the raw sums
__global__ void k_res_finish(double* __restrict__ r) {
    if (threadIdx.x != 0) return;
    const double tiny = 1e-300;
    const double px = sqrt((r[RESIDUAL_X_Y2] + r[RESIDUAL_X_Y3]) / fmax(r[RESIDUAL_X_NORM], tiny));
    const double pdx = sqrt(r[RESIDUAL_X_Y1] / fmax(r[RESIDUAL_DX_NORM], tiny));
    const double pd = sqrt((r[RESIDUAL_D_G1] + r[RESIDUAL_D_G3]) / fmax(2.0 * r[RESIDUAL_D_NORM], tiny));
    const double ptd = sqrt(r[RESIDUAL_D_G2] / fmax(r[RESIDUAL_TD_NORM], tiny));
    const double dd = sqrt((r[RESIDUAL_DUAL_G1] + r[RESIDUAL_DUAL_G3]) / fmax(r[RESIDUAL_G_NORM], tiny));
    r[RESIDUAL_REL_PRIMAL_X] = px;
    r[RESIDUAL_REL_PRIMAL_DX] = pdx;
    r[RESIDUAL_REL_PRIMAL_D] = pd;
    r[RESIDUAL_REL_PRIMAL_TD] = ptd;
    r[RESIDUAL_REL_DUAL_D] = dd;
    r[RESIDUAL_REL_MAX] = fmax(fmax(fmax(px, pdx), fmax(pd, ptd)), dd);
}

}  // namespace

size_t resid_part_doubles(int N, int F, int slots) {
    (void)N;
    const size_t nbb = (size_t)(F + 31) / 32;
    size_t n = (size_t)kRGrid * 5;
    if ((size_t)slots * nbb * 3 > n) n = (size_t)slots * nbb * 3;
    if ((size_t)152 * 8 * 5 > n) n = (size_t)152 * 8 * 5;
    return n;
}

int resid_finish(cdlgb_ctx* c) {
    k_res_finish<<<1, 32, 0, c->stream>>>(c->dres);
    LAUNCH_CHECK(c, "k_res_finish");
    return CDLGB_OK;
}

// X-step record from per-block partials (nb blocks x 5 values) already in memory
int resid_x_from_parts(cdlgb_ctx* c, const double* part, int nb) {
    ResMap m = {{RESIDUAL_X_Y2, RESIDUAL_X_Y3, RESIDUAL_X_NORM, RESIDUAL_X_Y1, RESIDUAL_DX_NORM}};
    k_res_sum<<<1, 5 * 32, 0, c->stream>>>(part, nb, 5, 1.0, m, c->dres);
    LAUNCH_CHECK(c, "k_res_sum");
    return resid_finish(c);
}

// X-step record from the arrays (X the current iterate)
int resid_x_from_arrays(cdlgb_ctx* c, const float* X) {
    k_xresid<<<kRGrid, kRB, 0, c->stream>>>((const float4*)X, (const float4*)c->y2,
                                            (const float4*)c->y3, c->DX, c->Y1, c->LMN / 4, c->LN,
                                            c->p.lambda, c->rpart);
    LAUNCH_CHECK(c, "k_xresid");
    return resid_x_from_parts(c, c->rpart, kRGrid);
}

// D-step increments of d from the spectral solve's partials (nb blocks x 3 values:
// Parseval sums of |d-hat - G1-hat|^2, |d-hat - G3-hat|^2, |d-hat|^2, times Lg)
int resid_d_from_spec_parts(cdlgb_ctx* c, int nb) {
    ResMap m = {{RESIDUAL_D_G1, RESIDUAL_D_G3, RESIDUAL_D_NORM, 0, 0}};
    k_res_sum<<<1, 3 * 32, 0, c->stream>>>(c->rpart, nb, 3, 1.0 / (double)c->Lg, m, c->dres);
    LAUNCH_CHECK(c, "k_res_sum");
    return CDLGB_OK;
}

// D-step increments of d from the time-domain arrays (G1, G3 before their update)
int resid_d_from_arrays(cdlgb_ctx* c) {
    k_dresid_time<<<kRGrid, kRB, 0, c->stream>>>((const float4*)c->d, (const float4*)c->G1,
                                                 (const float4*)c->G3, c->LMN / 4, c->LM / 4,
                                                 c->rpart);
    LAUNCH_CHECK(c, "k_dresid_time");
    ResMap m = {{RESIDUAL_D_G1, RESIDUAL_D_G3, RESIDUAL_D_NORM, 0, 0}};
    k_res_sum<<<1, 3 * 32, 0, c->stream>>>(c->rpart, kRGrid, 3, 1.0, m, c->dres);
    LAUNCH_CHECK(c, "k_res_sum");
    return CDLGB_OK;
}

// the g2 increment, after update_g2!
int resid_td(cdlgb_ctx* c) {
    k_tdresid<<<kRGrid, kRB, 0, c->stream>>>(c->Td, c->G2, c->LN, c->rpart);
    LAUNCH_CHECK(c, "k_tdresid");
    ResMap m = {{RESIDUAL_D_G2, RESIDUAL_TD_NORM, 0, 0, 0}};
    k_res_sum<<<1, 2 * 32, 0, c->stream>>>(c->rpart, kRGrid, 2, 1.0, m, c->dres);
    LAUNCH_CHECK(c, "k_res_sum");
    return CDLGB_OK;
}

// G1, G3 before the projections (called before k_dfinish / k_dprox overwrite them)
int resid_save_G(cdlgb_ctx* c) {
    CU_TRY(c, cudaMemcpyAsync(c->Gprev, c->G1, c->LM * 4, cudaMemcpyDeviceToDevice, c->stream));
    CU_TRY(c, cudaMemcpyAsync(c->Gprev + c->LM, c->G3, c->LM * 4, cudaMemcpyDeviceToDevice, c->stream));
    return CDLGB_OK;
}

// the dual residual after the projections, then the relative residuals
int resid_dual_and_finish(cdlgb_ctx* c) {
    k_gdual<<<1, 512, 0, c->stream>>>(c->G1, c->G3, c->Gprev, c->LM, c->N, c->dres);
    LAUNCH_CHECK(c, "k_gdual");
    return resid_finish(c);
}
