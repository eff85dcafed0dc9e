// ADMM state, initialisation, objective and the cuFFT-transform path of the X- and
// D-steps.
//
// Algebra (exact in real arithmetic; restates src/CDL/train.jl:1-89):
//   The reference keeps ~20 complex spectra and runs 6 LMN-sized c2c FFTs per X-step.
//   Because every signal is real and FFTs are linear, the X-step right-hand side
//     RHS = conj(G1h)(Y1h - y1h) + (Y2h - y2h) + (Y3h - y3h)
//   equals conj(G1h) * rfft(U) + rfft(V) with U = Y1 - y1', V = (Y2 - y2') + (Y3 - y3'),
//   and the Sherman-Morrison solve (csc_kernels.jl:8-49) reduces to one cross-filter sum
//     P = sum_m G1h[m] Vh[m],  alpha = (A Uh + P) / (A + k),  W = Uh - alpha,
//     Xh[m] = (Vh[m] + conj(G1h[m]) W) / k,   DXh = (P + A W) / k,   A = sum_m |G1h[m]|^2.
//   Y3 = projectionX(X + y3) holds at the start of every X-step, so it is recomputed
//   instead of stored.  In the D-step the consensus spectrum d-hat equals rfft(d), so it
//   is recomputed as well, and with H = (G1 - g1) + (G3 - g3), Z = G2 - g2:
//     B = sum|Y3h|^2, Q = sum Y3h Hh, T = sum Y3h rfft(d_old),
//     beta = (Zh B + Q) / (B + k),  dh[m] = Hh[m] + conj(Y3h[m]) (Zh - beta),  Td = irfft(T).
//   Half spectra (F = Lg/2 + 1 bins) replace full complex spectra.
#include "cdlgb_internal.h"

#include <math.h>
#include <stdlib.h>
#include <algorithm>
#include <vector>

namespace {

constexpr int kBlock = 256;

__host__ __device__ inline uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

__device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 c) {  // a*b + c
    return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y)));
}
__device__ __forceinline__ float2 cjfma(float2 a, float2 b, float2 c) {  // conj(a)*b + c
    return make_float2(fmaf(a.x, b.x, fmaf(a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(-a.y, b.x, c.y)));
}

// ---------------------------------------------------------------- init kernels
__global__ void k_bcast_plane(float4* __restrict__ dst, const float4* __restrict__ plane,
                              size_t pl4, size_t n4) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4;
         i += (size_t)gridDim.x * blockDim.x)
        dst[i] = plane[i % pl4];
}

// DXh[n,f] = scale * sum_m Gh[m,f] Xh[n,m,f]
__global__ void k_spec_dot(const float2* __restrict__ Xh, const float2* __restrict__ Gh,
                           float2* __restrict__ out, int F, int M, int N, float scale) {
    size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (t >= (size_t)F * N) return;
    int f = (int)(t % F);
    size_t n = t / F;
    float2 acc = make_float2(0.f, 0.f);
    const float2* x = Xh + n * M * F + f;
    for (int m = 0; m < M; ++m) acc = cfma(Gh[(size_t)m * F + f], x[(size_t)m * F], acc);
    out[t] = make_float2(acc.x * scale, acc.y * scale);
}

// A[f] = sum_m |Gh[m,f]|^2
__global__ void k_colnorm(const float2* __restrict__ Gh, float* __restrict__ A, int F, int M) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= F) return;
    float a = 0.f;
    for (int m = 0; m < M; ++m) {
        float2 g = Gh[(size_t)m * F + f];
        a = fmaf(g.x, g.x, fmaf(g.y, g.y, a));
    }
    A[f] = a;
}

// ---------------------------------------------------------------- X-step kernels
__device__ __forceinline__ void xprep1(float x, float a, float b, float lam, bool keep,
                                       float& na, float& nb, float& v) {
    float t = x + a;                                        // X + y2
    // shrink! (csc_kernels.jl:53-64) at lambda, not lambda / rho (REF_QUIRK_Q4, :61)
    float Y2 = copysignf(fmaxf(fabsf(t) - lam, 0.f), t);
    float Y3 = keep ? x + b : 0.f;                          // projectionX! (:68-82)
    na = (a + x) - Y2;                                      // y2 .+ X .- Y2  (train.jl:13)
    nb = (b + x) - Y3;                                      // y3 .+ X .- Y3  (train.jl:14)
    v = (Y2 - na) + (Y3 - nb);
}

__global__ void k_xprep(const float4* __restrict__ X, float4* __restrict__ y2,
                        float4* __restrict__ y3, float4* __restrict__ V, size_t n4, float lam) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4;
         i += (size_t)gridDim.x * blockDim.x) {
        float4 x = X[i], a = y2[i], b = y3[i], na, nb, v;
        xprep1(x.x, a.x, b.x, lam, true, na.x, nb.x, v.x);
        xprep1(x.y, a.y, b.y, lam, false, na.y, nb.y, v.y);
        xprep1(x.z, a.z, b.z, lam, false, na.z, nb.z, v.z);
        xprep1(x.w, a.w, b.w, lam, false, na.w, nb.w, v.w);
        y2[i] = na;
        y3[i] = nb;
        V[i] = v;
    }
}

// y1' = y1 + DX - Y1 (train.jl:12); U = Y1 - y1'
__global__ void k_xprep_ln(float* __restrict__ y1, const float* __restrict__ DX,
                           const float* __restrict__ Y1, float* __restrict__ U, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        float Yv = Y1[i];
        float yn = (y1[i] + DX[i]) - Yv;
        y1[i] = yn;
        U[i] = Yv - yn;
    }
}

// Per (f, n): the Sherman-Morrison code solve (csc_kernels.jl:8-49, train.jl:18-27), with
// the consensus G1-hat, not d-hat (REF_QUIRK_Q5).
__global__ void k_xsolve(float2* __restrict__ Vh, const float2* __restrict__ Uh,
                         const float2* __restrict__ G1h, const float* __restrict__ Ah,
                         float2* __restrict__ DXh, int F, int M, int nfb, float kc, float scale) {
    int fb = blockIdx.x % nfb;
    size_t n = blockIdx.x / nfb;
    int f = fb * blockDim.x + threadIdx.x;
    if (f >= F) return;
    float2* v = Vh + n * M * F + f;
    float2 P = make_float2(0.f, 0.f);
    for (int m = 0; m < M; ++m) P = cfma(G1h[(size_t)m * F + f], v[(size_t)m * F], P);
    float A = Ah[f];
    float2 u = Uh[n * F + f];
    float inv_s = 1.f / (A + kc);
    float2 alpha = make_float2(fmaf(A, u.x, P.x) * inv_s, fmaf(A, u.y, P.y) * inv_s);
    float2 W = make_float2(u.x - alpha.x, u.y - alpha.y);
    float sc = scale / kc;
    for (int m = 0; m < M; ++m) {
        float2 x = cjfma(G1h[(size_t)m * F + f], W, v[(size_t)m * F]);
        v[(size_t)m * F] = make_float2(x.x * sc, x.y * sc);
    }
    DXh[n * F + f] = make_float2(fmaf(A, W.x, P.x) * sc, fmaf(A, W.y, P.y) * sc);
}

// Y1 = (W'S + rho (DX + y1')) / (W'W_ll + rho)   (update_Y1!, csc_kernels.jl:86-95)
// W'S and diag(W'W) are the data placed in rows gamma..gamma+4L-1 (CDL_setup.jl:213-217).
__global__ void k_mask_update(float* __restrict__ out, const float* __restrict__ a,
                              const float* __restrict__ b, const float* __restrict__ S,
                              int Lg, int L4, int gamma, size_t n, float pen) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        size_t nn = i / Lg;
        int l = (int)(i - nn * Lg);
        bool in = l >= gamma && l < gamma + L4;
        float wts = in ? S[nn * L4 + (l - gamma)] : 0.f;
        float dg = in ? 1.f : 0.f;
        // separately rounded product and sum (no contraction), as the reference's broadcast
        out[i] = __fadd_rn(wts, __fmul_rn(pen, a[i] + b[i])) / (dg + pen);
    }
}

// ---------------------------------------------------------------- D-step kernels
// Y3 = projectionX(X + y3), H = (G1 - g1) + (G3 - g3)
__global__ void k_dprep(const float4* __restrict__ X, const float4* __restrict__ y3,
                        const float4* __restrict__ g1, const float4* __restrict__ g3,
                        const float4* __restrict__ G1, const float4* __restrict__ G3,
                        float4* __restrict__ Y3o, float4* __restrict__ Ho, size_t n4, size_t pl4) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4;
         i += (size_t)gridDim.x * blockDim.x) {
        float4 x = X[i], b = y3[i], p = g1[i], q = g3[i];
        size_t j = i % pl4;
        float4 A = G1[j], C = G3[j];
        Y3o[i] = make_float4(x.x + b.x, 0.f, 0.f, 0.f);
        Ho[i] = make_float4((A.x - p.x) + (C.x - q.x), (A.y - p.y) + (C.y - q.y),
                            (A.z - p.z) + (C.z - q.z), (A.w - p.w) + (C.w - q.w));
    }
}

// Y3 = projectionX!(X + y3) (csc_kernels.jl:68-82) of a chunk, for the spectral D-step on
// lengths without the streaming transforms: X + 0 on the rows l % 4 == 0 (every row
// starts at a multiple of 4 floats, so those are the .x lanes), where every X-step
// leaves y3 = +0 exactly (projectionX! keeps X + y3 there, so y3' = (y3 + X) - Y3 = +0,
// as initialisation sets it), and 0 on the others -- the values k_dfwd transforms.
__global__ void k_y3(const float4* __restrict__ X, float4* __restrict__ Y3, size_t n4) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4;
         i += (size_t)gridDim.x * blockDim.x)
        Y3[i] = make_float4(X[i].x + 0.f, 0.f, 0.f, 0.f);
}

__global__ void k_sub(const float* __restrict__ a, const float* __restrict__ b,
                      float* __restrict__ o, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        o[i] = a[i] - b[i];
}

// Per (f, n): the Sherman-Morrison dictionary solve (cdl_kernels.jl:2-33, train.jl:52-61),
// with T = sum_m Y3h * rfft(d_old) for Td (train.jl:56).  Dh holds rfft(d_old) on entry
// (the imaginary parts of its f = 0 and f = Lg/2 bins, which a real transform has as
// zero, are read as zero) and the new d-hat times scale_out on exit; Th = T * scale.
// A CTA takes 32 bins of one
// sequence; warp w sums filters w, w + 8, w + 16, ... (lane = bin), the eight partial
// sums are added in warp order, and Y3h, Hh stay in shared memory between the sums and
// the update, so every spectrum is read from HBM once (STAGE; without it, for M too
// large for shared memory, the update reads them again).
constexpr int kDsBins = 32, kDsWarps = 8;
template <bool STAGE>
__global__ void __launch_bounds__(kDsBins * kDsWarps) k_dsolve(
    const float2* __restrict__ Yh, const float2* __restrict__ Hh, float2* __restrict__ Dh,
    const float2* __restrict__ Zh, float2* __restrict__ Th, int F, int M, int nfb, float kd,
    float scale, float scale_out) {
    extern __shared__ float4 ds_smem[];
    const int Ms = STAGE ? M : 0;
    float2* ys = reinterpret_cast<float2*>(ds_smem);       // [M][kDsBins]
    float2* hs = ys + (size_t)Ms * kDsBins;                // [M][kDsBins]
    float* pB = reinterpret_cast<float*>(hs + (size_t)Ms * kDsBins);  // [kDsWarps][kDsBins]
    float2* pQ = reinterpret_cast<float2*>(pB + kDsWarps * kDsBins);  // [kDsWarps][kDsBins]
    float2* pT = pQ + kDsWarps * kDsBins;
    const int fb = blockIdx.x % nfb;
    const size_t n = blockIdx.x / nfb;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int f = fb * kDsBins + lane;
    const bool on = f < F;
    const size_t base = n * M * F + (on ? f : 0);
    float B = 0.f;
    float2 Q = make_float2(0.f, 0.f), T = make_float2(0.f, 0.f);
    for (int m = w; m < M; m += kDsWarps) {
        float2 y = make_float2(0.f, 0.f), h = y, d = y;
        if (on) {
            y = Yh[base + (size_t)m * F];
            h = Hh[base + (size_t)m * F];
            d = Dh[base + (size_t)m * F];
            if (f == 0 || f == F - 1) d.y = 0.f;
        }
        if (STAGE) {
            ys[m * kDsBins + lane] = y;
            hs[m * kDsBins + lane] = h;
        }
        B = fmaf(y.x, y.x, fmaf(y.y, y.y, B));
        Q = cfma(y, h, Q);
        T = cfma(y, d, T);
    }
    pB[w * kDsBins + lane] = B;
    pQ[w * kDsBins + lane] = Q;
    pT[w * kDsBins + lane] = T;
    __syncthreads();
    B = 0.f;
    Q = T = make_float2(0.f, 0.f);
    for (int v = 0; v < kDsWarps; ++v) {
        B += pB[v * kDsBins + lane];
        Q = make_float2(Q.x + pQ[v * kDsBins + lane].x, Q.y + pQ[v * kDsBins + lane].y);
        T = make_float2(T.x + pT[v * kDsBins + lane].x, T.y + pT[v * kDsBins + lane].y);
    }
    if (!on) return;
    const float2 z = Zh[n * F + f];
    const float inv = 1.f / (B + kd);
    const float2 beta = make_float2(fmaf(z.x, B, Q.x) * inv, fmaf(z.y, B, Q.y) * inv);
    const float2 W = make_float2(z.x - beta.x, z.y - beta.y);
    for (int m = w; m < M; m += kDsWarps) {
        // REF_QUIRK_Q1: the combine has no 1/2, unlike the X-step's (cdl_kernels.jl:30)
        const float2 h = STAGE ? cjfma(ys[m * kDsBins + lane], W, hs[m * kDsBins + lane])
                               : cjfma(Yh[base + (size_t)m * F], W, Hh[base + (size_t)m * F]);
        Dh[base + (size_t)m * F] = make_float2(h.x * scale_out, h.y * scale_out);
    }
    if (w == 0) Th[n * F + f] = make_float2(T.x * scale, T.y * scale);
}

size_t dsolve_smem(int M, bool stage) {
    return (stage ? (size_t)2 * M * kDsBins * sizeof(float2) : 0) +
           (size_t)kDsWarps * kDsBins * (4 + 8 + 8);
}

// launches k_dsolve for cn sequences, staging the spectra when they fit shared memory;
// the new d-hat replaces Dh, times scale_out
int dsolve_launch(cdlgb_ctx* c, int cn, const float2* Yh, const float2* Hh, float2* Dh,
                  const float2* Zh, float2* Th, float scale_out) {
    const int F = c->F, M = c->M;
    const int nfb = (F + kDsBins - 1) / kDsBins;
    const size_t sm = dsolve_smem(M, true);
    const bool stage = sm <= (size_t)200 * 1024;
    if (stage && sm > 48 * 1024)
        CU_TRY(c, cudaFuncSetAttribute(k_dsolve<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    const dim3 g((unsigned)((size_t)nfb * cn)), b(kDsBins * kDsWarps);
    const float scale = 1.f / (float)c->Lg;
    if (stage)
        k_dsolve<true><<<g, b, sm, c->stream>>>(Yh, Hh, Dh, Zh, Th, F, M, nfb, c->p.sherman_const_cdl,
                                                scale, scale_out);
    else
        k_dsolve<false><<<g, b, dsolve_smem(M, false), c->stream>>>(Yh, Hh, Dh, Zh, Th, F, M, nfb,
                                                                    c->p.sherman_const_cdl, scale,
                                                                    scale_out);
    LAUNCH_CHECK(c, "k_dsolve");
    return CDLGB_OK;
}

// G2' = (W'S + sigma (Td + g2)) / (W'W_ll + sigma)  (update_g2!, cdl_kernels.jl:68-77);
// g2' = g2 + Td - G2'  (train.jl:71)
__global__ void k_dg2(const float* __restrict__ Td, float* __restrict__ g2,
                      float* __restrict__ G2, const float* __restrict__ S, int Lg, int L4,
                      int gamma, size_t n, float sigma) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        size_t nn = i / Lg;
        int l = (int)(i - nn * Lg);
        bool in = l >= gamma && l < gamma + L4;
        float wts = in ? S[nn * L4 + (l - gamma)] : 0.f;
        float dg = in ? 1.f : 0.f;
        float t = Td[i], g = g2[i];
        float Gn = __fadd_rn(wts, __fmul_rn(sigma, t + g)) / (dg + sigma);
        G2[i] = Gn;
        g2[i] = (g + t) - Gn;
    }
}

// g1 += d - G1, g3 += d - G3 (train.jl:70,72) and per-chunk partial sums over sequences
// of (d + g3'), (d + g1') and d for the consensus means (train.jl:76,83; update_best! :95).
__global__ void k_dcons(const float4* __restrict__ d, float4* __restrict__ g1,
                        float4* __restrict__ g3, const float4* __restrict__ G1,
                        const float4* __restrict__ G3, float4* __restrict__ part, size_t pl4,
                        int N, int nchunk) {
    size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (j >= pl4) return;
    int ch = blockIdx.y;
    int n0 = (int)((int64_t)N * ch / nchunk), n1 = (int)((int64_t)N * (ch + 1) / nchunk);
    float4 A = G1[j], C = G3[j];
    float4 s1 = make_float4(0, 0, 0, 0), s3 = s1, sd = s1;
    for (int n = n0; n < n1; ++n) {
        size_t i = (size_t)n * pl4 + j;
        float4 dv = d[i], a = g1[i], b = g3[i];
        a = make_float4((a.x + dv.x) - A.x, (a.y + dv.y) - A.y, (a.z + dv.z) - A.z, (a.w + dv.w) - A.w);
        b = make_float4((b.x + dv.x) - C.x, (b.y + dv.y) - C.y, (b.z + dv.z) - C.z, (b.w + dv.w) - C.w);
        g1[i] = a;
        g3[i] = b;
        s1.x += dv.x + a.x; s1.y += dv.y + a.y; s1.z += dv.z + a.z; s1.w += dv.w + a.w;
        s3.x += dv.x + b.x; s3.y += dv.y + b.y; s3.z += dv.z + b.z; s3.w += dv.w + b.w;
        sd.x += dv.x; sd.y += dv.y; sd.z += dv.z; sd.w += dv.w;
    }
    part[((size_t)ch * 3 + 0) * pl4 + j] = s1;
    part[((size_t)ch * 3 + 1) * pl4 + j] = s3;
    part[((size_t)ch * 3 + 2) * pl4 + j] = sd;
}

// v1 = sum(d+g1)/N, v2 = sum(d+g3)/N, dmean = sum(d)/N;  G3 = projection2box!(v2)
// (cdl_kernels.jl:37-51); P_D = 1 on rows l < filter_len.
__global__ void k_dfinish(const float* __restrict__ part, float* __restrict__ v1,
                          float* __restrict__ G3, float* __restrict__ dmean, size_t pl,
                          int Lg, int flen, int N, int nchunk) {
    size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (j >= pl) return;
    double s1 = 0, s3 = 0, sd = 0;
    for (int ch = 0; ch < nchunk; ++ch) {
        s1 += part[((size_t)ch * 3 + 0) * pl + j];
        s3 += part[((size_t)ch * 3 + 1) * pl + j];
        sd += part[((size_t)ch * 3 + 2) * pl + j];
    }
    float a = (float)(s1 / N), b = (float)(s3 / N);
    v1[j] = a;
    dmean[j] = (float)(sd / N);
    int l = (int)(j % Lg);
    bool sup = l < flen;
    G3[j] = b >= 1.f ? (sup ? 1.f : 0.f) : (b <= 0.f ? 0.f : (sup ? b : 0.f));
}

// prox_simplex_zeros! (cdl_kernels.jl:53-66), group index as in the reference: for
// 1-based row l the group is rows i+1..i+4 with i = 4*floor(l/4) (REF_QUIRK_Q2: rows
// l = 4, 8, ... take the next group, cdl_kernels.jl:59).
__global__ void k_dprox(const float* __restrict__ v1, float* __restrict__ G1, int Lg, int M,
                        int flen) {
    size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (j >= (size_t)Lg * M) return;
    int l0 = (int)(j % Lg);
    size_t col = j - l0;
    float out = 0.f;
    if (l0 < flen) {
        int i = 4 * ((l0 + 1) / 4);
        const float* v = v1 + col;
        double grp = (double)v[i] + v[i + 1] + v[i + 2] + v[i + 3];
        out = (float)((double)v[l0] - 0.25 * (grp - 1.0));
    }
    G1[j] = out;
}

// ---------------------------------------------------------------- reductions
__device__ __forceinline__ double block_sum_d(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
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

__global__ void k_abssum(const float4* __restrict__ X, size_t n4, double* __restrict__ out) {
    __shared__ double sh[32];
    double acc = 0.0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4;
         i += (size_t)gridDim.x * blockDim.x) {
        float4 v = X[i];
        acc += (double)((fabsf(v.x) + fabsf(v.y)) + (fabsf(v.z) + fabsf(v.w)));
    }
    acc = block_sum_d(acc, sh);
    if (threadIdx.x == 0) out[blockIdx.x] = acc;
}

// The initial X in one pass (CDL_setup.jl:191-192): standard normal on the rows
// (l-1) % 4 == 0 and zero elsewhere.  Lg % 4 == 0, so those rows are the .x components
// of the float4s; element 4 j draws from counter 4 j of the seed's splitmix64 stream
// (Box-Muller on two 24-bit uniforms).  A given X0 is masked to the same rows instead.
// Also y2 = y3 = 0 (CDL_setup.jl:220-230) and the per-block sums of |X| for the initial
// objective.  Launched on k_abssum's grid (304 blocks of kBlock), so every thread visits
// k_abssum's indices in its order: the same sums, bit for bit.
__global__ void k_init_x(float4* __restrict__ X, float4* __restrict__ y2, float4* __restrict__ y3,
                         size_t n4, uint64_t seed, int draw, double* __restrict__ out) {
    __shared__ double sh[32];
    double acc = 0.0;
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < n4;
         j += (size_t)gridDim.x * blockDim.x) {
        float4 v;
        if (draw) {
            const uint64_t h = splitmix64(seed * 0x2545F4914F6CDD1Dull ^ (uint64_t)(4 * j));
            const float u1 = ((float)(h >> 40) + 0.5f) * (1.0f / 16777216.0f);
            const float u2 = ((float)(h & 0xFFFFFFull) + 0.5f) * (1.0f / 16777216.0f);
            v = make_float4(sqrtf(-2.f * logf(u1)) * cospif(2.f * u2), 0.f, 0.f, 0.f);
        } else {
            v = make_float4(X[j].x, 0.f, 0.f, 0.f);
        }
        X[j] = v;
        y2[j] = z;
        y3[j] = z;
        acc += (double)((fabsf(v.x) + fabsf(v.y)) + (fabsf(v.z) + fabsf(v.w)));
    }
    acc = block_sum_d(acc, sh);
    if (threadIdx.x == 0) out[blockIdx.x] = acc;
}

// sum over the data window of (DX - S)^2  (||W*DX - S||^2)
__global__ void k_fit(const float* __restrict__ DX, const float* __restrict__ S, int Lg, int L4,
                      int gamma, size_t n, double* __restrict__ out) {
    __shared__ double sh[32];
    double acc = 0.0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        size_t nn = i / L4;
        int j = (int)(i - nn * L4);
        double r = (double)DX[nn * Lg + gamma + j] - (double)S[i];
        acc += r * r;
    }
    acc = block_sum_d(acc, sh);
    if (threadIdx.x == 0) out[blockIdx.x] = acc;
}

// out[0] = 0.5 * sum(pb[0..nb2)) + lam * sum(pa[0..nb1))
__global__ void k_obj_final(const double* __restrict__ pa, int nb1, const double* __restrict__ pb,
                            int nb2, double lam, double* __restrict__ out) {
    __shared__ double sh[32];
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < nb1; i += blockDim.x) a += pa[i];
    for (int i = threadIdx.x; i < nb2; i += blockDim.x) b += pb[i];
    a = block_sum_d(a, sh);
    b = block_sum_d(b, sh);
    if (threadIdx.x == 0) out[0] = 0.5 * b + lam * a;
}

// std of the positive entries: pass 1 count + sum, pass 2 sum of squared deviations
__global__ void k_pos_stats(const float4* __restrict__ X, size_t n4, const double* __restrict__ mu,
                            double* __restrict__ out) {
    __shared__ double sh[32];
    double c = 0.0, s = 0.0;
    double m = mu ? mu[0] : 0.0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4;
         i += (size_t)gridDim.x * blockDim.x) {
        float4 v = X[i];
        float e[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (e[k] > 0.f) {
                if (mu) { double t = (double)e[k] - m; s += t * t; }
                else { c += 1.0; s += (double)e[k]; }
            }
    }
    c = block_sum_d(c, sh);
    s = block_sum_d(s, sh);
    if (threadIdx.x == 0) {
        out[2 * blockIdx.x] = c;
        out[2 * blockIdx.x + 1] = s;
    }
}

__global__ void k_pos_final(const double* __restrict__ part, int nb, double* __restrict__ out,
                            int second) {
    __shared__ double sh[32];
    double c = 0.0, s = 0.0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
        c += part[2 * i];
        s += part[2 * i + 1];
    }
    c = block_sum_d(c, sh);
    s = block_sum_d(s, sh);
    if (threadIdx.x == 0) {
        if (!second) { out[0] = c; out[1] = c > 0 ? s / c : 0.0; }
        else out[2] = out[0] > 1 ? sqrt(s / (out[0] - 1.0)) : nan("");
    }
}

// host-side seeded normal (used for D0 when none is given)
double host_normal(uint64_t seed, uint64_t i) {
    uint64_t h = splitmix64(seed * 0x2545F4914F6CDD1Dull ^ (i + 0x9E37ull));
    double u1 = ((double)(h >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    uint64_t h2 = splitmix64(h);
    double u2 = ((double)(h2 >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    return sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2);
}
double host_uniform(uint64_t seed, uint64_t i) {
    uint64_t h = splitmix64(seed * 0x9E3779B97F4A7C15ull ^ (i + 0x51ull));
    return ((double)(h >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

struct PlanEntry { int dir; long long batch; cufftHandle h; void* work; };
typedef std::vector<PlanEntry> PlanCache;

// R2C (dir 0) or C2R (dir 1) plan of length Lg over `batch` contiguous columns
int get_plan(cdlgb_ctx* c, int dir, long long batch, cufftHandle* out) {
    if (!c->plans) c->plans = new PlanCache();
    PlanCache& pc = *(PlanCache*)c->plans;
    for (auto& e : pc)
        if (e.dir == dir && e.batch == batch) { *out = e.h; return CDLGB_OK; }
    long long n[1] = {c->Lg}, in_r[1] = {c->Lg}, in_c[1] = {c->F};
    size_t ws = 0;
    cufftHandle h;
    FFT_TRY(c, cufftCreate(&h));
    // the work area comes from the context's stream-ordered allocations, not from cuFFT
    FFT_TRY(c, cufftSetAutoAllocation(h, 0));
    if (dir == 0)
        FFT_TRY(c, cufftMakePlanMany64(h, 1, n, in_r, 1, c->Lg, in_c, 1, c->F, CUFFT_R2C, batch, &ws));
    else
        FFT_TRY(c, cufftMakePlanMany64(h, 1, n, in_c, 1, c->F, in_r, 1, c->Lg, CUFFT_C2R, batch, &ws));
    void* work = nullptr;
    int st = dev_alloc(c, &work, ws);
    if (st != CDLGB_OK) { cufftDestroy(h); return st; }
    cufftResult r = work ? cufftSetWorkArea(h, work) : CUFFT_SUCCESS;
    if (r == CUFFT_SUCCESS) r = cufftSetStream(h, c->stream);
    if (r != CUFFT_SUCCESS) {
        cufftDestroy(h);
        dev_free(c, work);
        return cdlgb_seterr(c, CDLGB_ECUDA, "cuFFT plan of %lld rows: work area / stream, status %d",
                            batch, (int)r);
    }
    pc.push_back({dir, batch, h, work});
    *out = h;
    return CDLGB_OK;
}

int set_plan_streams(cdlgb_ctx* c) {
    if (!c->plans) return CDLGB_OK;
    for (auto& e : *(PlanCache*)c->plans) FFT_TRY(c, cufftSetStream(e.h, c->stream));
    return CDLGB_OK;
}

void free_plans(cdlgb_ctx* c) {
    if (!c->plans) return;
    for (auto& e : *(PlanCache*)c->plans) {
        cufftDestroy(e.h);
        dev_free(c, e.work);
    }
    delete (PlanCache*)c->plans;
    c->plans = nullptr;
}

// the register-FFT row kernels where the context's length has them (the streaming
// transforms' plan), else cuFFT
static void* row_plan(cdlgb_ctx* c) {
    return c->fused && !c->rows_cufft ? fused_dfwd(c) : nullptr;
}

// `grp`: the rows come in groups of grp that belong to one object (the M filter rows of
// a sequence: grp = M; one row per sequence: grp = 1).  The row kernels transform two
// rows as one complex FFT, whose rounding of either row depends on the other, so they
// pair rows only inside a group: a sequence's bits never depend on another sequence's
// data, which keeps every per-sequence result independent of N and of the batch.
int r2c(cdlgb_ctx* c, long long batch, float* in, float2* out, int grp) {
    if (void* rp = row_plan(c)) return rows_r2c(c, rp, (long)batch, in, out, grp);
    cufftHandle p;
    ST_TRY(get_plan(c, 0, batch, &p));
    FFT_TRY(c, cufftExecR2C(p, (cufftReal*)in, (cufftComplex*)out));
    c->fft_calls++;
    return CDLGB_OK;
}
int c2r(cdlgb_ctx* c, long long batch, float2* in, float* out, int grp) {
    if (void* rp = row_plan(c)) return rows_c2r(c, rp, (long)batch, in, out, grp);
    cufftHandle p;
    ST_TRY(get_plan(c, 1, batch, &p));
    FFT_TRY(c, cufftExecC2R(p, (cufftComplex*)in, (cufftReal*)out));
    c->fft_calls++;
    return CDLGB_OK;
}

// sequences per chunk of the cuFFT passes: the per-sequence scratch (two real and
// three half-spectrum (Lg, M) slices) times the chunk stays near 2 GiB
int chunk_for(int N, int M, int Lg) {
    size_t F = Lg / 2 + 1;
    size_t per = (size_t)M * (2 * (size_t)Lg * 4 + 3 * F * 8);
    size_t ch = ((size_t)2 << 30) / per;
    if (ch < 1) ch = 1;
    if (ch > (size_t)N) ch = N;
    return (int)ch;
}

// Sequences per chunk of the spectral D-step: its only scratch is the Y3 half-spectra
// (M x F complex per sequence), so a chunk covers up to 6 GB of them (the whole dataset
// at N = 20000, L = 200, K = 64), never fewer than the cuFFT passes' chunk.
int spec_chunk_for(int N, int M, int Lg) {
    size_t F = Lg / 2 + 1;
    size_t ch = ((size_t)6 << 30) / ((size_t)M * F * 8);
    ch = std::max(ch, (size_t)chunk_for(N, M, Lg));
    if (ch > (size_t)N) ch = N;
    return (int)ch;
}

int device_sms() {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) {
        cudaGetLastError();
        return 152;
    }
    return sms;
}

// G1h = rfft(G1) and A = sum_m |G1h|^2
int refresh_G1h(cdlgb_ctx* c) {
    ST_TRY(r2c(c, c->M, c->G1, c->G1h, c->M));
    k_colnorm<<<(c->F + 127) / 128, 128, 0, c->stream>>>(c->G1h, c->Ah, c->F, c->M);
    LAUNCH_CHECK(c, "k_colnorm");
    return CDLGB_OK;
}

float* cur_X(cdlgb_ctx* c) { return c->Xb[c->xcur]; }

}  // namespace

// ============================================================================ API-level
// The D-step keeps d, g1, g3 as half-spectra (dspec.cu) on the fused path and on the
// automatically chosen cuFFT-transform path (not when cuFFT transforms are asked for
// explicitly, the form kept next to the reference's own), for M up to dspec_max_m();
// CDLGB_DSPEC=0 keeps them in the time domain.  With the spectral state, the
// time-domain d, g1, g3 are only a reader's copy, allocated at the first read.
bool spectral_state(const cdlgb_params* p, int fused) {
    if (p->M > dspec_max_m() || (!fused && p->fft_mode != 0)) return false;
    const char* e = getenv("CDLGB_DSPEC");
    return !e || atoi(e) != 0;
}

size_t admm_footprint(const cdlgb_params* p, int L4, int N, int fused) {
    size_t gamma = 4 * (size_t)p->filter_size, Lg = L4 + 2 * gamma, F = Lg / 2 + 1;
    size_t M = p->M, LMN = Lg * M * N, LN = Lg * N, LM = Lg * M;
    const bool spec = spectral_state(p, fused);
    size_t b = 0;
    b += (size_t)N * L4 * 4;                    // data
    b += 4 * LMN * 4;                           // X x2, y2, y3
    if (!spec) b += 3 * LMN * 4;                // d, g1, g3 (time-domain D-step)
    if (fused || spec) b += (size_t)N * M * F * 8;   // d-hat
    if (spec) b += (size_t)N * M * F * 8;            // g1-hat
    if (spec) {
        // spectral D-step: the sums' slots and the Y3 half-spectra beyond the cuFFT chunk
        const size_t sch = spec_chunk_for(N, (int)M, (int)Lg), ch = chunk_for(N, (int)M, (int)Lg);
        b += (size_t)dspec_slots(N, (int)sch, (int)F, device_sms()) * 2 * M * F * 8;
        b += (sch - ch) * M * F * 8;
    }
    b += 8 * LN * 4;                            // Y1 y1 DX Td G2 g2 + 2 scratch
    b += 8 * LM * 4 + M * F * 8 + F * 4;        // G1 G3 dmean Dbest v1 ... G1h A
    b += 2 * N * F * 8;                         // LN spectra
    if (fused) b += fused_scratch_bytes((int)Lg, (int)M, N);
    size_t ch = chunk_for(N, (int)M, (int)Lg);
    b += ch * M * (2 * Lg * 4 + 3 * F * 8);             // cuFFT-path scratch, one chunk
    b += ch * M * Lg * 4;                               // cuFFT work area (estimate)
    b += 64ull * 3 * LM * 4;                    // D-step partials
    b += resid_part_doubles(N, (int)F, 1 << 16) * 8 + 2 * LM * 4;   // residual partials, G_old
    b += (64u << 20);                           // reductions, scan scratch, slack
    return b;
}

int admm_alloc(cdlgb_ctx* c) {
    const size_t LMN = c->LMN, LN = c->LN, LM = c->LM;
    auto A = [&](void** p, size_t bytes) -> int { return dev_alloc(c, p, bytes); };
    ST_TRY(A((void**)&c->Xb[0], LMN * 4));
    ST_TRY(A((void**)&c->Xb[1], LMN * 4));
    ST_TRY(A((void**)&c->y2, LMN * 4));
    ST_TRY(A((void**)&c->y3, LMN * 4));
    const bool spec = spectral_state(&c->p, c->fused);
    if (!spec) {
        ST_TRY(A((void**)&c->d, LMN * 4));
        ST_TRY(A((void**)&c->g1, LMN * 4));
        ST_TRY(A((void**)&c->g3, LMN * 4));
    }
    // the previous D-step's d-hat (N, M, F) complex (the fused path's time-domain
    // D-step keeps it too); with the spectral D-step also g1-hat (g3-hat is g1-hat
    // minus one shared spectrum), G3-hat and the sums' spectra
    if (c->fused || spec) {
        const size_t nmf = (size_t)c->N * c->M * c->F;
        ST_TRY(A((void**)&c->Dhs, nmf * 8));
        if (spec) {
            ST_TRY(A((void**)&c->g1h, nmf * 8));
            ST_TRY(A((void**)&c->Dg, (size_t)c->M * c->F * 8));
            ST_TRY(A((void**)&c->G3h, (size_t)c->M * c->F * 8));
            ST_TRY(A((void**)&c->sumspec, (size_t)3 * c->M * c->F * 8));
        }
    }
    c->dh_valid = 0;
    c->dspec = 0;
    c->time_stale = 0;
    ST_TRY(A((void**)&c->Y1, LN * 4));
    ST_TRY(A((void**)&c->y1, LN * 4));
    ST_TRY(A((void**)&c->DX, LN * 4));
    ST_TRY(A((void**)&c->Td, LN * 4));
    ST_TRY(A((void**)&c->G2, LN * 4));
    ST_TRY(A((void**)&c->g2, LN * 4));
    ST_TRY(A((void**)&c->sU, LN * 4));
    ST_TRY(A((void**)&c->G1, LM * 4));
    ST_TRY(A((void**)&c->G3, LM * 4));
    ST_TRY(A((void**)&c->dsum, LM * 4));
    ST_TRY(A((void**)&c->Dbest, LM * 4));
    ST_TRY(A((void**)&c->vbar, LM * 4));
    ST_TRY(A((void**)&c->G1h, (size_t)c->M * c->F * 8));
    ST_TRY(A((void**)&c->Ah, (size_t)c->F * 4));
    ST_TRY(A((void**)&c->sUh, (size_t)c->N * c->F * 8));
    ST_TRY(A((void**)&c->sVh, (size_t)c->N * c->F * 8));
    // cuFFT-path scratch for one chunk of sequences (init's DX, the D-step, and the
    // X-step when no fused kernel covers Lg)
    c->chunk = chunk_for(c->N, c->M, c->Lg);
    c->schunk = c->chunk;
    c->nsm = device_sms();
    if (c->g1h) {
        c->schunk = spec_chunk_for(c->N, c->M, c->Lg);
        c->dslots = dspec_slots(c->N, c->schunk, c->F, c->nsm);
        ST_TRY(A((void**)&c->spart, dspec_part_bytes(c->M, c->F, c->dslots)));
    }
    const size_t cLMN = (size_t)c->chunk * c->M * c->Lg, cSp = (size_t)c->chunk * c->M * c->F;
    ST_TRY(A((void**)&c->sA, cLMN * 4));
    // the first Y3-hat scratch also holds a chunk of the spectral D-step
    ST_TRY(A((void**)&c->sAh, (size_t)c->schunk * c->M * c->F * 8));
    ST_TRY(A((void**)&c->sB, cLMN * 4));
    ST_TRY(A((void**)&c->sBh, cSp * 8));
    ST_TRY(A((void**)&c->sCh, cSp * 8));
    c->nchunk = std::max(1, std::min(64, c->N));
    ST_TRY(A((void**)&c->part, (size_t)c->nchunk * 3 * LM * 4));
    c->nred = 152 * 4;
    ST_TRY(A((void**)&c->dred, (size_t)c->nred * 4 * sizeof(double)));
    ST_TRY(A((void**)&c->dscalar, 8 * sizeof(double)));
    c->hscalar = host_scalars_get();
    c->hscalar_own = false;
    if (!c->hscalar) {
        CU_TRY(c, cudaMallocHost((void**)&c->hscalar, 8 * sizeof(double)));
        c->hscalar_own = true;
    }
    ST_TRY(A((void**)&c->dres, RESIDUAL_COUNT * sizeof(double)));
    ST_TRY(A((void**)&c->rpart, resid_part_doubles(c->N, c->F, c->dslots) * sizeof(double)));
    ST_TRY(A((void**)&c->Gprev, 2 * LM * 4));
    return CDLGB_OK;
}

void admm_free(cdlgb_ctx* c) {
    float** fl[] = {&c->Xb[0], &c->Xb[1], &c->y2, &c->y3, &c->d, &c->g1, &c->g3, &c->Y1,
                    &c->y1, &c->DX, &c->Td, &c->G2, &c->g2, &c->sU, &c->G1, &c->G3,
                    &c->dsum, &c->Dbest, &c->vbar, &c->Ah, &c->sA, &c->sB, &c->part};
    for (auto p : fl) { dev_free(c, *p); *p = nullptr; }
    float2** cl[] = {&c->G1h, &c->sUh, &c->sVh, &c->sAh, &c->sBh, &c->sCh, &c->Dhs,
                     &c->g1h, &c->Dg, &c->G3h, &c->spart, &c->sumspec};
    for (auto p : cl) { dev_free(c, *p); *p = nullptr; }
    dev_free(c, c->dred);
    dev_free(c, c->dscalar);
    if (c->hscalar) {
        // the slot may still be the target of a copy in flight on the stream
        cudaStreamSynchronize(c->stream);
        if (c->hscalar_own) cudaFreeHost(c->hscalar);
        else host_scalars_put(c->hscalar);
    }
    dev_free(c, c->dres);
    dev_free(c, c->rpart);
    dev_free(c, c->Gprev);
    c->dred = nullptr; c->dscalar = nullptr; c->hscalar = nullptr;
    c->dres = nullptr; c->rpart = nullptr; c->Gprev = nullptr;
    free_plans(c);
}

int cdlgb_set_plan_streams(cdlgb_ctx* c) { return set_plan_streams(c); }

// the time-domain d, g1, g3 of the spectral form, allocated at their first reader
static int ensure_time_state(cdlgb_ctx* c) {
    for (float** p : {&c->d, &c->g1, &c->g3})
        if (!*p) ST_TRY(dev_alloc(c, (void**)p, c->LMN * 4));
    return CDLGB_OK;
}

// the initial time-domain dictionary state: d = G1 broadcast over n, g1 = g3 = 0
static int write_time_init(cdlgb_ctx* c) {
    const size_t LMN = c->LMN;
    ST_TRY(ensure_time_state(c));
    k_bcast_plane<<<grid_for(LMN / 4, kBlock), kBlock, 0, c->stream>>>(
        (float4*)c->d, (const float4*)c->G1, c->LM / 4, LMN / 4);
    LAUNCH_CHECK(c, "k_bcast_plane");
    CU_TRY(c, cudaMemsetAsync(c->g1, 0, LMN * 4, c->stream));
    CU_TRY(c, cudaMemsetAsync(c->g3, 0, LMN * 4, c->stream));
    c->time_init = 0;
    return CDLGB_OK;
}

int admm_init(cdlgb_ctx* c, const float* X0, const float* D0, uint64_t seed) {
    cudaStream_t s = c->stream;
    const int Lg = c->Lg, M = c->M, N = c->N, flen = 4 * c->p.filter_size;
    const size_t LMN = c->LMN, LN = c->LN, LM = c->LM;
    c->xcur = 0;
    c->best_is_cur = 1;
    c->absx_fused = 0;
    c->dh_valid = 0;
    c->outer_done = 0;
    CU_TRY(c, cudaMemsetAsync(c->dres, 0, RESIDUAL_COUNT * sizeof(double), c->stream));
    float* X = c->Xb[0];
    // X0 (CDL_setup.jl:191-192): given, or standard normal; masked to the 4-stride; with
    // y2 = y3 = 0 and sum |X| for the initial objective in the same pass
    if (X0) CU_TRY(c, cudaMemcpyAsync(X, X0, LMN * 4, cudaMemcpyHostToDevice, s));
    k_init_x<<<152 * 2, kBlock, 0, s>>>((float4*)X, (float4*)c->y2, (float4*)c->y3, LMN / 4, seed,
                                        X0 ? 0 : 1, c->dred);
    LAUNCH_CHECK(c, "k_init_x");
    // the spectral D-step (dspec.cu) where its transforms cover Lg and M
    c->dspec = 0;
    c->time_stale = 0;
    c->time_init = 0;
    if (c->g1h) c->dspec = 1;                 // spectral_state() held at allocation
    // D0 (CDL_setup.jl:182-183), masked by P_D
    std::vector<float> D(LM, 0.f);
    if (D0) {
        for (int m = 0; m < M; ++m)
            for (int l = 0; l < flen; ++l) D[(size_t)m * Lg + l] = D0[(size_t)m * Lg + l];
    } else if (c->p.init_mode == 1) {
        // the reference's draw: per 4-row group a uniform point on the simplex
        uint64_t ctr = 0;
        for (int m = 0; m < M; ++m)
            for (int g = 0; g < flen / 4; ++g) {
                double u[3];
                for (int k = 0; k < 3; ++k) u[k] = host_uniform(seed, ctr++);
                std::sort(u, u + 3);
                double w[5] = {0, u[0], u[1], u[2], 1};
                for (int k = 0; k < 4; ++k) D[(size_t)m * Lg + 4 * g + k] = (float)(w[k + 1] - w[k]);
            }
    } else {
        uint64_t ctr = 0;
        for (int m = 0; m < M; ++m) {
            double nrm = 0;
            std::vector<double> v(flen);
            for (int l = 0; l < flen; ++l) { v[l] = host_normal(seed, ctr++); nrm += v[l] * v[l]; }
            nrm = sqrt(nrm);
            for (int l = 0; l < flen; ++l) D[(size_t)m * Lg + l] = (float)(v[l] / nrm);
        }
    }
    CU_TRY(c, cudaMemcpyAsync(c->G1, D.data(), LM * 4, cudaMemcpyHostToDevice, s));
    CU_TRY(c, cudaMemcpyAsync(c->G3, c->G1, LM * 4, cudaMemcpyDeviceToDevice, s));
    CU_TRY(c, cudaMemcpyAsync(c->Dbest, c->G1, LM * 4, cudaMemcpyDeviceToDevice, s));
    CU_TRY(c, cudaMemcpyAsync(c->dsum, c->G1, LM * 4, cudaMemcpyDeviceToDevice, s));
    // d = real(ifft(d-hat)) with d-hat = D-hat broadcast (CDL_setup.jl:207-210); the duals
    // g1, g3 start at zero (CDL_setup.jl:220-230).  In the spectral form nothing reads
    // these time-domain arrays before a D-step replaces them: written when first read.
    if (c->dspec) {
        c->time_init = 1;
    } else {
        ST_TRY(write_time_init(c));
    }
    // Y1 and the LN duals start at zero
    CU_TRY(c, cudaMemsetAsync(c->Y1, 0, LN * 4, s));
    CU_TRY(c, cudaMemsetAsync(c->y1, 0, LN * 4, s));
    CU_TRY(c, cudaMemsetAsync(c->g2, 0, LN * 4, s));
    CU_TRY(c, cudaMemsetAsync(c->Td, 0, LN * 4, s));
    ST_TRY(refresh_G1h(c));
    // spectral D-step: d-hat = D-hat broadcast, g1-hat = g3-hat = 0
    if (c->dspec) {
        const size_t nmf = (size_t)N * M * c->F;
        ST_TRY(dspec_bcast(c, c->Dhs, c->G1h));
        CU_TRY(c, cudaMemsetAsync(c->g1h, 0, nmf * 8, s));
        CU_TRY(c, cudaMemsetAsync(c->Dg, 0, (size_t)M * c->F * 8, s));
    }
    // DX = real(ifft(sum_m D-hat .* X-hat)) (CDL_setup.jl:197-203); G2 = DX
    for (int n0 = 0; n0 < N; n0 += c->chunk) {
        const int cn = std::min(c->chunk, N - n0);
        ST_TRY(r2c(c, (long long)M * cn, X + (size_t)n0 * M * Lg, c->sAh, M));
        size_t FN = (size_t)c->F * cn;
        k_spec_dot<<<(unsigned)((FN + 255) / 256), 256, 0, s>>>(c->sAh, c->G1h, c->sVh + (size_t)n0 * c->F,
                                                              c->F, M, cn, 1.f / (float)Lg);
        LAUNCH_CHECK(c, "k_spec_dot");
    }
    ST_TRY(c2r(c, N, c->sVh, c->DX, 1));
    CU_TRY(c, cudaMemcpyAsync(c->G2, c->DX, LN * 4, cudaMemcpyDeviceToDevice, s));
    c->initialized = true;
    double obj = 0;
    c->absx_init = 1;           // dred[0, 304) = k_init_x's sums of |X|, consumed here
    ST_TRY(admm_objective(c, &obj));
    c->obj_best = obj;
    return CDLGB_OK;
}

int admm_code_update(cdlgb_ctx* c, int iters) {
    cudaStream_t s = c->stream;
    const size_t LN = c->LN;
    const int F = c->F, M = c->M, N = c->N;
    if (iters > 0 && c->fused && fused_has_multi(c)) {
        // all iterations in one launch, the state on chip in between
        cdlgb_phase_begin(c, PH_XSTEP);
        float* Xin = cur_X(c);
        float* Xout = c->best_is_cur ? c->Xb[1 - c->xcur] : Xin;
        ST_TRY(fused_xsteps(c, Xin, Xout, iters));
        c->absx_fused = 1;
        if (Xout != Xin) {
            c->xcur = 1 - c->xcur;
            c->best_is_cur = 0;
        }
        // the residuals of the final iterate, from the kernel's store pass
        const double* rp = nullptr;
        int nr = 0;
        if (c->res_on) {
            if (fused_resid(c, &rp, &nr)) ST_TRY(resid_x_from_parts(c, rp, nr));
            else ST_TRY(resid_x_from_arrays(c, cur_X(c)));
        }
        cdlgb_phase_end_n(c, PH_XSTEP, iters);
        return CDLGB_OK;
    }
    for (int it = 0; it < iters; ++it) {
        cdlgb_phase_begin(c, PH_XSTEP);
        // X_best aliases the current buffer: write the new X into the other one
        float* Xin = cur_X(c);
        float* Xout = c->best_is_cur ? c->Xb[1 - c->xcur] : Xin;
        if (c->fused) {
            ST_TRY(fused_xstep(c, Xin, Xout, 0));
            c->absx_fused = 1;
        } else {
            c->absx_fused = 0;
            const int Lg = c->Lg;
            k_xprep_ln<<<grid_for(LN, kBlock), kBlock, 0, s>>>(c->y1, c->DX, c->Y1, c->sU, LN);
            LAUNCH_CHECK(c, "k_xprep_ln");
            ST_TRY(r2c(c, N, c->sU, c->sUh, 1));
            const int nfb = (F + 127) / 128;
            for (int n0 = 0; n0 < N; n0 += c->chunk) {
                const int cn = std::min(c->chunk, N - n0);
                const size_t off = (size_t)n0 * M * Lg, cl = (size_t)cn * M * Lg;
                k_xprep<<<grid_for(cl / 4, kBlock), kBlock, 0, s>>>(
                    (const float4*)(Xin + off), (float4*)(c->y2 + off), (float4*)(c->y3 + off),
                    (float4*)c->sA, cl / 4, c->p.lambda);
                LAUNCH_CHECK(c, "k_xprep");
                ST_TRY(r2c(c, (long long)M * cn, c->sA, c->sAh, M));
                k_xsolve<<<(unsigned)((size_t)nfb * cn), 128, 0, s>>>(
                    c->sAh, c->sUh + (size_t)n0 * F, c->G1h, c->Ah, c->sVh + (size_t)n0 * F, F, M, nfb,
                    c->p.sherman_const_csc, 1.f / (float)Lg);
                LAUNCH_CHECK(c, "k_xsolve");
                ST_TRY(c2r(c, (long long)M * cn, c->sAh, Xout + off, M));
            }
            ST_TRY(c2r(c, N, c->sVh, c->DX, 1));
            k_mask_update<<<grid_for(LN, kBlock), kBlock, 0, s>>>(c->Y1, c->DX, c->y1, c->S, c->Lg,
                                                                 c->L4, c->gamma, LN, c->p.rho);
            LAUNCH_CHECK(c, "k_mask_update");
        }
        if (Xout != Xin) {
            c->xcur = 1 - c->xcur;
            c->best_is_cur = 0;
        }
        if (c->res_on && it == iters - 1) ST_TRY(resid_x_from_arrays(c, cur_X(c)));
        cdlgb_phase_end(c, PH_XSTEP);
    }
    return CDLGB_OK;
}

int admm_dict_update(cdlgb_ctx* c, int iters) {
    cudaStream_t s = c->stream;
    const size_t LN = c->LN, LM = c->LM;
    const int F = c->F, M = c->M, N = c->N, Lg = c->Lg;
    for (int it = 0; it < iters; ++it) {
        cdlgb_phase_begin(c, PH_DSTEP);
        if (c->dspec) {
            // the state in the frequency domain: only Y3 is transformed (dspec.cu)
            k_sub<<<grid_for(LN, kBlock), kBlock, 0, s>>>(c->G2, c->g2, c->sU, LN);
            LAUNCH_CHECK(c, "k_sub");
            ST_TRY(r2c(c, N, c->sU, c->sUh, 1));
            ST_TRY(r2c(c, M, c->G3, c->G3h, M));
            void* fw = fused_dfwd(c);
            int slot0 = 0;
            for (int n0 = 0; n0 < N; n0 += c->schunk) {
                const int cn = std::min(c->schunk, N - n0);
                if (fw) {
                    ST_TRY(dfwd_run(c, fw, cur_X(c), n0, cn, c->sAh, nullptr, nullptr));
                } else {
                    // lengths without the streaming transforms: Y3 formed in the time
                    // domain and transformed, a cuFFT chunk at a time
                    for (int m0 = n0; m0 < n0 + cn; m0 += c->chunk) {
                        const int cm = std::min(c->chunk, n0 + cn - m0);
                        const size_t cl = (size_t)cm * M * Lg;
                        k_y3<<<grid_for(cl / 4, kBlock), kBlock, 0, s>>>(
                            (const float4*)(cur_X(c) + (size_t)m0 * M * Lg), (float4*)c->sA, cl / 4);
                        LAUNCH_CHECK(c, "k_y3");
                        ST_TRY(r2c(c, (long long)M * cm, c->sA, c->sAh + (size_t)(m0 - n0) * M * F, M));
                    }
                }
                ST_TRY(dspec_launch(c, c->sAh, c->G3h, n0, n0 + cn, slot0));
                slot0 += dspec_nsub(cn, F, c->nsm);
            }
            if (c->res_on) ST_TRY(resid_d_from_spec_parts(c, slot0 * ((F + 31) / 32)));
            ST_TRY(c2r(c, N, c->sVh, c->Td, 1));
            k_dg2<<<grid_for(LN, kBlock), kBlock, 0, s>>>(c->Td, c->g2, c->G2, c->S, Lg, c->L4,
                                                         c->gamma, LN, c->p.sigma);
            LAUNCH_CHECK(c, "k_dg2");
            if (c->res_on) ST_TRY(resid_td(c));
            // the three sums over n, back in the time domain: part as one chunk
            ST_TRY(dspec_sums(c, c->G3h, c->sumspec));
            ST_TRY(c2r(c, 3LL * M, c->sumspec, c->part, 3 * M));
            c->time_stale = 1;
            c->time_init = 0;
            int flen = 4 * c->p.filter_size;
            if (c->res_on) ST_TRY(resid_save_G(c));
            k_dfinish<<<(unsigned)((LM + 255) / 256), 256, 0, s>>>(c->part, c->vbar, c->G3, c->dsum,
                                                                   LM, Lg, flen, N, 1);
            LAUNCH_CHECK(c, "k_dfinish");
            k_dprox<<<(unsigned)((LM + 255) / 256), 256, 0, s>>>(c->vbar, c->G1, Lg, M, flen);
            LAUNCH_CHECK(c, "k_dprox");
            if (c->res_on) ST_TRY(resid_dual_and_finish(c));
            ST_TRY(refresh_G1h(c));
            cdlgb_phase_end(c, PH_DSTEP);
            continue;
        }
        {
            k_sub<<<grid_for(LN, kBlock), kBlock, 0, s>>>(c->G2, c->g2, c->sU, LN);
            LAUNCH_CHECK(c, "k_sub");
            ST_TRY(r2c(c, N, c->sU, c->sUh, 1));
            void* fw = c->fused && c->Dhs ? fused_dfwd(c) : nullptr;
            for (int n0 = 0; n0 < N; n0 += c->chunk) {
                const int cn = std::min(c->chunk, N - n0);
                const size_t off = (size_t)n0 * M * Lg, cl = (size_t)cn * M * Lg;
                if (fw) {
                    // Y3 and H formed and transformed in one streaming pass; rfft(d_old)
                    // is the previous D-step's d-hat, kept in Dhs (transformed from d
                    // only when there is none)
                    float2* Dh = c->Dhs + (size_t)n0 * M * F;
                    ST_TRY(dfwd_run(c, fw, cur_X(c), n0, cn, c->sAh, c->sBh, c->dh_valid ? nullptr : Dh));
                    ST_TRY(dsolve_launch(c, cn, c->sAh, c->sBh, Dh, c->sUh + (size_t)n0 * F,
                                         c->sVh + (size_t)n0 * F, 1.f));
                    ST_TRY(dinv_run(c, fw, Dh, n0, cn, 1.f / (float)Lg));
                } else {
                    k_dprep<<<grid_for(cl / 4, kBlock), kBlock, 0, s>>>(
                        (const float4*)(cur_X(c) + off), (const float4*)(c->y3 + off),
                        (const float4*)(c->g1 + off), (const float4*)(c->g3 + off),
                        (const float4*)c->G1, (const float4*)c->G3, (float4*)c->sA, (float4*)c->sB,
                        cl / 4, LM / 4);
                    LAUNCH_CHECK(c, "k_dprep");
                    ST_TRY(r2c(c, (long long)M * cn, c->sA, c->sAh, M));
                    ST_TRY(r2c(c, (long long)M * cn, c->sB, c->sBh, M));
                    ST_TRY(r2c(c, (long long)M * cn, c->d + off, c->sCh, M));
                    ST_TRY(dsolve_launch(c, cn, c->sAh, c->sBh, c->sCh, c->sUh + (size_t)n0 * F,
                                         c->sVh + (size_t)n0 * F, 1.f / (float)Lg));
                    ST_TRY(c2r(c, (long long)M * cn, c->sCh, c->d + off, M));
                }
            }
            c->dh_valid = fw != nullptr;
            ST_TRY(c2r(c, N, c->sVh, c->Td, 1));
            k_dg2<<<grid_for(LN, kBlock), kBlock, 0, s>>>(c->Td, c->g2, c->G2, c->S, Lg, c->L4,
                                                         c->gamma, LN, c->p.sigma);
            LAUNCH_CHECK(c, "k_dg2");
            size_t pl4 = LM / 4;
            dim3 g((unsigned)((pl4 + 255) / 256), (unsigned)c->nchunk);
            k_dcons<<<g, 256, 0, s>>>((const float4*)c->d, (float4*)c->g1, (float4*)c->g3,
                                      (const float4*)c->G1, (const float4*)c->G3,
                                      (float4*)c->part, pl4, N, c->nchunk);
            LAUNCH_CHECK(c, "k_dcons");
            if (c->res_on) {
                ST_TRY(resid_td(c));
                ST_TRY(resid_d_from_arrays(c));
            }
        }
        int flen = 4 * c->p.filter_size;
        if (c->res_on) ST_TRY(resid_save_G(c));
        k_dfinish<<<(unsigned)((LM + 255) / 256), 256, 0, s>>>(c->part, c->vbar, c->G3, c->dsum,
                                                               LM, Lg, flen, N, c->nchunk);
        LAUNCH_CHECK(c, "k_dfinish");
        k_dprox<<<(unsigned)((LM + 255) / 256), 256, 0, s>>>(c->vbar, c->G1, Lg, M, flen);
        LAUNCH_CHECK(c, "k_dprox");
        if (c->res_on) ST_TRY(resid_dual_and_finish(c));
        ST_TRY(refresh_G1h(c));
        cdlgb_phase_end(c, PH_DSTEP);
    }
    return CDLGB_OK;
}

// objective into c->dscalar[0] (device), no host sync
static int objective_async(cdlgb_ctx* c) {
    cudaStream_t s = c->stream;
    int nb1 = 152 * 2, nb2 = 152;
    const double* pa = c->dred;
    const double* fp = nullptr;
    int nf = 0;
    if (c->absx_init) {
        // sum |X| came with the initial X (k_init_x)
        c->absx_init = 0;
    } else if (c->absx_fused && fused_absx(c, &fp, &nf)) {
        // sum |X| came with the last fused X-step
        pa = fp;
        nb1 = nf;
    } else {
        k_abssum<<<nb1, kBlock, 0, s>>>((const float4*)cur_X(c), c->LMN / 4, c->dred);
        LAUNCH_CHECK(c, "k_abssum");
    }
    k_fit<<<nb2, kBlock, 0, s>>>(c->DX, c->S, c->Lg, c->L4, c->gamma, (size_t)c->N * c->L4,
                                 c->dred + 152 * 2);
    LAUNCH_CHECK(c, "k_fit");
    k_obj_final<<<1, kBlock, 0, s>>>(pa, nb1, c->dred + 152 * 2, nb2, (double)c->p.lambda,
                                     c->dscalar);
    LAUNCH_CHECK(c, "k_obj_final");
    return CDLGB_OK;
}

int admm_objective(cdlgb_ctx* c, double* obj) {
    cdlgb_phase_begin(c, PH_OBJ);
    ST_TRY(objective_async(c));
    CU_TRY(c, cudaMemcpyAsync(c->hscalar, c->dscalar, sizeof(double), cudaMemcpyDeviceToHost,
                              c->stream));
    cdlgb_phase_end(c, PH_OBJ);
    CU_TRY(c, cudaStreamSynchronize(c->stream));
    *obj = c->hscalar[0];
    return CDLGB_OK;
}

int admm_update_best(cdlgb_ctx* c, double* obj, int* improved) {
    double o = 0;
    ST_TRY(admm_objective(c, &o));
    int imp = o < c->obj_best;
    if (imp) {
        c->obj_best = o;
        // D_best = sum(d, dims=3) / N (train.jl:95), kept up to date by the D-step;
        // X_best = copy(X) (:96) becomes an alias of the current X buffer.
        CU_TRY(c, cudaMemcpyAsync(c->Dbest, c->dsum, c->LM * 4, cudaMemcpyDeviceToDevice,
                                  c->stream));
        c->best_is_cur = 1;
    }
    if (obj) *obj = o;
    if (improved) *improved = imp;
    return CDLGB_OK;
}

int admm_code_threshold(cdlgb_ctx* c, double* thr) {
    cudaStream_t s = c->stream;
    const float* Xbest = c->best_is_cur ? c->Xb[c->xcur] : c->Xb[1 - c->xcur];
    int nb = 152 * 2;
    k_pos_stats<<<nb, kBlock, 0, s>>>((const float4*)Xbest, c->LMN / 4, nullptr, c->dred);
    LAUNCH_CHECK(c, "k_pos_stats");
    k_pos_final<<<1, kBlock, 0, s>>>(c->dred, nb, c->dscalar, 0);
    LAUNCH_CHECK(c, "k_pos_final");
    k_pos_stats<<<nb, kBlock, 0, s>>>((const float4*)Xbest, c->LMN / 4, c->dscalar + 1, c->dred);
    LAUNCH_CHECK(c, "k_pos_stats");
    k_pos_final<<<1, kBlock, 0, s>>>(c->dred, nb, c->dscalar, 1);
    LAUNCH_CHECK(c, "k_pos_final");
    CU_TRY(c, cudaMemcpyAsync(c->hscalar, c->dscalar, 3 * sizeof(double), cudaMemcpyDeviceToHost, s));
    CU_TRY(c, cudaStreamSynchronize(s));
    *thr = c->hscalar[2] * (double)c->p.std_threshold_multiplier;
    return CDLGB_OK;
}

// d, g1, g3 in the time domain from the spectral state (for readers of those fields);
// the spectra are copied to scratch first (the inverse transform may overwrite its input)
int admm_sync_time_state(cdlgb_ctx* c) {
    if (!c->dspec) return CDLGB_OK;
    if (c->time_init) return write_time_init(c);    // no D-step since the initialisation
    if (!c->time_stale) return CDLGB_OK;
    ST_TRY(ensure_time_state(c));
    const int M = c->M, Lg = c->Lg, F = c->F;
    const float2* src[3] = {c->Dhs, c->g1h, c->g1h};
    float* dst[3] = {c->d, c->g1, c->g3};
    for (int q = 0; q < 3; ++q)
        for (int n0 = 0; n0 < c->N; n0 += c->chunk) {
            const int cn = std::min(c->chunk, c->N - n0);
            const size_t sp = (size_t)cn * M * F, tp = (size_t)cn * M * Lg;
            const float2* sq = src[q] + (size_t)n0 * M * F;
            if (q == 2) {
                ST_TRY(dspec_g3(c, c->sAh, sq, (size_t)cn * M));       // g3 = g1 - Dg
            } else {
                CU_TRY(c, cudaMemcpyAsync(c->sAh, sq, sp * 8, cudaMemcpyDeviceToDevice, c->stream));
            }
            ST_TRY(c2r(c, (long long)M * cn, c->sAh, dst[q] + (size_t)n0 * M * Lg, M));
            ST_TRY(dspec_scale(c, dst[q] + (size_t)n0 * M * Lg, tp, 1.f / (float)Lg));
        }
    c->time_stale = 0;
    return CDLGB_OK;
}
