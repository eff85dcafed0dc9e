// The D-step with the per-sequence dictionary state held as half-spectra.
//
// dict_update! (src/CDL/train.jl:46-89) transforms Y3, H = (G1 - g1) + (G3 - g3) and d to
// the frequency domain, solves per frequency, returns d to the time domain, updates the
// duals g1 += d - G1 and g3 += d - G3 (:70, :72) and averages d + g1, d + g3 and d over
// the sequences (:76, :83; and D_best, :91-98).  Every one of those steps after the
// solve is linear, and nothing outside the D-step reads d, g1 or g3.  So they are kept
// as half-spectra, with one more reduction:
//   * g1 and g3 start at zero and both receive the same d; their difference changes by
//     G3 - G1, the same for every sequence.  So g1 - g3 is one (M, F) spectrum Dg shared
//     by all sequences, and g3 = g1 - Dg: only d-hat and g1-hat are per sequence;
//   * H-hat = (G1-hat - g1-hat) + (G3-hat - g3-hat) with g3-hat = g1-hat - Dg, the duals
//     g1-hat += d-hat - G1-hat and Dg += G3-hat - G1-hat, and the averages of d + g1 and
//     d (that of d + g3 is the first minus Dg) are (M, F) spectra, returned to the time
//     domain once per D-step for the projections.  A D-step then transforms only Y3.
// The reference's statements applied to the transforms, with g3 recovered from the
// shared difference; results differ from the time-domain path by FP32 rounding.
#include "cdlgb_internal.h"

#include <cuda_pipeline_primitives.h>

#include <algorithm>

namespace {

__device__ __forceinline__ float2 cadd2(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub2(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cfma2(float2 a, float2 b, float2 c) {   // a*b + c
    return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y)));
}
__device__ __forceinline__ float2 cjfma2(float2 a, float2 b, float2 c) {  // conj(a)*b + c
    return make_float2(fmaf(a.x, b.x, fmaf(a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(-a.y, b.x, c.y)));
}

struct SArgs {
    const float2* Yh;     // scratch (c1 - c0, M, F): Y3-hat of sequences [c0, c1)
    const float2* G1h;    // (M, F)
    const float2* G3h;    // (M, F)
    const float2* Dg;     // (M, F): g1-hat - g3-hat, the same for every sequence
    float2* Dh;           // (N, M, F): rfft(d_old) in, the new d-hat out
    float2* g1h;          // (N, M, F)
    const float2* Zh;     // (N, F): rfft(G2 - g2)
    float2* Th;           // (N, F): scale * sum_m Y3h rfft(d_old)
    float2* part;         // (slots, 2, M, F): sums of d + g1 and of d over a sub-range
    double* rpart;        // (slots, nbb, 3): Parseval sums of |d-hat - G1-hat|^2,
                          // |d-hat - G3-hat|^2, |d-hat|^2 of a CTA (the residual record)
    int N, M, F, c0, c1, slot0;
    float kd, scale;
};

constexpr int kBins = 32, kWarps = 16;
constexpr int kArr = 3;      // staged spectra: Y3-hat, g1-hat, d-hat

// grid (ceil(F / 32), nsub): a CTA takes 32 bins and sub-range s of the sequences
// [c0, c1), in order, and writes that sub-range's sums to slot slot0 + s; warp w owns
// filters w, w + 16, ...  With PIPE, each thread's spectra of sequence n + 1 are copied
// to shared memory (asynchronous copies, two buffers) while sequence n is computed.
// RES: also the residual partials (compiled out when false)
template <int MW, bool PIPE, bool RES>
__global__ void __launch_bounds__(kBins * kWarps, 1) k_dspec(SArgs A) {
    extern __shared__ float4 sm4[];
    const int M = A.M, F = A.F;
    const int j = blockIdx.y, cn = A.c1 - A.c0;
    const int n0 = A.c0 + (int)((int64_t)cn * j / gridDim.y);
    const int n1 = A.c0 + (int)((int64_t)cn * (j + 1) / gridDim.y);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int f = blockIdx.x * kBins + lane;
    const bool on = f < F;
    const bool edge = f == 0 || f == F - 1;
    float2* G1s = reinterpret_cast<float2*>(sm4);          // [M][32]
    // Ks = G1-hat + G3-hat + Dg: H = (G1 - g1) + (G3 - g3) with g3 = g1 - Dg is
    // Ks - 2 g1, one shared spectrum instead of three (G3s is kept for the residuals)
    float2* Ks = G1s + (size_t)M * kBins;                  // [M][32]
    float2* G3s = Ks + (size_t)M * kBins;                  // [M][32]
    // the warps' partial sums of B, Q.x, Q.y, T.x, T.y per bin, [5][kWarps][32], and
    // their totals, [5][32]: each total is summed once, by one thread, in warp order
    float* pp = reinterpret_cast<float*>(G3s + (size_t)M * kBins);
    float* tot = pp + 5 * kWarps * kBins;
    for (int i = threadIdx.x; i < M * kBins; i += blockDim.x) {
        const int m = i / kBins, ff = blockIdx.x * kBins + i % kBins;
        const bool in = ff < F;
        const float2 g1 = in ? A.G1h[(size_t)m * F + ff] : make_float2(0.f, 0.f);
        const float2 g3 = in ? A.G3h[(size_t)m * F + ff] : make_float2(0.f, 0.f);
        const float2 dg = in ? A.Dg[(size_t)m * F + ff] : make_float2(0.f, 0.f);
        G1s[i] = g1;
        G3s[i] = g3;
        Ks[i] = cadd2(cadd2(g1, g3), dg);
    }
    float2 s1[MW], sd[MW];
#pragma unroll
    for (int k = 0; k < MW; ++k) s1[k] = sd[k] = make_float2(0.f, 0.f);
    // compensated (Kahan) float32 sums over this thread's sequences of the g1 and g3
    // increments' and d's squared magnitudes (Parseval weights: 1 at the edge bins, 2
    // elsewhere), combined in float64 at the end
    float rs[3] = {0.f, 0.f, 0.f}, rc[3] = {0.f, 0.f, 0.f};
    __syncthreads();
    const int fl = on ? f : 0;                             // lanes past F load bin 0
    // staging: [2][kArr][MW][threads], each thread's own slots
    float2* stg = reinterpret_cast<float2*>(tot + 5 * kBins);
    const int nt = blockDim.x, tid = threadIdx.x;
    auto stage = [&](int n, int buf) {
        const size_t base = (size_t)n * M * F + fl;
        const size_t ybase = (size_t)(n - A.c0) * M * F + fl;
#pragma unroll
        for (int k = 0; k < MW; ++k) {
            const int m = min(w + kWarps * k, M - 1);
            float2* d0 = stg + ((size_t)(buf * kArr + 0) * MW + k) * nt + tid;
            __pipeline_memcpy_async(d0, A.Yh + ybase + (size_t)m * F, sizeof(float2));
            __pipeline_memcpy_async(d0 + (size_t)MW * nt, A.g1h + base + (size_t)m * F, sizeof(float2));
            __pipeline_memcpy_async(d0 + (size_t)2 * MW * nt, A.Dh + base + (size_t)m * F, sizeof(float2));
        }
        __pipeline_commit();
    };
    if (PIPE && n0 < n1) stage(n0, 0);
    // rfft(G2 - g2) of the bin, loaded one sequence ahead (it is needed after the
    // cross-warp sums, where a load issued then would stall every warp)
    float2 zn = (on && n0 < n1) ? A.Zh[(size_t)n0 * F + f] : make_float2(0.f, 0.f);
    for (int n = n0; n < n1; ++n) {
        const float2 z = zn;
        if (on && n + 1 < n1) zn = A.Zh[(size_t)(n + 1) * F + f];
        // every load of this sequence first (independent), then the arithmetic
        float2 yv[MW], g1v[MW], dv[MW];
        if (PIPE) {
            if (n + 1 < n1) {
                stage(n + 1, (n + 1 - n0) & 1);
                __pipeline_wait_prior(1);
            } else {
                __pipeline_wait_prior(0);
            }
            const int buf = (n - n0) & 1;
#pragma unroll
            for (int k = 0; k < MW; ++k) {
                const float2* s0 = stg + ((size_t)(buf * kArr + 0) * MW + k) * nt + tid;
                yv[k] = s0[0];
                g1v[k] = s0[(size_t)MW * nt];
                dv[k] = s0[(size_t)2 * MW * nt];
            }
        } else {
            const size_t base = (size_t)n * M * F + fl;
            const size_t ybase = (size_t)(n - A.c0) * M * F + fl;
#pragma unroll
            for (int k = 0; k < MW; ++k) {
                const int m = min(w + kWarps * k, M - 1);  // in bounds; unused when m >= M
                yv[k] = A.Yh[ybase + (size_t)m * F];
                g1v[k] = A.g1h[base + (size_t)m * F];
                dv[k] = A.Dh[base + (size_t)m * F];
            }
        }
        float2 hv[MW];
        float B = 0.f;
        float2 Q = make_float2(0.f, 0.f), T = make_float2(0.f, 0.f);
#pragma unroll
        for (int k = 0; k < MW; ++k) {
            const int m = w + kWarps * k;
            const bool use = on && m < M;
            const int ms = use ? m : 0;
            const float2 y = use ? yv[k] : make_float2(0.f, 0.f);
            float2 d = use ? dv[k] : make_float2(0.f, 0.f);
            if (edge) d.y = 0.f;
            // H = (G1 - g1) + (G3 - g3) with g3 = g1 - Dg  (train.jl:52-54), = Ks - 2 g1
            const float2 h = use ? csub2(Ks[ms * kBins + lane], cadd2(g1v[k], g1v[k]))
                                 : make_float2(0.f, 0.f);
            hv[k] = h;
            B = fmaf(y.x, y.x, fmaf(y.y, y.y, B));
            Q = cfma2(y, h, Q);
            T = cfma2(y, d, T);
        }
        pp[(0 * kWarps + w) * kBins + lane] = B;
        pp[(1 * kWarps + w) * kBins + lane] = Q.x;
        pp[(2 * kWarps + w) * kBins + lane] = Q.y;
        pp[(3 * kWarps + w) * kBins + lane] = T.x;
        pp[(4 * kWarps + w) * kBins + lane] = T.y;
        __syncthreads();
        if (w < 5) {
            // warp w sums component w over the warps for its lane's bin, warp 0 first
            // (the order every thread summed all of them in before: the same bits)
            const float* src = pp + w * kWarps * kBins + lane;
            float acc = 0.f;
#pragma unroll
            for (int v = 0; v < kWarps; ++v) acc += src[v * kBins];
            tot[w * kBins + lane] = acc;
        }
        __syncthreads();                                   // totals written; partials read
        B = tot[lane];
        Q = make_float2(tot[kBins + lane], tot[2 * kBins + lane]);
        T = make_float2(tot[3 * kBins + lane], tot[4 * kBins + lane]);
        if (on) {
            const float inv = 1.f / (B + A.kd);
            const float2 beta = make_float2(fmaf(z.x, B, Q.x) * inv, fmaf(z.y, B, Q.y) * inv);
            const float2 W = csub2(z, beta);
            float q[3] = {0.f, 0.f, 0.f};
#pragma unroll
            for (int k = 0; k < MW; ++k) {
                const int m = w + kWarps * k;
                if (m >= M) continue;
                // REF_QUIRK_Q1: the combine has no 1/2, unlike the X-step's (cdl_kernels.jl:30)
                float2 dh = cjfma2(yv[k], W, hv[k]);
                if (edge) dh.y = 0.f;                      // the transform of a real d
                const size_t i = (size_t)n * M * F + (size_t)m * F + f;
                // g1 += d - G1 with G1 before the update (train.jl:70)
                const float2 e1 = csub2(dh, G1s[m * kBins + lane]);
                const float2 g1n = cadd2(g1v[k], e1);
                A.Dh[i] = dh;
                A.g1h[i] = g1n;
                s1[k] = cadd2(s1[k], cadd2(dh, g1n));
                sd[k] = cadd2(sd[k], dh);
                if (!RES) continue;
                const float2 e3 = csub2(dh, G3s[m * kBins + lane]);   // g3 += d - G3 (:72)
                q[0] = fmaf(e1.x, e1.x, fmaf(e1.y, e1.y, q[0]));
                q[1] = fmaf(e3.x, e3.x, fmaf(e3.y, e3.y, q[1]));
                q[2] = fmaf(dh.x, dh.x, fmaf(dh.y, dh.y, q[2]));
            }
            const float wt = edge ? 1.f : 2.f;
#pragma unroll
            for (int k = 0; k < (RES ? 3 : 0); ++k) {
                const float y = __fsub_rn(__fmul_rn(wt, q[k]), rc[k]);
                const float t = __fadd_rn(rs[k], y);
                rc[k] = __fsub_rn(__fsub_rn(t, rs[k]), y);
                rs[k] = t;
            }
            if (w == 0) A.Th[(size_t)n * F + f] = make_float2(T.x * A.scale, T.y * A.scale);
        }
    }
    if (RES) {
        // the CTA's residual partials, in float64, added in warp order
        __shared__ double rsh[3][kWarps];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            double v = (double)rs[k] - (double)rc[k];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) rsh[k][w] = v;
        }
        __syncthreads();
        if (threadIdx.x < 3) {
            double t = 0.0;
            for (int v = 0; v < kWarps; ++v) t += rsh[threadIdx.x][v];
            A.rpart[((size_t)(A.slot0 + j) * gridDim.x + blockIdx.x) * 3 + threadIdx.x] = t;
        }
    }
    if (!on) return;
#pragma unroll
    for (int k = 0; k < MW; ++k) {
        const int m = w + kWarps * k;
        if (m >= M) continue;
        const size_t pi = (size_t)m * F + f;
        const size_t q = (size_t)(A.slot0 + j) * 2 * M * F;
        A.part[q + pi] = s1[k];
        A.part[q + (size_t)M * F + pi] = sd[k];
    }
}

// The three sums' spectra, scaled by 1/Lg so that the unnormalised inverse transform
// gives the time-domain sums: out[0] = sum (d + g1), out[2] = sum d (over the slots, in
// double), out[1] = sum (d + g3) = out[0] - N Dg (Dg after this D-step's update).  Four
// threads per output take the slots j = t mod 4 in order; the four partials are added in
// a fixed order.
__global__ void k_dspec_sum(const float2* __restrict__ part, const float2* __restrict__ Dg,
                            float2* __restrict__ out, size_t mf, int slots, int N, double inv_lg) {
    const size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const size_t i = g >> 2;                                // 0 .. 2 mf - 1
    const int t = (int)(g & 3);
    double re = 0.0, im = 0.0;
    if (i < 2 * mf)
        for (int j = t; j < slots; j += 4) {
            const float2 v = part[(size_t)j * 2 * mf + i];
            re += v.x;
            im += v.y;
        }
    re += __shfl_down_sync(0xffffffffu, re, 1);
    im += __shfl_down_sync(0xffffffffu, im, 1);
    re += __shfl_down_sync(0xffffffffu, re, 2);
    im += __shfl_down_sync(0xffffffffu, im, 2);
    if (t != 0 || i >= 2 * mf) return;
    if (i < mf) {
        out[i] = make_float2((float)(re * inv_lg), (float)(im * inv_lg));
        const float2 dg = Dg[i];
        out[mf + i] = make_float2((float)((re - (double)N * dg.x) * inv_lg),
                                  (float)((im - (double)N * dg.y) * inv_lg));
    } else {
        out[mf + i] = make_float2((float)(re * inv_lg), (float)(im * inv_lg));
    }
}

// Dg += G3-hat - G1-hat (the change of g1 - g3 in one D-step, train.jl:70, 72)
__global__ void k_dg_update(float2* __restrict__ Dg, const float2* __restrict__ G1h,
                            const float2* __restrict__ G3h, size_t mf) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= mf) return;
    Dg[i] = cadd2(Dg[i], csub2(G3h[i], G1h[i]));
}

// broadcast of an (M, F) spectrum over n
__global__ void k_bcast_spec(float2* __restrict__ dst, const float2* __restrict__ plane, size_t mf,
                             size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        dst[i] = plane[i % mf];
}

// dst = a - plane, the plane broadcast over n (g3-hat = g1-hat - Dg)
__global__ void k_sub_bcast(float2* __restrict__ dst, const float2* __restrict__ a,
                            const float2* __restrict__ plane, size_t mf, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        dst[i] = csub2(a[i], plane[i % mf]);
}

__global__ void k_scale(float* __restrict__ x, size_t n, float s) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        x[i] *= s;
}

}  // namespace

int dspec_max_m() { return kWarps * 8; }

size_t dspec_part_bytes(int M, int F, int slots) { return (size_t)slots * 2 * M * F * sizeof(float2); }

// Sub-ranges of one launch over cn sequences.  One CTA fits per SM, so a launch runs
// ceil(nbb nsub / nsm) waves of CTAs that each take ceil(cn / nsub) sequences after a
// start-up (the block's G1-hat, G3-hat, Dg and the first staged sequence) worth about
// two sequences; the count minimising that estimate is taken (the smallest on ties).
// It depends only on (cn, F, nsm), so the slot layout and the order of the sums are
// fixed for a given device and size.
int dspec_nsub(int cn, int F, int nsm) {
    const int nbb = (F + kBins - 1) / kBins;
    if (nsm < 1) nsm = 1;
    int best = 1;
    long long bt = -1;
    for (int s = 1; s <= std::min(cn, 2048); ++s) {
        const long long waves = ((long long)nbb * s + nsm - 1) / nsm;
        const long long t = waves * ((cn + s - 1) / s + 2);
        if (bt < 0 || t < bt) { bt = t; best = s; }
    }
    return best;
}

int dspec_slots(int N, int chunk, int F, int nsm) {
    int slots = 0;
    for (int n0 = 0; n0 < N; n0 += chunk) slots += dspec_nsub(std::min(chunk, N - n0), F, nsm);
    return slots;
}

int dspec_launch(cdlgb_ctx* c, const float2* Yh, const float2* G3h, int c0, int c1, int slot0) {
    SArgs a;
    a.Yh = Yh; a.G1h = c->G1h; a.G3h = G3h; a.Dg = c->Dg; a.Dh = c->Dhs; a.g1h = c->g1h;
    a.Zh = c->sUh; a.Th = c->sVh; a.part = c->spart; a.rpart = c->rpart;
    a.N = c->N; a.M = c->M; a.F = c->F; a.c0 = c0; a.c1 = c1; a.slot0 = slot0;
    a.kd = c->p.sherman_const_cdl; a.scale = 1.f / (float)c->Lg;
    const dim3 g((unsigned)((c->F + kBins - 1) / kBins), (unsigned)dspec_nsub(c1 - c0, c->F, c->nsm));
    const size_t sm = (size_t)3 * c->M * kBins * sizeof(float2) + (size_t)kWarps * kBins * 5 * sizeof(float) +
                      (size_t)5 * kBins * sizeof(float);
    if (c->M <= 4 * kWarps) {
        // + the two staging buffers: 2 x 3 spectra x 4 filters x 512 threads
        const size_t smp = sm + (size_t)2 * kArr * 4 * kBins * kWarps * sizeof(float2);
        auto k = c->res_on ? k_dspec<4, true, true> : k_dspec<4, true, false>;
        CU_TRY(c, cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smp));
        k<<<g, kBins * kWarps, smp, c->stream>>>(a);
    } else {
        auto k = c->res_on ? k_dspec<8, false, true> : k_dspec<8, false, false>;
        if (sm > 48 * 1024) CU_TRY(c, cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        k<<<g, kBins * kWarps, sm, c->stream>>>(a);
    }
    LAUNCH_CHECK(c, "k_dspec");
    return CDLGB_OK;
}

// the Dg update (after every chunk has used the old Dg) and the three sums: out (3, M, F)
int dspec_sums(cdlgb_ctx* c, const float2* G3h, float2* out) {
    const size_t mf = (size_t)c->M * c->F;
    k_dg_update<<<(unsigned)((mf + 255) / 256), 256, 0, c->stream>>>(c->Dg, c->G1h, G3h, mf);
    LAUNCH_CHECK(c, "k_dg_update");
    k_dspec_sum<<<(unsigned)((4 * 2 * mf + 255) / 256), 256, 0, c->stream>>>(
        c->spart, c->Dg, out, mf, c->dslots, c->N, 1.0 / (double)c->Lg);
    LAUNCH_CHECK(c, "k_dspec_sum");
    return CDLGB_OK;
}

int dspec_bcast(cdlgb_ctx* c, float2* dst, const float2* plane) {
    const size_t mf = (size_t)c->M * c->F;
    k_bcast_spec<<<grid_for(mf * c->N, 256), 256, 0, c->stream>>>(dst, plane, mf, mf * c->N);
    LAUNCH_CHECK(c, "k_bcast_spec");
    return CDLGB_OK;
}

// g3-hat of rows (sequence x filter) [0, rows) of g1h into dst
int dspec_g3(cdlgb_ctx* c, float2* dst, const float2* g1h, size_t rows) {
    const size_t mf = (size_t)c->M * c->F;
    k_sub_bcast<<<grid_for(rows * c->F, 256), 256, 0, c->stream>>>(dst, g1h, c->Dg, mf, rows * c->F);
    LAUNCH_CHECK(c, "k_sub_bcast");
    return CDLGB_OK;
}

int dspec_scale(cdlgb_ctx* c, float* x, size_t n, float s) {
    k_scale<<<grid_for(n, 256), 256, 0, c->stream>>>(x, n, s);
    LAUNCH_CHECK(c, "k_scale");
    return CDLGB_OK;
}
