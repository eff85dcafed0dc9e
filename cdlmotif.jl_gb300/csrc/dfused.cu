// Fused D-step (dict_update!, src/CDL/train.jl:46-89): one launch per D-step iteration
// for the transform lengths with register-resident FFTs (regfft.cuh).
//
// A cluster of CS CTAs takes one sequence n at a time; each CTA owns MC filters
// (MC / 2 pairs).  Per pair it transforms three packed real pairs,
//   Y3 = projectionX!(X + y3)            (cdl_kernels.jl:68-82 layout, train.jl:52)
//   H  = (G1 - g1) + (G3 - g3)           (the RHS terms of sherman_CDL_RHS!, :2-22)
//   d  (the previous iterate, for Td)    (train.jl:56-57)
// and the sequence's Z = G2 - g2.  Per frequency the CTA sums over its filters, in
// filter order, B = sum |Y3h|^2, Q = sum Y3h Hh, T = sum Y3h dh_old; the cluster adds
// the CTA parts in rank order (distributed shared memory), every CTA forms
//   beta = (Zh B + Q) / (B + k),  dh = Hh + conj(Y3h) (Zh - beta)   (no 1/2: quirk Q1)
// for its filters and inverts them in place; rank 0 also inverts Th = T for Td and
// updates G2 and g2 (update_g2!, cdl_kernels.jl:68-77).  The consensus duals
// g1 = (g1 + d) - G1, g3 = (g3 + d) - G3 (train.jl:70-72) are written with d; their
// means over n are formed by a separate read-only pass (k_dsum in admm.cu).
//
// The packed spectra are split with doubled values (2 Y3h, 2 Hh, 2 dh_old): B, Q, T
// come out exactly 4x and dh exactly 2x, and are rescaled by powers of two.
#include "cdlgb_internal.h"
#include "regfft.cuh"

#include <cooperative_groups.h>
#include <stdlib.h>
#include <vector>

namespace cg = cooperative_groups;

namespace {

struct DArgs {
    const float* X;
    const float* y3;
    float* d;
    float* g1;
    float* g3;
    const float* G1;
    const float* G3;
    float* G2;
    float* g2;
    float* Td;
    const float* S;
    const float2* tw2;
    int N, M, L4, gamma;
    float kd, sigma;
};

// 2 Xa[f], 2 Xb[f] of a packed spectrum Z = Xa + i Xb of two real sequences
__device__ __forceinline__ void split2(const float2 z1, const float2 z2, float2& a, float2& b) {
    a = f2(z1.x + z2.x, z1.y - z2.y);
    b = f2(z1.y + z2.y, z2.x - z1.x);
}

template <int N1, int P, int NT, int MINB, int MC>
__global__ void __launch_bounds__(NT, MINB) k_dfused(DArgs A) {
    constexpr int Lg = N1 * P;
    constexpr int G = 32 / N1;
    constexpr int RS = N1 + 1;
    constexpr int BUF = (P * RS + 1) & ~1;
    constexpr int half = Lg / 2;
    constexpr int F = Lg / 2 + 1;
    constexpr int Fp = (F + 1) & ~1;
    constexpr int B = MC / 2;                   // pairs
    constexpr int NSL = 3 * B + 1;              // Y3 pairs, H pairs, d pairs, Z
    constexpr int NG = (NT / 32) * G;           // lane groups
    constexpr int QMAX = (NSL + NG - 1) / NG;   // slots per lane group
    constexpr int NFR = (F + NT - 1) / NT;      // bins per thread in the block phases
    static_assert(MC % 2 == 0, "filters per CTA must pair up");
    extern __shared__ float4 smem4[];
    cg::cluster_group cluster = cg::this_cluster();
    const int CS = (int)cluster.num_blocks();
    const int rank = (int)cluster.block_rank();
    const int cid = blockIdx.x / CS;
    const int nclusters = gridDim.x / CS;
    const int M = A.M;

    float2* bufs = reinterpret_cast<float2*>(smem4);       // [NSL][BUF]
    float2* tw2 = bufs + (size_t)NSL * BUF;                // [P][N1]
    float2* Qp = tw2 + P * N1;                             // [2][Fp] this CTA's Q part
    float2* Tp = Qp + 2 * Fp;                              // [2][Fp] this CTA's T part
    float* Bp = reinterpret_cast<float*>(Tp + 2 * Fp);     // [2][Fp] this CTA's B part

    for (int t = threadIdx.x; t < P * N1; t += blockDim.x) tw2[t] = A.tw2[t];
    __syncthreads();

    const int m0 = rank * MC;
    const int lane = threadIdx.x & 31;
    const int grp = (threadIdx.x >> 5) * G + lane / N1;
    const int gl = lane % N1;
    const bool keep = (gl & 3) == 0;                      // rows l % 4 == 0
    const float scale = 1.f / (float)Lg;
    int it = 0;

    for (int n = cid; n < A.N; n += nclusters, ++it) {
        // ---------------- inputs and forward transforms, slot by slot
#pragma unroll 1
        for (int q = 0; q < QMAX; ++q) {
            const int sl = grp + q * NG;
            const bool act = sl < NSL;
            float2* sb = bufs + (size_t)(act ? sl : 0) * BUF;
            if (act) {
                if (sl < B) {                              // Y3 pair
                    const size_t ra = ((size_t)n * M + m0 + 2 * sl) * Lg + gl;
#pragma unroll 4
                    for (int n2 = 0; n2 < P; ++n2) {
                        const int o = N1 * n2;
                        float2 v = f2(0.f, 0.f);
                        if (keep) v = f2(A.X[ra + o] + A.y3[ra + o], A.X[ra + Lg + o] + A.y3[ra + Lg + o]);
                        sb[n2 * RS + gl] = v;
                    }
                } else if (sl < 2 * B) {                   // H pair
                    const int s = sl - B;
                    const int ma = m0 + 2 * s;
                    const size_t ra = ((size_t)n * M + ma) * Lg + gl;
                    const size_t pa = (size_t)ma * Lg + gl;
#pragma unroll 4
                    for (int n2 = 0; n2 < P; ++n2) {
                        const int o = N1 * n2;
                        const float ha = (A.G1[pa + o] - A.g1[ra + o]) + (A.G3[pa + o] - A.g3[ra + o]);
                        const float hb = (A.G1[pa + Lg + o] - A.g1[ra + Lg + o]) +
                                         (A.G3[pa + Lg + o] - A.g3[ra + Lg + o]);
                        sb[n2 * RS + gl] = f2(ha, hb);
                    }
                } else if (sl < 3 * B) {                   // d (previous iterate) pair
                    const int s = sl - 2 * B;
                    const size_t ra = ((size_t)n * M + m0 + 2 * s) * Lg + gl;
#pragma unroll 4
                    for (int n2 = 0; n2 < P; ++n2) {
                        const int o = N1 * n2;
                        sb[n2 * RS + gl] = f2(A.d[ra + o], A.d[ra + Lg + o]);
                    }
                } else {                                   // Z = G2 - g2
                    const size_t r = (size_t)n * Lg + gl;
#pragma unroll 4
                    for (int n2 = 0; n2 < P; ++n2) {
                        const int o = N1 * n2;
                        sb[n2 * RS + gl] = f2(A.G2[r + o] - A.g2[r + o], 0.f);
                    }
                }
                fwd_step1<N1, P>(sb, gl, tw2);
            }
            __syncwarp();
            fwd_step2<N1, P>(sb, gl, act);
        }
        __syncthreads();

        // ---------------- this CTA's parts of B, Q, T (filter order)
        const int par = it & 1;
#pragma unroll 1
        for (int r = 0; r < NFR; ++r) {
            const int f = threadIdx.x + r * NT;
            if (f >= F) break;
            const bool edge = (f == 0) || (f == half);
            const int fr = edge ? f : Lg - f;
            float Bs = 0.f;
            float2 Qs = f2(0.f, 0.f), Ts = f2(0.f, 0.f);
#pragma unroll
            for (int s = 0; s < B; ++s) {
                float2 ya, yb, ha, hb, da, db;
                split2(bufs[s * BUF + f], bufs[s * BUF + fr], ya, yb);
                split2(bufs[(B + s) * BUF + f], bufs[(B + s) * BUF + fr], ha, hb);
                split2(bufs[(2 * B + s) * BUF + f], bufs[(2 * B + s) * BUF + fr], da, db);
                Bs = fmaf(ya.x, ya.x, fmaf(ya.y, ya.y, Bs));
                Qs = cfma(ya, ha, Qs);
                Ts = cfma(ya, da, Ts);
                Bs = fmaf(yb.x, yb.x, fmaf(yb.y, yb.y, Bs));
                Qs = cfma(yb, hb, Qs);
                Ts = cfma(yb, db, Ts);
            }
            // every term was exactly 4x
            Bp[par * Fp + f] = 0.25f * Bs;
            Qp[par * Fp + f] = f2(0.25f * Qs.x, 0.25f * Qs.y);
            Tp[par * Fp + f] = f2(0.25f * Ts.x, 0.25f * Ts.y);
        }
        cluster.sync();

        // ---------------- sums over the cluster, beta, dh for this CTA's filters (packed
        // back into the H slots), Th into the Z slot
        float2* ZS = bufs + (size_t)(3 * B) * BUF;
#pragma unroll 1
        for (int r = 0; r < NFR; ++r) {
            const int f = threadIdx.x + r * NT;
            if (f >= F) break;
            float Bv[8];
            float2 Qv[8], Tv[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                if (k < CS) {
                    Bv[k] = cluster.map_shared_rank(Bp + par * Fp, k)[f];
                    Qv[k] = cluster.map_shared_rank(Qp + par * Fp, k)[f];
                    Tv[k] = cluster.map_shared_rank(Tp + par * Fp, k)[f];
                }
            }
            float Bt = 0.f;
            float2 Qt = f2(0.f, 0.f), Tt = f2(0.f, 0.f);
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                if (k < CS) {
                    Bt += Bv[k];
                    Qt = cadd(Qt, Qv[k]);
                    Tt = cadd(Tt, Tv[k]);
                }
            }
            const bool edge = (f == 0) || (f == half);
            const int fr = edge ? f : Lg - f;
            const float2 z = ZS[f];
            const float inv = 1.f / (Bt + A.kd);
            const float2 beta = f2(fmaf(z.x, Bt, Qt.x) * inv, fmaf(z.y, Bt, Qt.y) * inv);
            const float2 W = csub(z, beta);
            const float sch = 0.5f * scale;
#pragma unroll
            for (int s = 0; s < B; ++s) {
                float2 ya, yb, ha, hb;
                split2(bufs[s * BUF + f], bufs[s * BUF + fr], ya, yb);
                float2* HS = bufs + (size_t)(B + s) * BUF;
                split2(HS[f], HS[fr], ha, hb);
                float2 xa = cjfma(ya, W, ha);              // 2 dh
                float2 xb = cjfma(yb, W, hb);
                xa = f2(__fmul_rn(xa.x, sch), __fmul_rn(xa.y, sch));
                xb = f2(__fmul_rn(xb.x, sch), __fmul_rn(xb.y, sch));
                if (edge) {
                    HS[f] = f2(xa.x, xb.x);
                } else {
                    HS[f] = f2(xa.x - xb.y, xa.y + xb.x);
                    HS[Lg - f] = f2(xa.x + xb.y, xb.x - xa.y);
                }
            }
            const float2 Th = f2(Tt.x * scale, Tt.y * scale);
            if (edge) {
                ZS[f] = f2(Th.x, 0.f);
            } else {
                ZS[f] = Th;
                ZS[Lg - f] = f2(Th.x, -Th.y);
            }
        }
        __syncthreads();

        // ---------------- inverse transforms of the H slots (new d) and, on rank 0, of
        // the Z slot (Td); the outputs
#pragma unroll 1
        for (int q = 0; q < QMAX; ++q) {
            const int sl = grp + q * NG;
            const bool inv = (sl >= B && sl < 2 * B) || (sl == 3 * B && rank == 0);
            float2* sb = bufs + (size_t)(inv ? sl : 0) * BUF;
            inv_step2<N1, P, false>(sb, gl, inv, tw2);
            if (!inv) continue;
            inv_step1<N1, P, true>(sb, gl, tw2);
            if (sl < 2 * B) {
                const int ma = m0 + 2 * (sl - B);
                const size_t ra = ((size_t)n * M + ma) * Lg + gl;
                const size_t pa = (size_t)ma * Lg + gl;
#pragma unroll 4
                for (int n2 = 0; n2 < P; ++n2) {
                    const int o = N1 * n2;
                    const float2 dv = sb[n2 * RS + gl];
                    A.d[ra + o] = dv.x;
                    A.d[ra + Lg + o] = dv.y;
                    A.g1[ra + o] = (A.g1[ra + o] + dv.x) - A.G1[pa + o];
                    A.g1[ra + Lg + o] = (A.g1[ra + Lg + o] + dv.y) - A.G1[pa + Lg + o];
                    A.g3[ra + o] = (A.g3[ra + o] + dv.x) - A.G3[pa + o];
                    A.g3[ra + Lg + o] = (A.g3[ra + Lg + o] + dv.y) - A.G3[pa + Lg + o];
                }
            } else {
                // G2 = (W'S + sigma (Td + g2)) / (W'W + sigma), g2 += Td - G2
                const size_t r = (size_t)n * Lg + gl;
#pragma unroll 4
                for (int n2 = 0; n2 < P; ++n2) {
                    const int o = N1 * n2;
                    const int l = gl + o;
                    const bool in = l >= A.gamma && l < A.gamma + A.L4;
                    const float wts = in ? A.S[(size_t)n * A.L4 + (l - A.gamma)] : 0.f;
                    const float dg = in ? 1.f : 0.f;
                    const float t = sb[n2 * RS + gl].x, g = A.g2[r + o];
                    const float Gn = __fadd_rn(wts, __fmul_rn(A.sigma, t + g)) / (dg + A.sigma);
                    A.Td[r + o] = t;
                    A.G2[r + o] = Gn;
                    A.g2[r + o] = (g + t) - Gn;
                }
            }
        }
    }
    cluster.sync();
}

typedef void (*kern_t)(DArgs);
constexpr size_t kCap = 226 * 1024;
struct Variant { int N1, P, MC, threads; kern_t k; };
const Variant kVariants[] = {
    {32, 29, 16, 288, k_dfused<32, 29, 288, 1, 16>},
    {16, 31, 16, 160, k_dfused<16, 31, 160, 1, 16>},
};

size_t dfused_smem(int N1, int P, int MC) {
    const int Lg = N1 * P, F = Lg / 2 + 1, Fp = (F + 1) & ~1;
    const size_t buf = ((size_t)P * (N1 + 1) + 1) & ~(size_t)1;
    const int nsl = 3 * (MC / 2) + 1;
    return ((size_t)nsl * buf + (size_t)P * N1 + 4 * (size_t)Fp) * sizeof(float2) +
           2 * (size_t)Fp * sizeof(float);
}

struct DPlan {
    kern_t k;
    int CS, threads, grid;
    size_t smem;
    float2* tw2;
};

}  // namespace

// Opt-in (CDLGB_DFUSED=1): the first variant whose transform length is Lg and whose
// filters per CTA divide M into 1, 2, 4 or 8 CTAs.  Measured at L=200, K=64 it takes
// 37.8 ms per D-step against 25.7 ms for the cuFFT D-step: with one CTA per SM the
// per-slot HBM loads are not hidden.  Returns nullptr when off or without a variant.
void* dfused_plan_create(cdlgb_ctx* c, int* status) {
    *status = CDLGB_OK;
    const char* on = getenv("CDLGB_DFUSED");
    if (!on || atoi(on) == 0) return nullptr;
    const Variant* v = nullptr;
    int cs = 0;
    for (const Variant& cand : kVariants) {
        if (cand.N1 * cand.P != c->Lg || c->M % cand.MC) continue;
        cs = c->M / cand.MC;
        if (cs != 1 && cs != 2 && cs != 4 && cs != 8) continue;
        if (dfused_smem(cand.N1, cand.P, cand.MC) > kCap) continue;
        v = &cand;
        break;
    }
    if (!v) return nullptr;
    DPlan* P = new DPlan();
    P->k = v->k; P->CS = cs; P->threads = v->threads;
    P->smem = dfused_smem(v->N1, v->P, v->MC);
    std::vector<float2> tw2 = regfft_twiddles(v->N1, v->P);
    cudaError_t e = regfft_upload_tables();
    if (e == cudaSuccess) e = cudaMalloc((void**)&P->tw2, tw2.size() * sizeof(float2));
    if (e == cudaSuccess) e = cudaMemcpy(P->tw2, tw2.data(), tw2.size() * sizeof(float2), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(P->k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kCap);
    int nclusters = 0;
    if (e == cudaSuccess) {
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = P->CS;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3(P->CS * 152 * 4, 1, 1);
        cfg.blockDim = dim3(P->threads, 1, 1);
        cfg.dynamicSmemBytes = P->smem;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        e = cudaOccupancyMaxActiveClusters(&nclusters, (void*)P->k, &cfg);
    }
    if (e != cudaSuccess || nclusters < 1) {
        *status = cdlgb_seterr(c, CDLGB_ECUDA, "fused D-step setup failed: %s",
                               e != cudaSuccess ? cudaGetErrorString(e) : "no cluster fits");
        if (P->tw2) cudaFree(P->tw2);
        delete P;
        return nullptr;
    }
    if (nclusters > c->N) nclusters = c->N;
    P->grid = nclusters * P->CS;
    return P;
}

void dfused_plan_free(void* p) {
    DPlan* P = (DPlan*)p;
    if (!P) return;
    if (P->tw2) cudaFree(P->tw2);
    delete P;
}

// One fused D-step pass over all sequences (everything of dict_update! but the
// consensus means and the projections).
int dfused_step(cdlgb_ctx* c, void* p, const float* X) {
    DPlan* P = (DPlan*)p;
    DArgs a;
    a.X = X; a.y3 = c->y3; a.d = c->d; a.g1 = c->g1; a.g3 = c->g3;
    a.G1 = c->G1; a.G3 = c->G3; a.G2 = c->G2; a.g2 = c->g2; a.Td = c->Td; a.S = c->S;
    a.tw2 = P->tw2;
    a.N = c->N; a.M = c->M; a.L4 = c->L4; a.gamma = c->gamma;
    a.kd = c->p.sherman_const_cdl; a.sigma = c->p.sigma;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = P->CS;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(P->grid, 1, 1);
    cfg.blockDim = dim3(P->threads, 1, 1);
    cfg.dynamicSmemBytes = P->smem;
    cfg.stream = c->stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cdlgb_phase_begin(c, PH_DFUSED_A);
    CU_TRY(c, cudaLaunchKernelEx(&cfg, P->k, a));
    LAUNCH_CHECK(c, "k_dfused");
    cdlgb_phase_end(c, PH_DFUSED_A);
    return CDLGB_OK;
}
