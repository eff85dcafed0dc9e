// Fused X-step, one ADMM X-step per launch, with register-resident four-step FFTs
// (regfft.cuh).  Same algebra and cluster structure as the generic fused kernel
// (fused.cu), but each packed column pair (and the U / DX slot) is owned by a group
// of N1 lanes that transforms it without block-wide barriers.  The block-wide phases
// between the transforms (split of the packed spectra, cross-filter sums,
// Sherman-Morrison combine) read and write the spectra in shared memory; the
// cross-filter sum over the cluster goes through distributed shared memory in fixed
// rank order.  The state streams through HBM once per X-step.
#include "cdlgb_internal.h"
#include "regfft.cuh"

#include <cooperative_groups.h>
#include <math.h>
#include <stdlib.h>
#include <vector>

namespace cg = cooperative_groups;

namespace {

constexpr int kMaxThreads = 160;
constexpr size_t kWarpSmemCap = 72 * 1024;   // three CTAs per SM

struct WArgs {
    const float* Xin;
    float* Xout;
    float* y2;
    float* y3;
    float* Y1;
    float* y1;
    float* DX;
    const float* S;
    const float2* G1h;
    const float* Ah;
    const float2* tw2;      // [P][N1] exp(-2 pi i n1 k2 / Lg)
    double* absx_part;
    int N, M, F, L4, gamma;
    float lam, rho, kc;
    int Mc, B;
};

template <int N1, int P, int MINB, bool G1S>
__global__ void __launch_bounds__(kMaxThreads, MINB) k_xstep_warp(WArgs A) {
    constexpr int Lg = N1 * P;
    constexpr int Lg4 = Lg / 4;
    constexpr int G = 32 / N1;                  // lane groups per warp
    constexpr int RS = N1 + 1;                  // row stride of the transposed layout
    constexpr int BUF = (P * RS + 1) & ~1;      // complex entries per group buffer, kept even
                                                // so every region after it stays 16-byte aligned
    constexpr int half = Lg / 2;
    constexpr int F = Lg / 2 + 1;
    constexpr int Fp = (F + 1) & ~1;
    extern __shared__ float4 smem4[];
    cg::cluster_group cluster = cg::this_cluster();
    const int CS = (int)cluster.num_blocks();
    const int rank = (int)cluster.block_rank();
    const int cid = blockIdx.x / CS;
    const int nclusters = gridDim.x / CS;
    const int B = A.B, Mc = A.Mc, M = A.M;
    const int NG = (blockDim.x >> 5) * G;      // lane groups in the CTA
    const int Q = (B + 1 + NG - 1) / NG;       // slots (B pairs + the U/DX slot) per group

    float2* tw2 = reinterpret_cast<float2*>(smem4);
    float2* bufs = tw2 + P * N1;
    float2* Ppart = bufs + (size_t)(B + 1) * BUF;
    float2* Wv = Ppart + 2 * Fp;
    float* y1s = reinterpret_cast<float*>(Wv + Fp);
    float2* g1s = reinterpret_cast<float2*>(y1s + Lg);   // [Mc][F] slice of G1h (G1S only)
    __shared__ double red[kMaxThreads / 32];

    for (int t = threadIdx.x; t < P * N1; t += blockDim.x) tw2[t] = A.tw2[t];
    const int m0 = (int)cluster.block_rank() * A.Mc;
    if (G1S) {
        for (int t = threadIdx.x; t < A.Mc * F; t += blockDim.x) g1s[t] = A.G1h[(size_t)m0 * F + t];
    }
    // filter m's spectrum at bin f
    const float2* g1 = G1S ? g1s : A.G1h + (size_t)m0 * F;
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const int grp = (threadIdx.x >> 5) * G + lane / N1;   // lane group; transforms slots grp + q*NG
    const int gl = lane % N1;                             // lane within the group
    const float sc = 1.f / (A.kc * (float)Lg);
    const float lam = A.lam;
    double absacc = 0.0;

    // Streamed pass over the items (slot, 4 consecutive rows): stores the results of
    // sequence ns (X of the filter pairs; on rank 0 also DX, y1', Y1) from the group
    // buffers and loads sequence nl (shrink!, projectionX!, the dual updates written
    // back, V and U packed into the same buffer positions).  Either may be -1.  Loads of
    // kB items are issued before any item is processed.
    auto streamed = [&](int ns, int nl) {
        constexpr int kB = 2;
        const int nitems = (B + 1) * Lg4;
        for (int base = threadIdx.x; base < nitems; base += kB * blockDim.x) {
            float4 x[kB][2], a[kB][2], c[kB][2];
#pragma unroll
            for (int u = 0; u < kB; ++u) {
                const int idx = base + u * blockDim.x;
                const int sl = idx / Lg4;
                const int l = 4 * (idx - sl * Lg4);
                x[u][0] = x[u][1] = a[u][0] = a[u][1] = c[u][0] = c[u][1] = make_float4(0, 0, 0, 0);
                if (idx < nitems && nl >= 0) {
                    if (sl < B) {
                        const size_t ba = ((size_t)nl * M + m0 + 2 * sl) * Lg + l;
                        x[u][0] = *reinterpret_cast<const float4*>(A.Xin + ba);
                        a[u][0] = *reinterpret_cast<const float4*>(A.y2 + ba);
                        c[u][0] = *reinterpret_cast<const float4*>(A.y3 + ba);
                        if (2 * sl + 1 < Mc) {
                            x[u][1] = *reinterpret_cast<const float4*>(A.Xin + ba + Lg);
                            a[u][1] = *reinterpret_cast<const float4*>(A.y2 + ba + Lg);
                            c[u][1] = *reinterpret_cast<const float4*>(A.y3 + ba + Lg);
                        }
                    } else {
                        const size_t bl = (size_t)nl * Lg + l;
                        x[u][0] = *reinterpret_cast<const float4*>(A.Y1 + bl);
                        a[u][0] = *reinterpret_cast<const float4*>(A.y1 + bl);
                        c[u][0] = *reinterpret_cast<const float4*>(A.DX + bl);
                    }
                }
            }
#pragma unroll
            for (int u = 0; u < kB; ++u) {
                const int idx = base + u * blockDim.x;
                if (idx >= nitems) break;
                const int sl = idx / Lg4;
                const int l = 4 * (idx - sl * Lg4);
                float2* z = bufs + (size_t)sl * BUF + (l / N1) * RS + (l % N1);
                // ---- results of sequence ns
                if (ns >= 0) {
                    const float2 z0 = z[0], z1 = z[1], z2 = z[2], z3 = z[3];
                    if (sl < B) {
                        const size_t ba = ((size_t)ns * M + m0 + 2 * sl) * Lg + l;
                        const float4 xa = make_float4(z0.x, z1.x, z2.x, z3.x);
                        *reinterpret_cast<float4*>(A.Xout + ba) = xa;
                        float s4 = (fabsf(xa.x) + fabsf(xa.y)) + (fabsf(xa.z) + fabsf(xa.w));
                        if (2 * sl + 1 < Mc) {
                            const float4 xb = make_float4(z0.y, z1.y, z2.y, z3.y);
                            *reinterpret_cast<float4*>(A.Xout + ba + Lg) = xb;
                            s4 += (fabsf(xb.x) + fabsf(xb.y)) + (fabsf(xb.z) + fabsf(xb.w));
                        }
                        absacc += (double)s4;
                    } else if (rank == 0) {
                        // Y1 = (W'S + rho (DX + y1')) / (W'W + rho)  (update_Y1!, csc_kernels.jl:86-95)
                        const float dx[4] = {z0.x, z1.x, z2.x, z3.x};
                        const float4 yn4 = *reinterpret_cast<const float4*>(y1s + l);
                        const float yn[4] = {yn4.x, yn4.y, yn4.z, yn4.w};
                        float Yo[4];
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            const int le = l + e;
                            const bool in = le >= A.gamma && le < A.gamma + A.L4;
                            const float wts = in ? A.S[(size_t)ns * A.L4 + (le - A.gamma)] : 0.f;
                            const float dg = in ? 1.f : 0.f;
                            Yo[e] = __fadd_rn(wts, __fmul_rn(A.rho, dx[e] + yn[e])) / (dg + A.rho);
                        }
                        const size_t bs = (size_t)ns * Lg + l;
                        *reinterpret_cast<float4*>(A.DX + bs) = make_float4(dx[0], dx[1], dx[2], dx[3]);
                        *reinterpret_cast<float4*>(A.y1 + bs) = yn4;
                        *reinterpret_cast<float4*>(A.Y1 + bs) = make_float4(Yo[0], Yo[1], Yo[2], Yo[3]);
                    }
                }
                // ---- inputs of sequence nl
                if (nl >= 0) {
                    if (sl < B) {
                        const size_t ba = ((size_t)nl * M + m0 + 2 * sl) * Lg + l;
                        float4 na, nb, va, vb = make_float4(0, 0, 0, 0);
                        xprep1(x[u][0].x, a[u][0].x, c[u][0].x, lam, true, na.x, nb.x, va.x);   // .x: 4-stride
                        xprep1(x[u][0].y, a[u][0].y, c[u][0].y, lam, false, na.y, nb.y, va.y);
                        xprep1(x[u][0].z, a[u][0].z, c[u][0].z, lam, false, na.z, nb.z, va.z);
                        xprep1(x[u][0].w, a[u][0].w, c[u][0].w, lam, false, na.w, nb.w, va.w);
                        *reinterpret_cast<float4*>(A.y2 + ba) = na;
                        *reinterpret_cast<float4*>(A.y3 + ba) = nb;
                        if (2 * sl + 1 < Mc) {
                            xprep1(x[u][1].x, a[u][1].x, c[u][1].x, lam, true, na.x, nb.x, vb.x);
                            xprep1(x[u][1].y, a[u][1].y, c[u][1].y, lam, false, na.y, nb.y, vb.y);
                            xprep1(x[u][1].z, a[u][1].z, c[u][1].z, lam, false, na.z, nb.z, vb.z);
                            xprep1(x[u][1].w, a[u][1].w, c[u][1].w, lam, false, na.w, nb.w, vb.w);
                            *reinterpret_cast<float4*>(A.y2 + ba + Lg) = na;
                            *reinterpret_cast<float4*>(A.y3 + ba + Lg) = nb;
                        }
                        z[0] = f2(va.x, vb.x);
                        z[1] = f2(va.y, vb.y);
                        z[2] = f2(va.z, vb.z);
                        z[3] = f2(va.w, vb.w);
                    } else {
                        // U = Y1 - y1', y1' = y1 + DX - Y1  (train.jl:12)
                        const float4 Yv = x[u][0], yv = a[u][0], dv = c[u][0];
                        const float4 yn = make_float4((yv.x + dv.x) - Yv.x, (yv.y + dv.y) - Yv.y,
                                                      (yv.z + dv.z) - Yv.z, (yv.w + dv.w) - Yv.w);
                        *reinterpret_cast<float4*>(y1s + l) = yn;
                        z[0] = f2(Yv.x - yn.x, 0.f);
                        z[1] = f2(Yv.y - yn.y, 0.f);
                        z[2] = f2(Yv.z - yn.z, 0.f);
                        z[3] = f2(Yv.w - yn.w, 0.f);
                    }
                }
            }
        }
    };

    int it = 0;
    if (cid < A.N) streamed(-1, cid);
    __syncthreads();
    for (int n = cid; n < A.N; n += nclusters, ++it) {
        // ---------------- forward transforms, Q slots per lane group
        for (int q = 0; q < Q; ++q) {
            const int sl = grp + q * NG;
            // a group with no slot left (sl > B) still runs the row DFT's loads, reading
            // slot 0 and storing nothing: its own slot would lie past the buffers
            float2* sb = bufs + (size_t)(sl <= B ? sl : 0) * BUF;
            if (sl <= B) fwd_step1<N1, P>(sb, gl, tw2);
            __syncwarp();
            fwd_step2<N1, P>(sb, gl, sl <= B);
        }
        __syncthreads();

        // ---------------- split + this CTA's part of P = sum_m G1h[m] Vh[m]
        float2* Pp = Ppart + (it & 1) * Fp;
        for (int f = threadIdx.x; f < F; f += blockDim.x)
            Pp[f] = partial_P<Lg>(bufs, BUF, B, Mc, F, f, g1);
        cluster.sync();

        // ---------------- P over the cluster (fixed rank order), alpha, W; rank 0 packs
        // DXh = (P + A W)/(k Lg); every CTA repacks Xh = (Vh + conj(G1h) W)/(k Lg)
        {
            float2* ZU = bufs + (size_t)B * BUF;
            for (int f = threadIdx.x; f < F; f += blockDim.x) {
                const float2 P_ = cluster_sum<8>(cluster, Pp, CS, f);
                const float Av = A.Ah[f];
                const float2 U = ZU[f];
                const float inv_s = 1.f / (Av + A.kc);
                const float2 alpha = f2(fmaf(Av, U.x, P_.x) * inv_s, fmaf(Av, U.y, P_.y) * inv_s);
                const float2 W = csub(U, alpha);
                const bool edge = (f == 0) || (f == half);
                if (rank == 0) {
                    const float2 D = f2(fmaf(Av, W.x, P_.x) * sc, fmaf(Av, W.y, P_.y) * sc);
                    if (edge) {
                        ZU[f] = f2(D.x, 0.f);
                    } else {
                        ZU[f] = D;
                        ZU[Lg - f] = f2(D.x, -D.y);
                    }
                }
                repack_X<Lg>(bufs, BUF, B, Mc, F, f, g1, W, sc);
            }
        }
        __syncthreads();

        // ---------------- inverse transforms (rank 0 also transforms DX)
        for (int q = 0; q < Q; ++q) {
            const int sl = grp + q * NG;
            float2* sb = bufs + (size_t)(sl <= B ? sl : 0) * BUF;     // as in the forward pass
            const bool act = sl < B || (sl == B && rank == 0);
            inv_step2<N1, P>(sb, gl, act, tw2);
            if (act) inv_step1<N1, P>(sb, gl);
        }
        __syncthreads();

        // ---------------- store this sequence, load the cluster's next one
        const int nn = n + nclusters;
        streamed(n, nn < A.N ? nn : -1);
        __syncthreads();
    }
    cluster.sync();

    for (int o = 16; o > 0; o >>= 1) absacc += __shfl_xor_sync(0xffffffffu, absacc, o);
    if (lane == 0) red[threadIdx.x >> 5] = absacc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        A.absx_part[blockIdx.x] = t;
    }
}

// ------------------------------------------------------------------ dispatch
typedef void (*kern_t)(WArgs);
// k3: three CTAs per SM, G1h read through L2; k2: two CTAs per SM (more registers),
// the CTA's slice of G1h cached in shared memory
// k2n: two CTAs per SM, G1h read through L2 (for CTAs too large for three per SM)
struct Variant { int N1, P; kern_t k3, k2, k2n; };
const Variant kVariants[] = {
    {32, 29, k_xstep_warp<32, 29, 3, false>, k_xstep_warp<32, 29, 2, true>,
     k_xstep_warp<32, 29, 2, false>},
    {16, 31, k_xstep_warp<16, 31, 3, false>, k_xstep_warp<16, 31, 2, true>,
     k_xstep_warp<16, 31, 2, false>},
};

const Variant* find_variant(int Lg) {
    for (const Variant& v : kVariants)
        if (v.N1 * v.P == Lg) return &v;
    return nullptr;
}

size_t warp_smem(int N1, int P, int slots, int g1s_filters) {
    int Lg = N1 * P, F = Lg / 2 + 1, Fp = (F + 1) & ~1;
    size_t buf = ((size_t)P * (N1 + 1) + 1) & ~(size_t)1;
    return ((size_t)P * N1 + (size_t)slots * buf + 3 * (size_t)Fp) * sizeof(float2) +
           (size_t)Lg * sizeof(float) + (size_t)g1s_filters * F * sizeof(float2);
}

}  // namespace

int warp_variant_exists(int Lg, int M) {
    const Variant* v = find_variant(Lg);
    if (!v) return 0;
    for (int cs : {1, 2, 4, 8})
        if (M % cs == 0 && warp_smem(v->N1, v->P, (M / cs + 1) / 2 + 1, 0) <= 110 * 1024) return 1;
    return 0;
}

struct WarpPlan {
    const Variant* v;
    kern_t k;
    int CS, Mc, B, threads;
    size_t smem;
    int grid;
    float2* tw2;
    double* absx_part;
};

// Picks the smallest cluster whose CTA fits 2 per SM; returns nullptr when the size
// has no register-FFT variant.
void* warp_plan_create(cdlgb_ctx* c, int* status) {
    *status = CDLGB_OK;
    const Variant* v = find_variant(c->Lg);
    if (!v) return nullptr;
    int want_cs = 0;
    if (const char* e = getenv("CDLGB_CLUSTER")) want_cs = atoi(e);
    WarpPlan* P = nullptr;
    // smallest cluster whose slots (B pairs + 1) fit two CTAs per SM with at most 5
    // warps, each lane group transforming ceil(slots / groups) slots; CDLGB_CLUSTER
    // forces a cluster size
    for (int cs : {1, 2, 4, 8}) {
        if (c->M % cs) continue;
        if (want_cs && cs != want_cs) continue;
        int mc = c->M / cs;
        int B = (mc + 1) / 2;
        int G = 32 / v->N1;
        int slots = B + 1;
        int warps = (slots + G - 1) / G;
        if (warps > kMaxThreads / 32) warps = kMaxThreads / 32;
        int threads = warps * 32;
        const size_t sm = warp_smem(v->N1, v->P, slots, 0);        // G1h through L2
        const size_t sm2 = warp_smem(v->N1, v->P, slots, mc);      // G1h slice in shared memory
        const char* ev = getenv("CDLGB_WARP_VARIANT");
        const bool force3 = ev && atoi(ev) == 3;
        // Fewest CTAs per cluster that still fit two per SM: each lane group then
        // transforms more slots per cluster barrier and the U slot is shared by more
        // filters (measured at L=200, K=64: 4-CTA clusters with two slots per group,
        // 10.5 ms per X-step, vs 8-CTA clusters with one, 11.7 ms).
        kern_t k = nullptr;
        size_t bytes = 0;
        if (force3 && sm <= kWarpSmemCap) { k = v->k3; bytes = sm; }       // three per SM
        else if (sm2 <= 110 * 1024) { k = v->k2; bytes = sm2; }            // G1h slice in smem
        else if (sm <= 110 * 1024) { k = v->k2n; bytes = sm; }             // G1h through L2
        if (!k) continue;
        P = new WarpPlan();
        P->v = v; P->CS = cs; P->Mc = mc; P->B = B; P->threads = threads; P->smem = bytes;
        P->k = k;
        break;
    }
    if (!P) return nullptr;
    {
        // the float4 view of y1s needs a 16-byte aligned offset
        int F = c->Lg / 2 + 1, Fp = (F + 1) & ~1;
        size_t buf = ((size_t)v->P * (v->N1 + 1) + 1) & ~(size_t)1;
        size_t off = ((size_t)v->P * v->N1 + (size_t)(P->B + 1) * buf + 3 * (size_t)Fp) * sizeof(float2);
        if (off % 16) {
            delete P;
            *status = cdlgb_seterr(c, CDLGB_ENOTSUP, "register-FFT layout misaligned (internal)");
            return nullptr;
        }
    }
    // tables
    const int N1 = v->N1, Pp = v->P;
    std::vector<float2> tw2 = regfft_twiddles(N1, Pp);
    cudaError_t e = regfft_upload_tables();
    if (e == cudaSuccess) e = dev_copy_in(c, (void**)&P->tw2, tw2.data(), tw2.size() * sizeof(float2));
    // process-wide per kernel: the same cap for every context
    if (e == cudaSuccess) e = cudaFuncSetAttribute(P->k, cudaFuncAttributeMaxDynamicSharedMemorySize, 110 * 1024);
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
        *status = cdlgb_seterr(c, CDLGB_ECUDA, "register-FFT X-step setup failed: %s",
                               e != cudaSuccess ? cudaGetErrorString(e) : "no cluster fits");
        dev_free(c, P->tw2);
        delete P;
        return nullptr;
    }
    if (nclusters > c->N) nclusters = c->N;
    P->grid = nclusters * P->CS;
    e = dev_malloc(c, (void**)&P->absx_part, (size_t)P->grid * sizeof(double));
    if (e != cudaSuccess) {
        *status = cdlgb_seterr(c, CDLGB_ECUDA, "device allocation: %s", cudaGetErrorString(e));
        dev_free(c, P->tw2);
        delete P;
        return nullptr;
    }
    return P;
}

void warp_plan_free(cdlgb_ctx* c, void* p) {
    WarpPlan* P = (WarpPlan*)p;
    if (!P) return;
    dev_free(c, P->tw2);
    dev_free(c, P->absx_part);
    delete P;
}

int warp_plan_cluster(void* p) { return p ? ((WarpPlan*)p)->CS : 0; }
int warp_plan_filters(void* p) { return p ? ((WarpPlan*)p)->Mc : 0; }

int warp_xstep(cdlgb_ctx* c, void* p, const float* Xin, float* Xout) {
    return warp_xstep_n(c, p, Xin, Xout, c->N);
}

// one X-step over the first Nlim sequences (the autotuner times on a prefix)
int warp_xstep_n(cdlgb_ctx* c, void* p, const float* Xin, float* Xout, int Nlim) {
    WarpPlan* P = (WarpPlan*)p;
    WArgs a;
    a.Xin = Xin; a.Xout = Xout; a.y2 = c->y2; a.y3 = c->y3;
    a.Y1 = c->Y1; a.y1 = c->y1; a.DX = c->DX; a.S = c->S;
    a.G1h = c->G1h; a.Ah = c->Ah; a.tw2 = P->tw2; a.absx_part = P->absx_part;
    a.N = Nlim; a.M = c->M; a.F = c->F; a.L4 = c->L4; a.gamma = c->gamma;
    a.lam = c->p.lambda; a.rho = c->p.rho; a.kc = c->p.sherman_const_csc;
    a.Mc = P->Mc; a.B = P->B;
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
    cdlgb_phase_begin(c, PH_XFUSED);
    CU_TRY(c, cudaLaunchKernelEx(&cfg, P->k, a));
    LAUNCH_CHECK(c, "k_xstep_warp");
    cdlgb_phase_end(c, PH_XFUSED);
    return CDLGB_OK;
}

int warp_absx(void* p, const double** part, int* n) {
    WarpPlan* P = (WarpPlan*)p;
    if (!P) return 0;
    *part = P->absx_part;
    *n = P->grid;
    return 1;
}
