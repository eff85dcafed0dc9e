// Fused X-step: one kernel per code_update! iteration (src/CDL/train.jl:5-43).
//
// A thread-block cluster of CS CTAs owns one sequence n at a time (persistent loop
// over sequences); CTA `rank` owns filters [rank*Mc, (rank+1)*Mc).  Per sequence:
//   1. stream X, y2, y3 of its filters from HBM once: shrink!, projectionX!, the
//      dual updates (written back), and V = (Y2 - y2') + (Y3 - y3') packed two real
//      columns per complex sequence in shared memory; U = Y1 - y1' in one extra slot;
//   2. forward FFTs of all slots in shared memory (mixed-radix Stockham, radices
//      8/4/2 and odd primes <= 31);
//   3. split the packed spectra and form this CTA's part of P = sum_m G1h[m] Vh[m];
//   4. cluster barrier, sum the CS partial P's through distributed shared memory
//      (fixed rank order, so every CTA gets bit-identical P), then
//      alpha = (A Uh + P)/(A + k), W = Uh - alpha;
//   5. Xh[m] = (Vh[m] + conj(G1h[m]) W)/(k Lg), repacked; rank 0 also packs
//      DXh = (P + A W)/(k Lg);
//   6. inverse FFTs in shared memory;
//   7. store X (and sum |X| for the objective); rank 0 stores DX, y1' and
//      Y1 = (W'S + rho (DX + y1'))/(W'W + rho)  (update_Y1!, csc_kernels.jl:86-95).
// HBM traffic per X-step is the algorithmic minimum: X, y2, y3 read once, y2, y3,
// X written once, plus the per-sequence vectors.
#include "cdlgb_internal.h"

#include <mutex>

#include <algorithm>

#include <cooperative_groups.h>
#include <math.h>
#include <stdlib.h>
#include <vector>

namespace cg = cooperative_groups;

namespace {

constexpr int kThreads = 256;
constexpr int kMaxFactors = 12;

// cos/sin(2 pi m / p) for the odd primes 3..31, concatenated
__constant__ float2 c_trig[3 + 5 + 7 + 11 + 13 + 17 + 19 + 23 + 29 + 31];

__host__ __device__ constexpr int trig_off(int p) {
    return p == 3 ? 0 : p == 5 ? 3 : p == 7 ? 8 : p == 11 ? 15 : p == 13 ? 26 : p == 17 ? 39
         : p == 19 ? 56 : p == 23 ? 75 : p == 29 ? 98 : p == 31 ? 127 : -1;
}
const int kPrimes[] = {3, 5, 7, 11, 13, 17, 19, 23, 29, 31};

struct FusedPlan {
    int Lg, F;
    int nfac;
    int fac[kMaxFactors];
    int CS, Mc, B;          // cluster size, filters per CTA, packed pairs per CTA
    size_t smem;
    int grid;               // CTAs (multiple of CS)
    float2* tw;             // Lg twiddles exp(-2 pi i t / Lg), device
    double* absx_part;      // one partial sum of |X| per CTA
    void* warp;             // register-FFT variant (xwarp.cu) when Lg has one
    void* iter;             // multi-iteration register-FFT variant (xiter.cu)
    void* dfwd;             // streaming forward transforms of the D-step (dstream.cu)
};

struct XArgs {
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
    const float2* tw;
    double* absx_part;
    int N, M, Lg, F, L4, gamma;
    float lam, rho, kc;
    int Mc, B;
    int nfac;
    int fac[kMaxFactors];
};

__device__ __forceinline__ float2 f2(float x, float y) { return make_float2(x, y); }

// L2 prefetch of the rows the CTA reads for sequence n (its Mc filter rows of X, y2,
// y3; rank 0 also Y1, y1, DX and the W'S window), issued by the 32 lanes of one warp
// while the current sequence is transformed.  Bulk prefetches are hints: nothing waits
// on them.  Every row is a multiple of 16 bytes long (Lg and L4 are multiples of 4
// floats); a base pointer that is not 16-byte aligned skips the hint.
__device__ __forceinline__ void l2_hint(const void* p, unsigned bytes) {
    if (((uintptr_t)p & 15) == 0)
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" :: "l"(p), "r"(bytes) : "memory");
}
__device__ __forceinline__ void prefetch_sequence(const XArgs& A, int n, int m0, int rank, int lane) {
    if (n >= A.N) return;
    const unsigned rb = (unsigned)A.Lg * 4u;
    const size_t r0 = ((size_t)n * A.M + m0) * A.Lg;
    const int rows = 3 * A.Mc, extra = rank == 0 ? 4 : 0;
    for (int q = lane; q < rows + extra; q += 32) {
        if (q < rows) {
            const float* base = q < A.Mc ? A.Xin : q < 2 * A.Mc ? A.y2 : A.y3;
            l2_hint(base + r0 + (size_t)(q % A.Mc) * A.Lg, rb);
        } else if (q < rows + 3) {
            const float* base = q == rows ? A.Y1 : q == rows + 1 ? A.y1 : A.DX;
            l2_hint(base + (size_t)n * A.Lg, rb);
        } else {
            l2_hint(A.S + (size_t)n * A.L4, (unsigned)A.L4 * 4u);
        }
    }
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return f2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return f2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return f2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 c) {  // a*b + c
    return f2(fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y)));
}
__device__ __forceinline__ float2 cjfma(float2 a, float2 b, float2 c) {  // conj(a)*b + c
    return f2(fmaf(a.x, b.x, fmaf(a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(-a.y, b.x, c.y)));
}
// multiply by i*SIGN
template <int SIGN>
__device__ __forceinline__ float2 mul_i(float2 a) {
    return SIGN > 0 ? f2(-a.y, a.x) : f2(a.y, -a.x);
}

// ------------------------------------------------------------------ radix passes
// One Stockham pass (radix R, span p) over `nslots` sequences of length Lg:
// out[s][(i/p)*p*R + k + r*p] = DFT_R( in[s][i + r*Lg/R] * w^(r*k) )_r, k = i mod p,
// w = exp(SIGN 2 pi i / (p R)).  SIGN = -1 forward, +1 inverse (unscaled).
template <int R, int SIGN>
__device__ __forceinline__ void load_twiddled(const float2* __restrict__ src, int NR, int k,
                                              int twstep, const float2* __restrict__ tw,
                                              float2 (&u)[R]) {
#pragma unroll
    for (int r = 0; r < R; ++r) u[r] = src[r * NR];
    if (k) {
#pragma unroll
        for (int r = 1; r < R; ++r) {
            float2 w = tw[r * k * twstep];
            if (SIGN > 0) w.y = -w.y;
            u[r] = cmul(u[r], w);
        }
    }
}

template <int SIGN>
__device__ __forceinline__ void dft4(float2& a0, float2& a1, float2& a2, float2& a3) {
    float2 s02 = cadd(a0, a2), d02 = csub(a0, a2), s13 = cadd(a1, a3), d13 = csub(a1, a3);
    float2 t = mul_i<SIGN>(d13);
    a0 = cadd(s02, s13);
    a2 = csub(s02, s13);
    a1 = cadd(d02, t);
    a3 = csub(d02, t);
}

template <int R, int SIGN>
__device__ void pass_pow2(const float2* __restrict__ in, float2* __restrict__ out, int nslots,
                          int Lg, int p, const float2* __restrict__ tw) {
    const int NR = Lg / R;
    const int total = nslots * NR;
    const int twstep = Lg / (p * R);
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        int s = idx / NR;
        int i = idx - s * NR;
        int q = i / p;
        int k = i - q * p;
        float2 u[R];
        load_twiddled<R, SIGN>(in + (size_t)s * Lg + i, NR, k, twstep, tw, u);
        if (R == 2) {
            float2 a = u[0];
            u[0] = cadd(a, u[1]);
            u[1] = csub(a, u[1]);
        } else if (R == 4) {
            dft4<SIGN>(u[0], u[1], u[2], u[3]);
        } else {  // R == 8: two radix-4 on even/odd, then combine with w8^k
            float2 e0 = u[0], e1 = u[2], e2 = u[4], e3 = u[6];
            float2 o0 = u[1], o1 = u[3], o2 = u[5], o3 = u[7];
            dft4<SIGN>(e0, e1, e2, e3);
            dft4<SIGN>(o0, o1, o2, o3);
            const float h = 0.70710678118654752f;
            float2 w1 = f2(h, SIGN * h), w3 = f2(-h, SIGN * h);
            o1 = cmul(o1, w1);
            o2 = mul_i<SIGN>(o2);
            o3 = cmul(o3, w3);
            u[0] = cadd(e0, o0); u[4] = csub(e0, o0);
            u[1] = cadd(e1, o1); u[5] = csub(e1, o1);
            u[2] = cadd(e2, o2); u[6] = csub(e2, o2);
            u[3] = cadd(e3, o3); u[7] = csub(e3, o3);
        }
        float2* dst = out + (size_t)s * Lg + q * p * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) dst[r * p] = u[r];
    }
}

// odd prime R: pairwise-symmetric DFT (about (R-1)^2 real FMAs per butterfly)
template <int R, int SIGN>
__device__ void pass_odd(const float2* __restrict__ in, float2* __restrict__ out, int nslots,
                         int Lg, int p, const float2* __restrict__ tw) {
    constexpr int H = (R - 1) / 2;
    constexpr int OFF = trig_off(R);
    const int NR = Lg / R;
    const int total = nslots * NR;
    const int twstep = Lg / (p * R);
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        int s = idx / NR;
        int i = idx - s * NR;
        int q = i / p;
        int k = i - q * p;
        const float2* src = in + (size_t)s * Lg + i;
        float2 x0 = src[0];
        float2 sm[H], df[H];
        float2 y0 = x0;
#pragma unroll
        for (int j = 1; j <= H; ++j) {
            float2 a = src[j * NR], b = src[(R - j) * NR];
            if (k) {
                float2 wa = tw[j * k * twstep], wb = tw[(R - j) * k * twstep];
                if (SIGN > 0) { wa.y = -wa.y; wb.y = -wb.y; }
                a = cmul(a, wa);
                b = cmul(b, wb);
            }
            sm[j - 1] = cadd(a, b);
            df[j - 1] = csub(a, b);
            y0 = cadd(y0, sm[j - 1]);
        }
        float2* dst = out + (size_t)s * Lg + q * p * R + k;
        dst[0] = y0;
#pragma unroll
        for (int kk = 1; kk <= H; ++kk) {
            float2 a = x0, b = f2(0.f, 0.f);
#pragma unroll
            for (int j = 1; j <= H; ++j) {
                const float2 cs = c_trig[OFF + (j * kk) % R];
                a.x = fmaf(sm[j - 1].x, cs.x, a.x);
                a.y = fmaf(sm[j - 1].y, cs.x, a.y);
                b.x = fmaf(df[j - 1].x, cs.y, b.x);
                b.y = fmaf(df[j - 1].y, cs.y, b.y);
            }
            float2 ib = mul_i<SIGN>(b);   // y_k = a + SIGN i b, y_{R-k} = a - SIGN i b
            dst[kk * p] = cadd(a, ib);
            dst[(R - kk) * p] = csub(a, ib);
        }
    }
}

template <int SIGN>
__device__ void run_pass(int R, const float2* in, float2* out, int nslots, int Lg, int p,
                         const float2* tw) {
    switch (R) {
        case 2: pass_pow2<2, SIGN>(in, out, nslots, Lg, p, tw); break;
        case 4: pass_pow2<4, SIGN>(in, out, nslots, Lg, p, tw); break;
        case 8: pass_pow2<8, SIGN>(in, out, nslots, Lg, p, tw); break;
        case 3: pass_odd<3, SIGN>(in, out, nslots, Lg, p, tw); break;
        case 5: pass_odd<5, SIGN>(in, out, nslots, Lg, p, tw); break;
        case 7: pass_odd<7, SIGN>(in, out, nslots, Lg, p, tw); break;
        case 11: pass_odd<11, SIGN>(in, out, nslots, Lg, p, tw); break;
        case 13: pass_odd<13, SIGN>(in, out, nslots, Lg, p, tw); break;
        case 17: pass_odd<17, SIGN>(in, out, nslots, Lg, p, tw); break;
        case 19: pass_odd<19, SIGN>(in, out, nslots, Lg, p, tw); break;
        case 23: pass_odd<23, SIGN>(in, out, nslots, Lg, p, tw); break;
        case 29: pass_odd<29, SIGN>(in, out, nslots, Lg, p, tw); break;
        case 31: pass_odd<31, SIGN>(in, out, nslots, Lg, p, tw); break;
        default: break;
    }
}

// all passes, ping-ponging between a and b; returns the buffer holding the result
template <int SIGN>
__device__ float2* fft_all(float2* a, float2* b, int nslots, int Lg, const int* fac, int nfac,
                           const float2* tw) {
    int p = 1;
    for (int t = 0; t < nfac; ++t) {
        run_pass<SIGN>(fac[t], a, b, nslots, Lg, p, tw);
        __syncthreads();
        float2* c = a; a = b; b = c;
        p *= fac[t];
    }
    return a;
}

__device__ __forceinline__ void xprep1(float x, float a, float b, float lam, bool keep,
                                       float& na, float& nb, float& v) {
    float t = x + a;                                        // X + y2
    // shrink! (csc_kernels.jl:53-64) at lambda, not lambda / rho (REF_QUIRK_Q4, :61)
    float Y2 = copysignf(fmaxf(fabsf(t) - lam, 0.f), t);
    float Y3 = keep ? x + b : 0.f;                          // projectionX! (:68-82)
    na = (a + x) - Y2;                                      // train.jl:13
    nb = (b + x) - Y3;                                      // train.jl:14
    v = (Y2 - na) + (Y3 - nb);
}
__device__ __forceinline__ void xprep4(float4 x, float4 a, float4 b, float lam, float4& na,
                                       float4& nb, float4& v) {
    xprep1(x.x, a.x, b.x, lam, true, na.x, nb.x, v.x);   // .x is on the 4-stride
    xprep1(x.y, a.y, b.y, lam, false, na.y, nb.y, v.y);
    xprep1(x.z, a.z, b.z, lam, false, na.z, nb.z, v.z);
    xprep1(x.w, a.w, b.w, lam, false, na.w, nb.w, v.w);
}

__global__ void __launch_bounds__(kThreads, 2) k_xstep_fused(XArgs A) {
    extern __shared__ float4 smem4[];
    cg::cluster_group cluster = cg::this_cluster();
    const int CS = (int)cluster.num_blocks();
    const int rank = (int)cluster.block_rank();
    const int cid = blockIdx.x / CS;
    const int nclusters = gridDim.x / CS;
    const int Lg = A.Lg, F = A.F, B = A.B, Mc = A.Mc, M = A.M;
    const int NS = B + 1;                      // packed filter pairs + the U / DX slot
    const int Lg4 = Lg >> 2;
    const int half = Lg >> 1;

    float2* bufA = reinterpret_cast<float2*>(smem4);
    float2* bufB = bufA + (size_t)NS * Lg;
    float2* tws = bufB + (size_t)NS * Lg;
    const int Fp = (F + 1) & ~1;               // keeps the float4 view of y1s aligned
    float2* Ppart = tws + Lg;                  // [2][Fp], double-buffered by sequence parity
    float2* Wv = Ppart + 2 * Fp;
    float* y1s = reinterpret_cast<float*>(Wv + Fp);
    __shared__ double red[kThreads / 32];

    __shared__ int fac[kMaxFactors];
    for (int t = threadIdx.x; t < Lg; t += blockDim.x) tws[t] = A.tw[t];
    if (threadIdx.x < kMaxFactors) fac[threadIdx.x] = A.fac[threadIdx.x];
    __syncthreads();

    const int m0 = rank * Mc;
    const float sc = 1.f / (A.kc * (float)Lg);
    double absacc = 0.0;
    int it = 0;
    for (int n = cid; n < A.N; n += nclusters, ++it) {
        // ---- 1. elementwise pass over this CTA's columns, packed into bufA
        for (int idx = threadIdx.x; idx < B * Lg4; idx += blockDim.x) {
            int j = idx / Lg4;
            int l4 = idx - j * Lg4;
            const int ma = m0 + 2 * j;
            bool hasb = (2 * j + 1) < Mc;
            size_t ba = ((size_t)n * M + ma) * Lg + 4 * (size_t)l4;
            size_t bb = ba + Lg;
            float4 xa = reinterpret_cast<const float4*>(A.Xin + ba)[0];
            float4 aa = reinterpret_cast<const float4*>(A.y2 + ba)[0];
            float4 ca = reinterpret_cast<const float4*>(A.y3 + ba)[0];
            float4 xb = make_float4(0, 0, 0, 0), ab = xb, cb = xb;
            if (hasb) {
                xb = reinterpret_cast<const float4*>(A.Xin + bb)[0];
                ab = reinterpret_cast<const float4*>(A.y2 + bb)[0];
                cb = reinterpret_cast<const float4*>(A.y3 + bb)[0];
            }
            float4 na, nb, va, vb;
            xprep4(xa, aa, ca, A.lam, na, nb, va);
            reinterpret_cast<float4*>(A.y2 + ba)[0] = na;
            reinterpret_cast<float4*>(A.y3 + ba)[0] = nb;
            if (hasb) {
                xprep4(xb, ab, cb, A.lam, na, nb, vb);
                reinterpret_cast<float4*>(A.y2 + bb)[0] = na;
                reinterpret_cast<float4*>(A.y3 + bb)[0] = nb;
            } else {
                vb = make_float4(0, 0, 0, 0);
            }
            float4* z = reinterpret_cast<float4*>(bufA + (size_t)j * Lg + 4 * l4);
            z[0] = make_float4(va.x, vb.x, va.y, vb.y);
            z[1] = make_float4(va.z, vb.z, va.w, vb.w);
        }
        // U = Y1 - y1', y1' = y1 + DX - Y1 (train.jl:12), into slot B
        for (int l4 = threadIdx.x; l4 < Lg4; l4 += blockDim.x) {
            size_t o = (size_t)n * Lg + 4 * (size_t)l4;
            float4 Yv = reinterpret_cast<const float4*>(A.Y1 + o)[0];
            float4 yv = reinterpret_cast<const float4*>(A.y1 + o)[0];
            float4 dv = reinterpret_cast<const float4*>(A.DX + o)[0];
            float4 yn = make_float4((yv.x + dv.x) - Yv.x, (yv.y + dv.y) - Yv.y,
                                    (yv.z + dv.z) - Yv.z, (yv.w + dv.w) - Yv.w);
            float4* z = reinterpret_cast<float4*>(bufA + (size_t)B * Lg + 4 * l4);
            z[0] = make_float4(Yv.x - yn.x, 0.f, Yv.y - yn.y, 0.f);
            z[1] = make_float4(Yv.z - yn.z, 0.f, Yv.w - yn.w, 0.f);
            if (rank == 0) reinterpret_cast<float4*>(y1s)[l4] = yn;
        }
        __syncthreads();

        // the next sequence's rows into L2 while this one is transformed
        if (threadIdx.x >= 32 && threadIdx.x < 64)
            prefetch_sequence(A, n + nclusters, m0, rank, threadIdx.x & 31);

        // ---- 2. forward FFTs
        float2* R = fft_all<-1>(bufA, bufB, NS, Lg, fac, A.nfac, tws);
        float2* other = (R == bufA) ? bufB : bufA;

        // ---- 3. split packed spectra, partial P over this CTA's filters
        float2* Pp = Ppart + (it & 1) * Fp;
        for (int f = threadIdx.x; f < F; f += blockDim.x) {
            float2 P = f2(0.f, 0.f);
            bool edge = (f == 0) || (f == half);
            for (int j = 0; j < B; ++j) {
                float2* Z = R + (size_t)j * Lg;
                float2 va, vb;
                if (edge) {
                    float2 z = Z[f];
                    va = f2(z.x, 0.f);
                    vb = f2(z.y, 0.f);
                } else {
                    float2 z1 = Z[f], z2 = Z[Lg - f];
                    va = f2(0.5f * (z1.x + z2.x), 0.5f * (z1.y - z2.y));
                    vb = f2(0.5f * (z1.y + z2.y), 0.5f * (z2.x - z1.x));
                    Z[f] = va;
                    Z[Lg - f] = vb;
                }
                int ma = m0 + 2 * j;
                P = cfma(A.G1h[(size_t)ma * F + f], va, P);
                if (2 * j + 1 < Mc) P = cfma(A.G1h[(size_t)(ma + 1) * F + f], vb, P);
            }
            Pp[f] = P;
        }
        cluster.sync();

        // ---- 4. full P from every CTA of the cluster, then alpha and W
        for (int f = threadIdx.x; f < F; f += blockDim.x) {
            float2 P = f2(0.f, 0.f);
            for (int r = 0; r < CS; ++r) {
                const float2* rp = cluster.map_shared_rank(Pp, r);
                P = cadd(P, rp[f]);
            }
            float Av = A.Ah[f];
            float2 U = R[(size_t)B * Lg + f];
            float inv_s = 1.f / (Av + A.kc);
            float2 alpha = f2(fmaf(Av, U.x, P.x) * inv_s, fmaf(Av, U.y, P.y) * inv_s);
            float2 W = csub(U, alpha);
            Wv[f] = W;
            if (rank == 0) {
                // DXh = (P + A W)/k, scaled by 1/Lg, packed as a Hermitian spectrum
                float2 D = f2(fmaf(Av, W.x, P.x) * sc, fmaf(Av, W.y, P.y) * sc);
                float2* Z = R + (size_t)B * Lg;
                if (f == 0 || f == half) {
                    Z[f] = f2(D.x, 0.f);
                } else {
                    Z[f] = D;
                    Z[Lg - f] = f2(D.x, -D.y);
                }
            }
        }
        __syncthreads();

        // ---- 5. Xh = (Vh + conj(G1h) W)/(k Lg), repacked two per complex sequence
        for (int f = threadIdx.x; f < F; f += blockDim.x) {
            float2 W = Wv[f];
            bool edge = (f == 0) || (f == half);
            for (int j = 0; j < B; ++j) {
                float2* Z = R + (size_t)j * Lg;
                int ma = m0 + 2 * j;
                bool hasb = 2 * j + 1 < Mc;
                float2 ga = A.G1h[(size_t)ma * F + f];
                float2 gb = hasb ? A.G1h[(size_t)(ma + 1) * F + f] : f2(0.f, 0.f);
                float2 va, vb;
                if (edge) {
                    float2 z = Z[f];
                    va = f2(z.x, 0.f);
                    vb = f2(z.y, 0.f);
                } else {
                    va = Z[f];
                    vb = Z[Lg - f];
                }
                float2 xa = cjfma(ga, W, va);
                float2 xb = hasb ? cjfma(gb, W, vb) : f2(0.f, 0.f);
                xa = f2(__fmul_rn(xa.x, sc), __fmul_rn(xa.y, sc));
                xb = f2(__fmul_rn(xb.x, sc), __fmul_rn(xb.y, sc));
                if (edge) {
                    Z[f] = f2(xa.x, xb.x);
                } else {
                    Z[f] = f2(xa.x - xb.y, xa.y + xb.x);
                    Z[Lg - f] = f2(xa.x + xb.y, xb.x - xa.y);
                }
            }
        }
        __syncthreads();

        // ---- 6. inverse FFTs (rank 0 also transforms DX in slot B)
        float2* Xr = fft_all<1>(R, other, rank == 0 ? NS : B, Lg, fac, A.nfac, tws);

        // ---- 7. store X; rank 0 stores DX, y1', Y1
        for (int idx = threadIdx.x; idx < B * Lg4; idx += blockDim.x) {
            int j = idx / Lg4;
            int l4 = idx - j * Lg4;
            int ma = m0 + 2 * j;
            const float4* z = reinterpret_cast<const float4*>(Xr + (size_t)j * Lg + 4 * l4);
            float4 z0 = z[0], z1 = z[1];
            float4 xa = make_float4(z0.x, z0.z, z1.x, z1.z);
            float4 xb = make_float4(z0.y, z0.w, z1.y, z1.w);
            size_t ba = ((size_t)n * M + ma) * Lg + 4 * (size_t)l4;
            reinterpret_cast<float4*>(A.Xout + ba)[0] = xa;
            float s = (fabsf(xa.x) + fabsf(xa.y)) + (fabsf(xa.z) + fabsf(xa.w));
            if (2 * j + 1 < Mc) {
                reinterpret_cast<float4*>(A.Xout + ba + Lg)[0] = xb;
                s += (fabsf(xb.x) + fabsf(xb.y)) + (fabsf(xb.z) + fabsf(xb.w));
            }
            absacc += (double)s;
        }
        if (rank == 0) {
            for (int l4 = threadIdx.x; l4 < Lg4; l4 += blockDim.x) {
                const float4* z = reinterpret_cast<const float4*>(Xr + (size_t)B * Lg + 4 * l4);
                float4 z0 = z[0], z1 = z[1];
                float dx[4] = {z0.x, z0.z, z1.x, z1.z};
                float4 yn4 = reinterpret_cast<const float4*>(y1s)[l4];
                float yn[4] = {yn4.x, yn4.y, yn4.z, yn4.w};
                float Yo[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    int l = 4 * l4 + e;
                    bool in = l >= A.gamma && l < A.gamma + A.L4;
                    float wts = in ? A.S[(size_t)n * A.L4 + (l - A.gamma)] : 0.f;
                    float dg = in ? 1.f : 0.f;
                    Yo[e] = __fadd_rn(wts, __fmul_rn(A.rho, dx[e] + yn[e])) / (dg + A.rho);
                }
                size_t o = (size_t)n * Lg + 4 * (size_t)l4;
                reinterpret_cast<float4*>(A.DX + o)[0] = make_float4(dx[0], dx[1], dx[2], dx[3]);
                reinterpret_cast<float4*>(A.y1 + o)[0] = yn4;
                reinterpret_cast<float4*>(A.Y1 + o)[0] = make_float4(Yo[0], Yo[1], Yo[2], Yo[3]);
            }
        }
        __syncthreads();
    }
    // keep this CTA's shared memory alive until every CTA of the cluster is done reading it
    cluster.sync();

    for (int o = 16; o > 0; o >>= 1) absacc += __shfl_xor_sync(0xffffffffu, absacc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = absacc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        A.absx_part[blockIdx.x] = t;
    }
}

// ------------------------------------------------------------------ host side
// The radices of the Stockham passes, the odd primes first: a pass of radix R and span
// p stores element r of a butterfly at q p R + k + r p, so the first pass (p = 1)
// stores with stride R, which is free of shared-memory bank conflicts for an odd R and
// 8-way conflicted for R = 8; with the powers of two last their spans are large.
bool factorize(int Lg, int* fac, int* nfac) {
    int n = Lg, k = 0, twos = 0;
    while (n % 2 == 0) { n /= 2; ++twos; }
    for (int p : kPrimes) {
        while (n % p == 0) {
            if (k >= kMaxFactors) return false;
            fac[k++] = p;
            n /= p;
        }
    }
    if (n != 1) return false;
    if (twos % 3 == 2) { if (k >= kMaxFactors) return false; fac[k++] = 4; }
    else if (twos % 3 == 1) { if (k >= kMaxFactors) return false; fac[k++] = 2; }
    for (; twos >= 3; twos -= 3) { if (k >= kMaxFactors) return false; fac[k++] = 8; }
    *nfac = k;
    return true;
}

size_t smem_bytes(int Lg, int F, int Mc) {
    int B = (Mc + 1) / 2;
    size_t NS = B + 1;
    size_t Fp = (F + 1) & ~1;
    return (2 * NS * Lg + Lg + 3 * Fp) * sizeof(float2) + (size_t)Lg * sizeof(float);
}

// Two CTAs per SM.  Longer transforms whose layout needs one CTA per SM (Lg = 2128 at
// K = 32 fits 216 KB at four CTAs per cluster) ran slower on this kernel than on the
// cuFFT-transform path (100 against 82 ms per outer iteration at N = 5000), so they
// are left to that path.
constexpr size_t kSmemCap = 110 * 1024;

// The smallest cluster whose CTAs fit two per SM; CDLGB_CLUSTER forces a cluster size
// (when it fits), as for the register-FFT kernels.
bool choose_cluster(int Lg, int M, int* CS, int* Mc) {
    int F = Lg / 2 + 1;
    int want = 0;
    if (const char* e = getenv("CDLGB_CLUSTER")) want = atoi(e);
    for (int cs : {1, 2, 4, 8}) {
        if (M % cs || (want && cs != want)) continue;
        int mc = M / cs;
        if (smem_bytes(Lg, F, mc) <= kSmemCap) { *CS = cs; *Mc = mc; return true; }
    }
    return false;
}

}  // namespace

// A fused X-step exists for Lg and M (L4 = Lg minus the two margins): the multi-iteration
// kernel, the one-X-step kernel, or the generic in-kernel-FFT kernel.
int fused_supported(int Lg, int M, int L4) {
    int fac[kMaxFactors], nf = 0, cs = 0, mc = 0;
    if (iter_variant_fits(Lg, M, L4)) return 1;
    if (warp_variant_exists(Lg, M)) return 1;
    if (Lg % 4) return 0;
    if (!factorize(Lg, fac, &nf)) return 0;
    if (!choose_cluster(Lg, M, &cs, &mc)) return 0;
    return 1;
}

size_t fused_scratch_bytes(int Lg, int M, int N) {
    (void)M; (void)N;
    return (size_t)Lg * 8 + 152 * 8 * 8 * sizeof(double);
}

// The odd primes' trig table in constant memory, uploaded once per device: every
// context reads the same values, and a context's setup must not write the table under
// another context's kernels.
static cudaError_t upload_trig_once() {
    static std::mutex mu;
    static bool done[64];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    if (dev >= 0 && dev < 64 && done[dev]) return cudaSuccess;
    std::vector<float2> trig(3 + 5 + 7 + 11 + 13 + 17 + 19 + 23 + 29 + 31);
    for (int p : kPrimes)
        for (int m = 0; m < p; ++m)
            trig[trig_off(p) + m] = make_float2((float)cos(2.0 * M_PI * m / p), (float)sin(2.0 * M_PI * m / p));
    e = cudaMemcpyToSymbol(c_trig, trig.data(), trig.size() * sizeof(float2));
    // the copy may return before it lands; the contexts' streams do not wait on the
    // legacy stream, so wait for it there
    if (e == cudaSuccess) e = cudaStreamSynchronize(0);
    if (e == cudaSuccess && dev >= 0 && dev < 64) done[dev] = true;
    return e;
}

int fused_setup(cdlgb_ctx* c) {
    FusedPlan* P = new FusedPlan();
    c->fplan = P;
    P->Lg = c->Lg;
    P->F = c->F;
    if (!getenv("CDLGB_GENERIC_FFT")) {
        int st = CDLGB_OK;
        P->dfwd = dfwd_plan_create(c, &st);
        if (st != CDLGB_OK) return st;
        P->iter = iter_plan_create(c, &st);
        if (st != CDLGB_OK) return st;
        if (P->iter) return CDLGB_OK;
        P->warp = warp_plan_create(c, &st);
        if (st != CDLGB_OK) return st;
        if (P->warp) return CDLGB_OK;
    }
    if (!factorize(c->Lg, P->fac, &P->nfac) || !choose_cluster(c->Lg, c->M, &P->CS, &P->Mc))
        return cdlgb_seterr(c, CDLGB_ENOTSUP, "fused path: unsupported Lg=%d / M=%d", c->Lg, c->M);
    for (int t = P->nfac; t < kMaxFactors; ++t) P->fac[t] = 1;
    P->B = (P->Mc + 1) / 2;
    P->smem = smem_bytes(P->Lg, P->F, P->Mc);
    // trig tables of the odd primes, twiddles exp(-2 pi i t / Lg), in double then rounded
    CU_TRY(c, upload_trig_once());
    std::vector<float2> tw(P->Lg);
    for (int t = 0; t < P->Lg; ++t)
        tw[t] = make_float2((float)cos(2.0 * M_PI * t / P->Lg), (float)-sin(2.0 * M_PI * t / P->Lg));
    CU_TRY(c, dev_copy_in(c, (void**)&P->tw, tw.data(), P->Lg * sizeof(float2)));
    // the attribute is process-wide per kernel: always the same cap, never a
    // context's own size (contexts with different Lg run concurrently)
    CU_TRY(c, cudaFuncSetAttribute(k_xstep_fused, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)kSmemCap));
    // persistent grid: as many clusters as can be resident at once (at most one per sequence)
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = P->CS;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(P->CS * 152 * 4, 1, 1);
    cfg.blockDim = dim3(kThreads, 1, 1);
    cfg.dynamicSmemBytes = P->smem;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    CU_TRY(c, cudaOccupancyMaxActiveClusters(&nclusters, (void*)k_xstep_fused, &cfg));
    if (nclusters < 1)
        return cdlgb_seterr(c, CDLGB_ENOTSUP, "fused path: no cluster of %d CTAs with %zu B fits",
                            P->CS, P->smem);
    if (nclusters > c->N) nclusters = c->N;
    P->grid = nclusters * P->CS;
    ST_TRY(dev_alloc(c, (void**)&P->absx_part, (size_t)P->grid * sizeof(double)));
    return CDLGB_OK;
}

void fused_free(cdlgb_ctx* c) {
    FusedPlan* P = (FusedPlan*)c->fplan;
    if (!P) return;
    dev_free(c, P->tw);
    dev_free(c, P->absx_part);
    warp_plan_free(c, P->warp);
    iter_plan_free(c, P->iter);
    dfwd_plan_free(c, P->dfwd);
    delete P;
    c->fplan = nullptr;
}

int fused_has_multi(cdlgb_ctx* c) {
    FusedPlan* P = (FusedPlan*)c->fplan;
    return P && P->iter;
}

int fused_xsteps(cdlgb_ctx* c, const float* Xin, float* Xout, int iters) {
    FusedPlan* P = (FusedPlan*)c->fplan;
    return iter_xsteps(c, P->iter, Xin, Xout, iters);
}

int fused_xstep(cdlgb_ctx* c, const float* Xin, float* Xout, int accum_abs) {
    (void)accum_abs;
    FusedPlan* P = (FusedPlan*)c->fplan;
    if (P->iter) return iter_xsteps(c, P->iter, Xin, Xout, 1);
    if (P->warp) return warp_xstep(c, P->warp, Xin, Xout);
    XArgs a;
    a.Xin = Xin; a.Xout = Xout; a.y2 = c->y2; a.y3 = c->y3;
    a.Y1 = c->Y1; a.y1 = c->y1; a.DX = c->DX; a.S = c->S;
    a.G1h = c->G1h; a.Ah = c->Ah; a.tw = P->tw; a.absx_part = P->absx_part;
    a.N = c->N; a.M = c->M; a.Lg = c->Lg; a.F = c->F; a.L4 = c->L4; a.gamma = c->gamma;
    a.lam = c->p.lambda; a.rho = c->p.rho; a.kc = c->p.sherman_const_csc;
    a.Mc = P->Mc; a.B = P->B; a.nfac = P->nfac;
    for (int t = 0; t < kMaxFactors; ++t) a.fac[t] = P->fac[t];
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = P->CS;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(P->grid, 1, 1);
    cfg.blockDim = dim3(kThreads, 1, 1);
    cfg.dynamicSmemBytes = P->smem;
    cfg.stream = c->stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cdlgb_phase_begin(c, PH_XFUSED);
    CU_TRY(c, cudaLaunchKernelEx(&cfg, k_xstep_fused, a));
    LAUNCH_CHECK(c, "k_xstep_fused");
    cdlgb_phase_end(c, PH_XFUSED);
    return CDLGB_OK;
}

void* fused_dfwd(cdlgb_ctx* c) {
    FusedPlan* P = (FusedPlan*)c->fplan;
    return P ? P->dfwd : nullptr;
}

// The X-step autotuner: every register-FFT X-step variant that fits (multi-iteration
// kernels with each filters-per-CTA choice, and the one-X-step kernel) is timed with
// CUDA events on a prefix of the loaded sequences (the state of that prefix is saved
// before and restored after every run), and the fastest is kept for this context.
int fused_autotune(cdlgb_ctx* c, int maxc, double* ms, int32_t* kind, int32_t* cs, int32_t* mc,
                   int32_t* n_out, int32_t* chosen) {
    FusedPlan* P = (FusedPlan*)c->fplan;
    if (!P || (!P->iter && !P->warp))
        return cdlgb_seterr(c, CDLGB_ENOTSUP, "autotune: no register-FFT X-step for Lg=%d", c->Lg);
    struct Cand { int kind; void* plan; };
    std::vector<Cand> cands;
    auto free_all = [&](int keep) {
        for (int i = 0; i < (int)cands.size(); ++i) {
            if (i == keep) continue;
            if (cands[i].kind == 1) iter_plan_free(c, cands[i].plan);
            else warp_plan_free(c, cands[i].plan);
        }
    };
    int st = CDLGB_OK;
    for (int nth = 0;; ++nth) {
        void* ip = iter_plan_create_nth(c, nth, 0, &st);
        if (st != CDLGB_OK) { free_all(-1); return st; }
        if (!ip) break;
        cands.push_back({1, ip});
    }
    {
        void* wp = warp_plan_create(c, &st);
        if (st != CDLGB_OK) { free_all(-1); return st; }
        if (wp) cands.push_back({2, wp});
    }
    if (cands.empty()) return cdlgb_seterr(c, CDLGB_ENOTSUP, "autotune: no candidate");
    if ((int)cands.size() > maxc) {
        free_all(-1);
        return cdlgb_seterr(c, CDLGB_EINVAL, "autotune: %zu candidates, room for %d", cands.size(), maxc);
    }
    // the prefix of sequences the candidates are timed on
    int maxcl = 1;
    for (const Cand& k : cands) {
        const int cl = k.kind == 1 ? iter_plan_grid(k.plan) / iter_plan_cluster(k.plan) : 0;
        maxcl = std::max(maxcl, cl);
    }
    // 64 sequences per cluster of the largest grid (the steady state of a persistent
    // grid, not its start-up), the saved state of the prefix at most 1 GB
    const size_t per_seq = ((size_t)3 * c->M + 3) * c->Lg * sizeof(float);
    const int Nl = (int)std::min<size_t>({(size_t)c->N, (size_t)64 * maxcl,
                                          std::max<size_t>(1, ((size_t)1 << 30) / per_seq)});
    const size_t lmn = (size_t)Nl * c->M * c->Lg, ln = (size_t)Nl * c->Lg;
    float* X = c->Xb[c->xcur];
    float* snap = nullptr;
    cudaStream_t s = c->stream;
    CU_TRY(c, cudaMallocAsync((void**)&snap, (3 * lmn + 3 * ln) * sizeof(float), s));
    float* src[6] = {X, c->y2, c->y3, c->Y1, c->y1, c->DX};
    const size_t cnt[6] = {lmn, lmn, lmn, ln, ln, ln};
    size_t off[6];
    {
        size_t o = 0;
        for (int i = 0; i < 6; ++i) { off[i] = o; o += cnt[i]; }
    }
    auto copy = [&](bool save) -> int {
        for (int i = 0; i < 6; ++i) {
            float* a = save ? snap + off[i] : src[i];
            const float* b = save ? src[i] : snap + off[i];
            CU_TRY(c, cudaMemcpyAsync(a, b, cnt[i] * sizeof(float), cudaMemcpyDeviceToDevice, s));
        }
        return CDLGB_OK;
    };
    auto run = [&](const Cand& k, int iters) -> int {
        if (k.kind == 1) return iter_xsteps_n(c, k.plan, X, X, iters, Nl);
        for (int it = 0; it < iters; ++it) ST_TRY(warp_xstep_n(c, k.plan, X, X, Nl));
        return CDLGB_OK;
    };
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int best = -1;
    double best_ms = 0.0;
    int rc = copy(true);
    if (rc == CDLGB_OK && cudaEventCreate(&e0) != cudaSuccess) rc = cdlgb_seterr(c, CDLGB_ECUDA, "event");
    if (rc == CDLGB_OK && cudaEventCreate(&e1) != cudaSuccess) rc = cdlgb_seterr(c, CDLGB_ECUDA, "event");
    // as many X-steps as a code update runs: the multi-iteration kernel loads and
    // stores the state once per launch
    const int kIters = std::max(1, (int)c->p.csc_iter_num);
    for (int i = 0; rc == CDLGB_OK && i < (int)cands.size(); ++i) {
        rc = run(cands[i], 1);                           // warm-up
        if (rc == CDLGB_OK) rc = copy(false);
        if (rc == CDLGB_OK) cudaEventRecord(e0, s);
        if (rc == CDLGB_OK) rc = run(cands[i], kIters);
        if (rc == CDLGB_OK) cudaEventRecord(e1, s);
        if (rc == CDLGB_OK && cudaEventSynchronize(e1) != cudaSuccess)
            rc = cdlgb_seterr(c, CDLGB_ECUDA, "autotune: %s", cudaGetErrorString(cudaGetLastError()));
        float t = 0.f;
        if (rc == CDLGB_OK) cudaEventElapsedTime(&t, e0, e1);
        if (rc == CDLGB_OK) rc = copy(false);
        const double per = (double)t / kIters;
        ms[i] = per;
        kind[i] = cands[i].kind;
        cs[i] = cands[i].kind == 1 ? iter_plan_cluster(cands[i].plan) : warp_plan_cluster(cands[i].plan);
        mc[i] = cands[i].kind == 1 ? iter_plan_filters(cands[i].plan) : warp_plan_filters(cands[i].plan);
        if (rc == CDLGB_OK && (best < 0 || per < best_ms)) { best = i; best_ms = per; }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFreeAsync(snap, s);
    if (rc != CDLGB_OK) { free_all(-1); return rc; }
    CU_TRY(c, cudaStreamSynchronize(s));
    // keep the winner
    iter_plan_free(c, P->iter);
    warp_plan_free(c, P->warp);
    P->iter = nullptr;
    P->warp = nullptr;
    if (cands[best].kind == 1) P->iter = cands[best].plan;
    else P->warp = cands[best].plan;
    free_all(best);
    c->absx_fused = 0;           // the partial sums of |X| belong to the timing runs
    *n_out = (int32_t)cands.size();
    *chosen = best;
    return CDLGB_OK;
}

// the X-step residual partials of the last multi-iteration launch (five per CTA)
int fused_resid(cdlgb_ctx* c, const double** part, int* n) {
    FusedPlan* P = (FusedPlan*)c->fplan;
    if (!P || !P->iter) return 0;
    return iter_resid(P->iter, part, n);
}

// partial sums of |X| written by the last fused X-step (one per CTA)
int fused_absx(cdlgb_ctx* c, const double** part, int* n) {
    FusedPlan* P = (FusedPlan*)c->fplan;
    if (!P) return 0;
    if (P->iter) return iter_absx(P->iter, part, n);
    if (P->warp) return warp_absx(P->warp, part, n);
    *part = P->absx_part;
    *n = P->grid;
    return 1;
}
