// Fused X-step with register-resident four-step FFTs (Lg = N1 * P, N1 in {16, 32}
// lanes, P an odd prime).  Same algebra and cluster structure as the generic fused
// kernel (fused.cu), but each packed column pair (and the U / DX slot) is owned by a
// group of N1 lanes that transforms it without block-wide barriers:
//   forward  x[n1 + N1 n2] (lane n1 holds n2 = 0..P-1)
//     1. DFT-P over n2 in registers (pairwise-symmetric form), twiddle w_Lg^(n1 k2),
//        write T[k2][n1] (row stride N1+1: conflict-free both ways);
//     2. lane j takes rows r = j + N1 q: DFT-N1 in registers (radix-2 DIF) gives
//        X[r + P k1], written in natural order into the same buffer.
//   inverse  the same steps backwards (inverse DFT-N1 per row, conjugate twiddles,
//     transpose, inverse DFT-P per lane, results streamed to HBM).
// The block-wide phases between the transforms (split of the packed spectra,
// cross-filter sums, Sherman-Morrison combine) read and write the spectra in shared
// memory; the cross-filter sum over the cluster goes through distributed shared
// memory in fixed rank order.
#include "cdlgb_internal.h"

#include <cooperative_groups.h>
#include <math.h>
#include <stdlib.h>
#include <vector>

namespace cg = cooperative_groups;

namespace {

constexpr int kMaxThreads = 160;
constexpr size_t kWarpSmemCap = 72 * 1024;   // three CTAs per SM

// cos/sin(2 pi m / p) for the odd primes 3..31, concatenated; exp(-2 pi i j / 32)
__constant__ float2 c_trigw[3 + 5 + 7 + 11 + 13 + 17 + 19 + 23 + 29 + 31];
__constant__ float2 c_w32[32];

__host__ __device__ constexpr int toff(int p) {
    return p == 3 ? 0 : p == 5 ? 3 : p == 7 ? 8 : p == 11 ? 15 : p == 13 ? 26 : p == 17 ? 39
         : p == 19 ? 56 : p == 23 ? 75 : p == 29 ? 98 : p == 31 ? 127 : -1;
}
const int kPrimesW[] = {3, 5, 7, 11, 13, 17, 19, 23, 29, 31};

__host__ __device__ constexpr int brev(int k, int bits) {
    int r = 0;
    for (int b = 0; b < bits; ++b) r |= ((k >> b) & 1) << (bits - 1 - b);
    return r;
}
__host__ __device__ constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n / 2); }

__device__ __forceinline__ float2 f2(float x, float y) { return make_float2(x, y); }
// Blackwell packed FP32x2 arithmetic (one instruction for both halves, IEEE-identical
// to the two scalar operations); the pairs are formed inside the asm so that the
// register allocator can keep them as adjacent registers
__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
    float2 r;
    asm("{\n\t.reg .b64 pa, pb, pd;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "add.rn.f32x2 pd, pa, pb;\n\tmov.b64 {%0, %1}, pd;\n\t}"
        : "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
    float2 r;
    asm("{\n\t.reg .b64 pa, pb, pd;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "sub.rn.f32x2 pd, pa, pb;\n\tmov.b64 {%0, %1}, pd;\n\t}"
        : "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
// a * (c, c) + b  for a complex a and a real c
__device__ __forceinline__ float2 rfma(float2 a, float c, float2 b) {
    float2 r;
    asm("{\n\t.reg .b64 pa, pc, pb, pd;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pc, {%4, %4};\n\t"
        "mov.b64 pb, {%5, %6};\n\tfma.rn.f32x2 pd, pa, pc, pb;\n\tmov.b64 {%0, %1}, pd;\n\t}"
        : "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(c), "f"(b.x), "f"(b.y));
    return r;
}
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return f2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {  // a * conj(b)
    return f2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}
// a*b + c = b*a.x + (-b.y, b.x)*a.y + c, two packed FMAs
__device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 c) {
    return rfma(f2(-b.y, b.x), a.y, rfma(b, a.x, c));
}
// conj(a)*b + c = b*a.x + (b.y, -b.x)*a.y + c
__device__ __forceinline__ float2 cjfma(float2 a, float2 b, float2 c) {
    return rfma(f2(b.y, -b.x), a.y, rfma(b, a.x, c));
}
template <int SIGN>
__device__ __forceinline__ float2 mul_i(float2 a) {  // SIGN * i * a
    return SIGN > 0 ? f2(-a.y, a.x) : f2(a.y, -a.x);
}

// in-register radix-2 DIF DFT of length N (16 or 32); X[k] ends in x[brev(k)]
template <int N, int SIGN>
__device__ __forceinline__ void dft_reg(float2 (&x)[N]) {
    constexpr int LOG = ilog2c(N);
#pragma unroll
    for (int st = 0; st < LOG; ++st) {
        const int span = N >> (st + 1);
#pragma unroll
        for (int blk = 0; blk < N; blk += 2 * span) {
#pragma unroll
            for (int j = 0; j < span; ++j) {
                float2 a = x[blk + j], b = x[blk + j + span];
                x[blk + j] = cadd(a, b);
                float2 t = csub(a, b);
                if (j == 0) {
                    x[blk + j + span] = t;
                } else if (4 * j == 2 * span) {          // w = SIGN * i
                    x[blk + j + span] = mul_i<SIGN>(t);
                } else {
                    float2 w = c_w32[j * (32 / (2 * span))];
                    x[blk + j + span] = SIGN < 0 ? cmul(t, w) : cmulc(t, w);
                }
            }
        }
    }
}

// Forward step 1, in place on this lane's column of the group buffer: inputs
// z[n2] at T[n2][n1], DFT-P over n2, twiddle by w_Lg^(n1 k2), outputs at T[k2][n1].
template <int N1, int P>
__device__ __forceinline__ void fwd_step1(float2* __restrict__ T, int n1,
                                          const float2* __restrict__ tw2) {
    constexpr int H = (P - 1) / 2;
    constexpr int OFF = toff(P);
    constexpr int RS = N1 + 1;
    float2 x0 = T[n1];
    float2 s[H], d[H];
    float2 y0 = x0;
#pragma unroll
    for (int j = 1; j <= H; ++j) {
        float2 a = T[j * RS + n1], b = T[(P - j) * RS + n1];
        s[j - 1] = cadd(a, b);
        d[j - 1] = csub(a, b);
        y0 = cadd(y0, s[j - 1]);
    }
    T[n1] = y0;
#pragma unroll
    for (int k = 1; k <= H; ++k) {
        float2 A = x0, B = f2(0.f, 0.f);
#pragma unroll
        for (int j = 1; j <= H; ++j) {
            const float2 cs = c_trigw[OFF + (j * k) % P];
            A = rfma(s[j - 1], cs.x, A);
            B = rfma(d[j - 1], cs.y, B);
        }
        float2 ib = mul_i<-1>(B);
        T[k * RS + n1] = cmul(cadd(A, ib), tw2[k * N1 + n1]);
        T[(P - k) * RS + n1] = cmul(csub(A, ib), tw2[(P - k) * N1 + n1]);
    }
}

// Inverse step 1, in place on this lane's column: inputs T[k2][n1] (already
// twiddled), inverse DFT-P over k2, outputs x[n1 + N1 n2] at T[n2][n1].
template <int N1, int P>
__device__ __forceinline__ void inv_step1(float2* __restrict__ T, int n1) {
    constexpr int H = (P - 1) / 2;
    constexpr int OFF = toff(P);
    constexpr int RS = N1 + 1;
    float2 x0 = T[n1];
    float2 s[H], d[H];
    float2 y0 = x0;
#pragma unroll
    for (int j = 1; j <= H; ++j) {
        float2 a = T[j * RS + n1], b = T[(P - j) * RS + n1];
        s[j - 1] = cadd(a, b);
        d[j - 1] = csub(a, b);
        y0 = cadd(y0, s[j - 1]);
    }
    T[n1] = y0;
#pragma unroll
    for (int k = 1; k <= H; ++k) {
        float2 A = x0, B = f2(0.f, 0.f);
#pragma unroll
        for (int j = 1; j <= H; ++j) {
            const float2 cs = c_trigw[OFF + (j * k) % P];
            A = rfma(s[j - 1], cs.x, A);
            B = rfma(d[j - 1], cs.y, B);
        }
        float2 ib = mul_i<1>(B);
        T[k * RS + n1] = cadd(A, ib);
        T[(P - k) * RS + n1] = csub(A, ib);
    }
}

// Forward step 2: rows of T -> DFT-N1 -> natural-order spectrum Z (same buffer).
template <int N1, int P>
__device__ __forceinline__ void fwd_step2(float2* __restrict__ buf, int j, bool active) {
    constexpr int RQ = (P + N1 - 1) / N1;
    constexpr int RS = N1 + 1;
    constexpr int LB = ilog2c(N1);
    float2 v[RQ][N1];
#pragma unroll
    for (int q = 0; q < RQ; ++q) {
        int r = j + N1 * q;
        if (active && r < P) {
#pragma unroll
            for (int t = 0; t < N1; ++t) v[q][t] = buf[r * RS + t];
        }
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < RQ; ++q) {
        int r = j + N1 * q;
        if (active && r < P) {
            dft_reg<N1, -1>(v[q]);
#pragma unroll
            for (int i = 0; i < N1; ++i) buf[r + P * brev(i, LB)] = v[q][i];   // X[k1] is v[brev(k1)]
        }
    }
    __syncwarp();
}

// Inverse step 2: natural-order spectrum -> inverse DFT-N1 per row -> conj twiddle -> T.
template <int N1, int P>
__device__ __forceinline__ void inv_step2(float2* __restrict__ buf, int j, bool active,
                                          const float2* __restrict__ tw2) {
    constexpr int RQ = (P + N1 - 1) / N1;
    constexpr int RS = N1 + 1;
    constexpr int LB = ilog2c(N1);
    float2 v[RQ][N1];
#pragma unroll
    for (int q = 0; q < RQ; ++q) {
        int r = j + N1 * q;
        if (active && r < P) {
#pragma unroll
            for (int k1 = 0; k1 < N1; ++k1) v[q][k1] = buf[r + P * k1];
        }
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < RQ; ++q) {
        int r = j + N1 * q;
        if (active && r < P) {
            dft_reg<N1, 1>(v[q]);
#pragma unroll
            for (int i = 0; i < N1; ++i) {
                const int n1 = brev(i, LB);
                buf[r * RS + n1] = cmulc(v[q][i], tw2[r * N1 + n1]);
            }
        }
    }
    __syncwarp();
}

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

__device__ __forceinline__ void xprep1(float x, float a, float b, float lam, bool keep,
                                       float& na, float& nb, float& v) {
    float t = x + a;                                        // X + y2
    float Y2 = copysignf(fmaxf(fabsf(t) - lam, 0.f), t);    // shrink!  (csc_kernels.jl:53-64)
    float Y3 = keep ? x + b : 0.f;                          // projectionX! (:68-82)
    na = (a + x) - Y2;                                      // train.jl:13
    nb = (b + x) - Y3;                                      // train.jl:14
    v = (Y2 - na) + (Y3 - nb);
}

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
                            Yo[e] = (wts + A.rho * (dx[e] + yn[e])) / (dg + A.rho);
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
            float2* sb = bufs + (size_t)sl * BUF;
            if (sl <= B) fwd_step1<N1, P>(sb, gl, tw2);
            __syncwarp();
            fwd_step2<N1, P>(sb, gl, sl <= B);
        }
        __syncthreads();

        // ---------------- split + this CTA's part of P = sum_m G1h[m] Vh[m]
        float2* Pp = Ppart + (it & 1) * Fp;
        for (int f = threadIdx.x; f < F; f += blockDim.x) {
            float2 P_ = f2(0.f, 0.f);
            const bool edge = (f == 0) || (f == half);
            const int fr = edge ? f : Lg - f;
            for (int sl = 0; sl < B; ++sl) {
                const float2* Z = bufs + (size_t)sl * BUF;
                const float2 z1 = Z[f], z2 = Z[fr];
                const float2 va = f2(0.5f * (z1.x + z2.x), 0.5f * (z1.y - z2.y));
                const float2 vb = f2(0.5f * (z1.y + z2.y), 0.5f * (z2.x - z1.x));
                P_ = cfma(g1[(2 * sl) * F + f], va, P_);
                if (2 * sl + 1 < Mc) P_ = cfma(g1[(2 * sl + 1) * F + f], vb, P_);
            }
            Pp[f] = P_;
        }
        cluster.sync();

        // ---------------- P over the cluster (fixed rank order), alpha, W; rank 0 packs
        // DXh = (P + A W)/(k Lg); every CTA repacks Xh = (Vh + conj(G1h) W)/(k Lg)
        {
            float2* ZU = bufs + (size_t)B * BUF;
            for (int f = threadIdx.x; f < F; f += blockDim.x) {
                float2 P_ = f2(0.f, 0.f);
                for (int r = 0; r < CS; ++r) P_ = cadd(P_, cluster.map_shared_rank(Pp, r)[f]);
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
                for (int sl = 0; sl < B; ++sl) {
                    float2* Z = bufs + (size_t)sl * BUF;
                    const bool hasb = 2 * sl + 1 < Mc;
                    const float2 z1 = Z[f], z2 = Z[edge ? f : Lg - f];
                    const float2 va = f2(0.5f * (z1.x + z2.x), 0.5f * (z1.y - z2.y));
                    const float2 vb = f2(0.5f * (z1.y + z2.y), 0.5f * (z2.x - z1.x));
                    float2 xa = cjfma(g1[(2 * sl) * F + f], W, va);
                    float2 xb = hasb ? cjfma(g1[(2 * sl + 1) * F + f], W, vb) : f2(0.f, 0.f);
                    xa = f2(xa.x * sc, xa.y * sc);
                    xb = f2(xb.x * sc, xb.y * sc);
                    if (edge) {
                        Z[f] = f2(xa.x, xb.x);
                    } else {
                        Z[f] = f2(xa.x - xb.y, xa.y + xb.x);
                        Z[Lg - f] = f2(xa.x + xb.y, xb.x - xa.y);
                    }
                }
            }
        }
        __syncthreads();

        // ---------------- inverse transforms (rank 0 also transforms DX)
        for (int q = 0; q < Q; ++q) {
            const int sl = grp + q * NG;
            float2* sb = bufs + (size_t)sl * BUF;
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
    std::vector<float2> trig(3 + 5 + 7 + 11 + 13 + 17 + 19 + 23 + 29 + 31);
    for (int p : kPrimesW)
        for (int m = 0; m < p; ++m)
            trig[toff(p) + m] = make_float2((float)cos(2.0 * M_PI * m / p), (float)sin(2.0 * M_PI * m / p));
    std::vector<float2> w32(32);
    for (int j = 0; j < 32; ++j) w32[j] = make_float2((float)cos(2.0 * M_PI * j / 32), (float)-sin(2.0 * M_PI * j / 32));
    int N1 = v->N1, Pp = v->P, Lg = N1 * Pp;
    std::vector<float2> tw2((size_t)Pp * N1);
    for (int k2 = 0; k2 < Pp; ++k2)
        for (int n1 = 0; n1 < N1; ++n1) {
            double a = 2.0 * M_PI * (double)((n1 * k2) % Lg) / Lg;
            tw2[(size_t)k2 * N1 + n1] = make_float2((float)cos(a), (float)-sin(a));
        }
    cudaError_t e = cudaMemcpyToSymbol(c_trigw, trig.data(), trig.size() * sizeof(float2));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_w32, w32.data(), 32 * sizeof(float2));
    if (e == cudaSuccess) e = cudaMalloc((void**)&P->tw2, tw2.size() * sizeof(float2));
    if (e == cudaSuccess) e = cudaMemcpy(P->tw2, tw2.data(), tw2.size() * sizeof(float2), cudaMemcpyHostToDevice);
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
        if (P->tw2) cudaFree(P->tw2);
        delete P;
        return nullptr;
    }
    if (nclusters > c->N) nclusters = c->N;
    P->grid = nclusters * P->CS;
    e = cudaMalloc((void**)&P->absx_part, (size_t)P->grid * sizeof(double));
    if (e != cudaSuccess) {
        *status = cdlgb_seterr(c, CDLGB_ECUDA, "cudaMalloc: %s", cudaGetErrorString(e));
        cudaFree(P->tw2);
        delete P;
        return nullptr;
    }
    return P;
}

void warp_plan_free(void* p) {
    WarpPlan* P = (WarpPlan*)p;
    if (!P) return;
    if (P->tw2) cudaFree(P->tw2);
    if (P->absx_part) cudaFree(P->absx_part);
    delete P;
}

int warp_plan_cluster(void* p) { return p ? ((WarpPlan*)p)->CS : 0; }

int warp_xstep(cdlgb_ctx* c, void* p, const float* Xin, float* Xout) {
    WarpPlan* P = (WarpPlan*)p;
    WArgs a;
    a.Xin = Xin; a.Xout = Xout; a.y2 = c->y2; a.y3 = c->y3;
    a.Y1 = c->Y1; a.y1 = c->y1; a.DX = c->DX; a.S = c->S;
    a.G1h = c->G1h; a.Ah = c->Ah; a.tw2 = P->tw2; a.absx_part = P->absx_part;
    a.N = c->N; a.M = c->M; a.F = c->F; a.L4 = c->L4; a.gamma = c->gamma;
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
