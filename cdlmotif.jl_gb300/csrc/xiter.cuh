// Fused X-steps: every iteration of one code update (code_update!, src/CDL/train.jl:1-44,
// csc_iter_num iterations) in one launch, with the per-sequence state resident on chip.
//
// The X-step couples the M filters of one sequence and nothing across sequences, and
// G1 (hence G1-hat and A = sum_m |G1-hat|^2) is fixed for the whole code update.  A
// cluster of CS CTAs therefore takes one sequence at a time and runs all the
// iterations on it before moving on:
//   * each CTA owns Mc = M / CS filters; their duals y2, y3 (2 x Mc x Lg floats) stay in
//     its shared memory for all iterations;
//   * X never leaves the chip between iterations: the inverse DFT-P of the X spectrum
//     leaves X[n1 + N1 n2] in lane n1's column of its slot buffer, where the next
//     iteration's shrink!/projectionX!/dual updates (csc_kernels.jl:53-82,
//     train.jl:12-14) turn it into V in place for the forward DFT-P;
//   * every CTA transforms DX itself (the cross-filter sum P is identical on every
//     rank, summed in fixed rank order) and keeps y1 in shared memory; Y1 is formed
//     from DX (update_Y1!, csc_kernels.jl:86-95) and consumed at once.
// HBM is touched once per sequence per code update: X, y2, y3, Y1, y1, DX are read at
// the first iteration and X, y2, y3, Y1, y1, DX written after the last.  The
// arithmetic of every iteration is the one-X-step kernel's (xwarp.cu), operation for
// operation, so both give the same bits.
//
// This header holds the kernel template; xiter_v*.cu instantiate its variants (one
// group per translation unit, so the build compiles them in parallel; every unit has
// its own copy of the register FFTs' constant tables and uploads it), and xiter.cu
// holds the host side.
#pragma once

#include "cdlgb_internal.h"
#include "regfft.cuh"

#include <cooperative_groups.h>
#include <stdlib.h>
#include <vector>

namespace xiter {

struct IArgs {
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
    double* res_part;       // per CTA: the five X-step residual sums of the final iterate
    int N, M, L4, gamma, iters;
    float lam, rho, kc;
    int ld, ld3;            // row strides (pairs) of the y2 and compacted y3 rows in shared memory
};

typedef void (*kern_t)(IArgs);
// (N1, P, filters per CTA, threads, CTAs per SM): threads = 32 ceil((MC/2 + 1) / (32 / N1))
// rounded to a warp; k without, kr with the residual sums; tables uploads the constant
// tables of the unit that instantiated k and kr
struct Variant { int N1, P, MC, threads, minb; kern_t k, kr; cudaError_t (*tables)(); };

}  // namespace xiter

namespace {

namespace cg = cooperative_groups;
using xiter::IArgs;

// this CTA's part of P = sum_m G1h[m] Vh[m] at bin f, G1h from registers (the sum in
// slot order, as partial_P)
template <int Lg, int MC>
__device__ __forceinline__ float2 partial_P_r(const float2* __restrict__ bufs, int BUF, int f,
                                             const float2 (&g)[MC]) {
    constexpr int B = (MC + 1) / 2;
    const bool edge = (f == 0) || (f == Lg / 2);
    const int fr = edge ? f : Lg - f;
    float2 z1[B], z2[B];
#pragma unroll
    for (int sl = 0; sl < B; ++sl) {
        z1[sl] = bufs[sl * BUF + f];
        z2[sl] = bufs[sl * BUF + fr];
    }
    float2 P_ = f2(0.f, 0.f);
#pragma unroll
    for (int sl = 0; sl < B; ++sl) {
        const float2 va = f2(z1[sl].x + z2[sl].x, z1[sl].y - z2[sl].y);      // 2 Vh[2 sl]
        const float2 vb = f2(z1[sl].y + z2[sl].y, z2[sl].x - z1[sl].x);      // 2 Vh[2 sl + 1]
        P_ = cfma(g[2 * sl], va, P_);
        if (2 * sl + 1 < MC) P_ = cfma(g[2 * sl + 1], vb, P_);
    }
    return f2(0.5f * P_.x, 0.5f * P_.y);      // every partial sum was exactly doubled
}

// Xh = (Vh + conj(G1h) W) * sc at bins f and Lg - f, packed back into the slots, G1h
// from registers (as repack_X)
template <int Lg, int MC>
__device__ __forceinline__ void repack_X_r(float2* __restrict__ bufs, int BUF, int f,
                                           const float2 (&g)[MC], float2 W, float sc) {
    constexpr int B = (MC + 1) / 2;
    const bool edge = (f == 0) || (f == Lg / 2);
    const int fr = edge ? f : Lg - f;
    // with 2 Vh and 2 W every term is exactly doubled; the scale sc / 2 undoes it
    const float2 W2 = f2(W.x + W.x, W.y + W.y);
    const float sch = 0.5f * sc;
    float2 z1[B], z2[B];
#pragma unroll
    for (int sl = 0; sl < B; ++sl) {
        z1[sl] = bufs[sl * BUF + f];
        z2[sl] = bufs[sl * BUF + fr];
    }
#pragma unroll
    for (int sl = 0; sl < B; ++sl) {
        const float2 va = f2(z1[sl].x + z2[sl].x, z1[sl].y - z2[sl].y);
        const float2 vb = f2(z1[sl].y + z2[sl].y, z2[sl].x - z1[sl].x);
        float2 xa = cjfma(g[2 * sl], W2, va);
        float2 xb = 2 * sl + 1 < MC ? cjfma(g[2 * sl + 1], W2, vb) : f2(0.f, 0.f);
        xa = f2(__fmul_rn(xa.x, sch), __fmul_rn(xa.y, sch));
        xb = f2(__fmul_rn(xb.x, sch), __fmul_rn(xb.y, sch));
        if (edge) {
            bufs[sl * BUF + f] = f2(xa.x, xb.x);
        } else {
            bufs[sl * BUF + f] = f2(xa.x - xb.y, xa.y + xb.x);
            bufs[sl * BUF + Lg - f] = f2(xa.x + xb.y, xb.x - xa.y);
        }
    }
}

// L2 prefetch of the rows sequence n will read at its first iteration (this CTA's MC
// filter rows of X, y2, y3; Y1, y1, DX and the W'S window), issued by the 32 lanes of
// one warp while the current sequence is still iterating.  Bulk prefetches are hints:
// nothing waits on them.  Every row is a multiple of 16 bytes long (Lg and L4 are
// multiples of 4 floats); a base pointer that is not 16-byte aligned skips the hint.
__device__ __forceinline__ void l2_prefetch(const void* p, unsigned bytes) {
    if (((uintptr_t)p & 15) == 0)
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" :: "l"(p), "r"(bytes) : "memory");
}
__device__ __forceinline__ void prefetch_next(const IArgs& A, int n, int m0, int MC, int Lg, int lane) {
    if (n >= A.N) return;
    const unsigned rb = (unsigned)Lg * 4u;
    const size_t r0 = ((size_t)n * A.M + m0) * Lg;
    for (int q = lane; q < 3 * MC + 4; q += 32) {
        if (q < 3 * MC) {
            const float* base = q < MC ? A.Xin : q < 2 * MC ? A.y2 : A.y3;
            l2_prefetch(base + r0 + (size_t)(q % MC) * Lg, rb);
        } else if (q < 3 * MC + 3) {
            const float* base = q == 3 * MC ? A.Y1 : q == 3 * MC + 1 ? A.y1 : A.DX;
            l2_prefetch(base + (size_t)n * Lg, rb);
        } else {
            l2_prefetch(A.S + (size_t)n * A.L4, (unsigned)A.L4 * 4u);
        }
    }
}

// MC filters per CTA (compile time), NT threads: every slot's lane group and every
// thread's bins of the cross-filter phases are fixed, and each thread keeps the G1h
// values of its bins in registers for the whole launch (G1 is fixed during a code update).
// RES: also the residual sums of the final iterates (compiled out when false, so the
// kernel without them is unchanged)
template <int N1, int P, int NT, int MINB, int MC, bool RES>
__global__ void __launch_bounds__(NT, MINB) k_xiter(IArgs A) {
    constexpr int Lg = N1 * P;
    constexpr int G = 32 / N1;                  // lane groups per warp
    constexpr int RS = N1 + 1;
    constexpr int BUF = (P * RS + 1) & ~1;
    constexpr int half = Lg / 2;
    constexpr int F = Lg / 2 + 1;
    constexpr int Fp = (F + 1) & ~1;
    extern __shared__ float4 smem4[];
    cg::cluster_group cluster = cg::this_cluster();
    const int CS = (int)cluster.num_blocks();
    const int rank = (int)cluster.block_rank();
    const int cid = blockIdx.x / CS;
    const int nclusters = gridDim.x / CS;
    constexpr int W3 = 3 * N1 / 4;              // y3 entries per n2 row (l % 4 != 0 only)
    constexpr int B = (MC + 1) / 2;             // packed pairs
    constexpr int Mc = MC;
    constexpr int NFR = (F + NT - 1) / NT;      // bins per thread in the cross-filter phases
    const int M = A.M, ld = A.ld, ld3 = A.ld3;

    float2* bufs = reinterpret_cast<float2*>(smem4);       // [B + 1][BUF] slot buffers
    float2* Ppart = bufs + (size_t)(B + 1) * BUF;          // [2][Fp] this CTA's part of P
    float2* tw2 = Ppart + 2 * Fp;                          // [P][N1] twiddles
    // the duals of the two filters of pair s, interleaved: [B][ld] (y2 of filters 2s, 2s+1)
    float2* y2s = tw2 + P * N1;
    // y3 is identically zero on the rows l % 4 == 0: there projectionX! keeps X + y3,
    // so the update y3 + X - Y3 is (y3 + X) - (X + y3) = +0 exactly.  Only the other
    // rows are kept, [B][ld3], row n2 of lane n1 at n2 W3 + n1 - n1/4 - 1.
    float2* y3s = y2s + (size_t)B * ld;
    float* y1s = reinterpret_cast<float*>(y3s + (size_t)B * ld3);   // [Lg]
    float* Ahs = y1s + Lg;                                 // [Fp] sum_m |G1h|^2
    float* Ss = Ahs + Fp;                                  // [L4] this sequence's W'S window
    __shared__ double red[NT / 32];
    // per warp: compensated (Kahan) float32 sums over its sequences of (X - Y2)^2,
    // (X - Y3)^2, X^2, (DX - Y1)^2, DX^2 of the final iterates, [warp][value][sum, comp]
    __shared__ float rsum[NT / 32][5][2];

    if (RES)
        for (int t = threadIdx.x; t < 10 * (NT / 32); t += blockDim.x) (&rsum[0][0][0])[t] = 0.f;
    // M need not be a multiple of MC: the last CTA of a cluster then holds Mr < MC real
    // filters (M even, so whole pairs), and its other pair slots stay zero throughout --
    // with zero G1-hat they add exactly nothing to P, and their X is never stored
    const int m0 = rank * Mc;
    const int Mr = max(0, min(Mc, M - m0));
    for (int t = threadIdx.x; t < P * N1; t += blockDim.x) tw2[t] = A.tw2[t];
    for (int t = threadIdx.x; t < F; t += blockDim.x) Ahs[t] = A.Ah[t];
    for (int t = threadIdx.x; t < (B - Mr / 2) * BUF; t += blockDim.x)
        bufs[(size_t)(Mr / 2) * BUF + t] = f2(0.f, 0.f);
    __syncthreads();

    float2 g1r[NFR][MC];
#pragma unroll
    for (int r = 0; r < NFR; ++r) {
        const int f = threadIdx.x + r * NT;
#pragma unroll
        for (int m = 0; m < MC; ++m)
            g1r[r][m] = f < F && m < Mr ? A.G1h[(size_t)(m0 + m) * F + f] : f2(0.f, 0.f);
    }
    const int lane = threadIdx.x & 31;
    const int grp = (threadIdx.x >> 5) * G + lane / N1;   // this lane group's slot
    const int gl = lane % N1;                             // lane within the group
    const bool pair = grp < B && 2 * grp < Mr;            // a pair of real filters
    const bool act = pair || grp == B;                    // ... or the U / DX group
    static_assert(MC % 2 == 0, "filters per CTA must pair up");
    float2* sb = bufs + (size_t)(act ? grp : 0) * BUF;
    float2* y2p = y2s + (size_t)(pair ? grp : 0) * ld + gl;
    const bool keep = (gl & 3) == 0;                      // l = gl + N1 n2, N1 % 4 == 0
    float2* y3p = y3s + (size_t)(pair ? grp : 0) * ld3 + (keep ? 0 : gl - (gl >> 2) - 1);
    const float sc = 1.f / (A.kc * (float)Lg);
    const float lam = A.lam, rho = A.rho;
    const unsigned gmask = N1 == 32 ? 0xffffffffu : (0xffffu << (lane & 16));   // this lane group
    double absacc = 0.0;
    int it = 0;                                           // parity of the P buffers

    for (int n = cid; n < A.N; n += nclusters) {
        // ---------------- first iteration's inputs, from HBM
        // (V and U are written to the slot buffer and transformed from there, so that
        // the HBM loads need no register array)
        if (pair) {
            const size_t ra = ((size_t)n * M + m0 + 2 * grp) * Lg + gl;
#pragma unroll 16
            for (int n2 = 0; n2 < P; ++n2) {
                const int o = N1 * n2;
                float2 a2 = f2(A.y2[ra + o], A.y2[ra + Lg + o]);
                float2 a3 = f2(A.y3[ra + o], A.y3[ra + Lg + o]);
                const float2 V = xprep2(f2(A.Xin[ra + o], A.Xin[ra + Lg + o]), a2, a3, lam, keep);
                y2p[o] = a2;
                if (!keep) y3p[W3 * n2] = a3;
                sb[n2 * RS + gl] = V;
            }
            fwd_step1<N1, P>(sb, gl, tw2);
        } else if (act) {
            // U = Y1 - y1', y1' = y1 + DX - Y1  (train.jl:12; REF_QUIRK_Q6: the previous
            // iteration's Y1, as the y3 update uses the previous Y3 and y2 the fresh Y2)
            __syncwarp(gmask);                  // the previous sequence's reads of Ss are done
            // the window in batches of 8 loads per lane, all issued before their stores
            const float* Sn = A.S + (size_t)n * A.L4;
            for (int t0 = gl; t0 < A.L4; t0 += 8 * N1) {
                float sv[8];
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    const int t = t0 + N1 * k;
                    sv[k] = t < A.L4 ? Sn[t] : 0.f;
                }
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    const int t = t0 + N1 * k;
                    if (t < A.L4) Ss[t] = sv[k];
                }
            }
            __syncwarp(gmask);
            const size_t r = (size_t)n * Lg + gl;
#pragma unroll 16
            for (int n2 = 0; n2 < P; ++n2) {
                const int o = N1 * n2;
                const float Yv = A.Y1[r + o], yv = A.y1[r + o], dv = A.DX[r + o];
                const float yn = (yv + dv) - Yv;
                y1s[gl + o] = yn;
                sb[n2 * RS + gl] = f2(Yv - yn, 0.f);
            }
            fwd_step1<N1, P>(sb, gl, tw2);
        }

        for (int t = 0; t < A.iters; ++t, ++it) {
            if (t == A.iters / 2 && threadIdx.x >= 32 && threadIdx.x < 64)
                prefetch_next(A, n + nclusters, m0, Mr, Lg, lane);
            __syncwarp();
            // a warp that is one idle lane group (padding pairs, 32-lane groups) skips the
            // row DFT's store-free loads; two groups sharing a warp both run it
            if (G > 1 || act) fwd_step2<N1, P>(sb, gl, act);
            __syncthreads();

            // ---------------- split + this CTA's part of P = sum_m G1h[m] Vh[m]
            float2* Pp = Ppart + (it & 1) * Fp;
#pragma unroll
            for (int r = 0; r < NFR; ++r) {
                const int f = threadIdx.x + r * NT;
                if (f < F) Pp[f] = partial_P_r<Lg, MC>(bufs, BUF, f, g1r[r]);
            }
            cluster.sync();

            // ---------------- P over the cluster (fixed rank order), alpha, W; every CTA
            // packs DXh = (P + A W)/(k Lg) and repacks Xh = (Vh + conj(G1h) W)/(k Lg)
            {
                float2* ZU = bufs + (size_t)B * BUF;
#pragma unroll
                for (int r = 0; r < NFR; ++r) {
                    const int f = threadIdx.x + r * NT;
                    if (f >= F) break;
                    const float2 P_ = cluster_sum<8>(cluster, Pp, CS, f);
                    const float Av = Ahs[f];
                    const float2 U = ZU[f];
                    const float inv_s = 1.f / (Av + A.kc);
                    const float2 alpha = f2(fmaf(Av, U.x, P_.x) * inv_s, fmaf(Av, U.y, P_.y) * inv_s);
                    const float2 W = csub(U, alpha);
                    const bool edge = (f == 0) || (f == half);
                    const float2 D = f2(fmaf(Av, W.x, P_.x) * sc, fmaf(Av, W.y, P_.y) * sc);
                    if (edge) {
                        ZU[f] = f2(D.x, 0.f);
                    } else {
                        ZU[f] = D;
                        ZU[Lg - f] = f2(D.x, -D.y);
                    }
                    repack_X_r<Lg, MC>(bufs, BUF, f, g1r[r], W, sc);
                }
            }
            __syncthreads();

            // ---------------- inverse transforms; then either the next iteration's
            // inputs (in registers, straight into the forward DFT-P) or the results
            if (G > 1 || act) inv_step2<N1, P, false>(sb, gl, act, tw2);
            const bool last = t == A.iters - 1;
            if (act) inv_step1<N1, P, true>(sb, gl, tw2);   // X (or DX) at T[n2][gl], l = gl + N1 n2
            // residuals of the final iterate: what the next dual updates would add
            // (train.jl:12-14): X - shrink(X + y2), X - projectionX(X + y3) (X off the
            // kept rows; +0 on them, where y3 = +0), DX - Y1
            float q2 = 0.f, q3 = 0.f, qx = 0.f, q1 = 0.f, qd = 0.f;
            if (pair) {
                if (!last) {
#pragma unroll 8
                    for (int n2 = 0; n2 < P; ++n2) {
                        const int o = N1 * n2;
                        const int o3 = W3 * n2;
                        float2 a2 = y2p[o];
                        float2 a3 = keep ? f2(0.f, 0.f) : y3p[o3];
                        const float2 V = xprep2(sb[n2 * RS + gl], a2, a3, lam, keep);
                        y2p[o] = a2;
                        if (!keep) y3p[o3] = a3;
                        sb[n2 * RS + gl] = V;
                    }
                    fwd_step1<N1, P>(sb, gl, tw2);
                } else {
                    const size_t ra = ((size_t)n * M + m0 + 2 * grp) * Lg + gl;
                    float s = 0.f;
#pragma unroll
                    for (int n2 = 0; n2 < P; ++n2) {
                        const int o = N1 * n2;
                        const float2 xv = sb[n2 * RS + gl];
                        const float2 a2 = y2p[o];
                        const float2 a3 = keep ? f2(0.f, 0.f) : y3p[W3 * n2];
                        A.Xout[ra + o] = xv.x;
                        A.Xout[ra + Lg + o] = xv.y;
                        A.y2[ra + o] = a2.x;
                        A.y2[ra + Lg + o] = a2.y;
                        A.y3[ra + o] = a3.x;
                        A.y3[ra + Lg + o] = a3.y;
                        s += fabsf(xv.x);
                        s += fabsf(xv.y);
                        if (!RES) continue;
                        const float2 t2 = cadd(xv, a2);
                        const float2 r2 = csub(xv, csub(t2, f2(fminf(fmaxf(t2.x, -lam), lam),
                                                               fminf(fmaxf(t2.y, -lam), lam))));
                        const float sx = fmaf(xv.x, xv.x, xv.y * xv.y);
                        q2 = fmaf(r2.x, r2.x, fmaf(r2.y, r2.y, q2));
                        if (!keep) q3 += sx;
                        qx += sx;
                    }
                    absacc += (double)s;
                }
            } else if (act) {
                // DX, then Y1 = (W'S + rho (DX + y1')) / (W'W + rho)  (update_Y1!,
                // csc_kernels.jl:86-95), then the next iteration's y1' and U
                const size_t r = (size_t)n * Lg + gl;
#pragma unroll 8
                for (int n2 = 0; n2 < P; ++n2) {
                    const int o = N1 * n2;
                    const int l = gl + o;
                    const bool in = l >= A.gamma && l < A.gamma + A.L4;
                    const float wts = in ? Ss[l - A.gamma] : 0.f;
                    const float dg = in ? 1.f : 0.f;
                    const float dx = sb[n2 * RS + gl].x, yp = y1s[l];
                    const float Y1n = __fadd_rn(wts, __fmul_rn(rho, dx + yp)) / (dg + rho);
                    if (!last) {
                        const float yn = (yp + dx) - Y1n;
                        y1s[l] = yn;
                        sb[n2 * RS + gl] = f2(Y1n - yn, 0.f);
                    } else if (rank == 0) {
                        A.DX[r + o] = dx;
                        A.Y1[r + o] = Y1n;
                        A.y1[r + o] = yp;
                        if (!RES) continue;
                        const float e = dx - Y1n;
                        q1 = fmaf(e, e, q1);
                        qd = fmaf(dx, dx, qd);
                    }
                }
                if (!last) fwd_step1<N1, P>(sb, gl, tw2);
            }
            if (RES && last) {
                // the warp's sums for this sequence, added by lane 0 into its
                // compensated running sums (no float64 work inside the sequence loop)
                float v[5] = {q2, q3, qx, q1, qd};
#pragma unroll
                for (int k = 0; k < 5; ++k) {
                    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
                    if (lane == 0) {
                        float* a = rsum[threadIdx.x >> 5][k];
                        const float y = __fsub_rn(v[k], a[1]);
                        const float t = __fadd_rn(a[0], y);
                        a[1] = __fsub_rn(__fsub_rn(t, a[0]), y);
                        a[0] = t;
                    }
                }
            }
        }
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
    if (RES && threadIdx.x < 5) {
        double t = 0.0;
        for (int w = 0; w < NT / 32; ++w) t += (double)rsum[w][threadIdx.x][0] - (double)rsum[w][threadIdx.x][1];
        A.res_part[(size_t)blockIdx.x * 5 + threadIdx.x] = t;
    }
}

}  // namespace

#define XITER_VARIANT(N1, P, NT, MINB, MC)                                                    \
    {N1, P, MC, NT, MINB, k_xiter<N1, P, NT, MINB, MC, false>, k_xiter<N1, P, NT, MINB, MC, true>, \
     regfft_upload_tables}
