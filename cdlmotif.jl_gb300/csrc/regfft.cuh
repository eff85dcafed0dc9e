// Register-resident FFT building blocks shared by the fused X-step kernels
// (xwarp.cu: one X-step per launch; xiter.cu: all X-steps of a code update per
// launch).  Lg = N1 * P with N1 in {16, 32} lanes and P an odd prime:
//   forward  x[n1 + N1 n2] (lane n1 holds n2 = 0..P-1)
//     1. DFT-P over n2 in registers (pairwise-symmetric form), twiddle w_Lg^(n1 k2),
//        write T[k2][n1] (row stride N1+1: conflict-free both ways);
//     2. lane j takes rows r = j + N1 q: DFT-N1 in registers (radix-2 DIF) gives
//        X[r + P k1], written in natural order into the same buffer.
//   inverse  the same steps backwards.
// Each translation unit that includes this header has its own copy of the constant
// tables and uploads them with regfft_upload_tables().
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <mutex>
#include <vector>

namespace {

// cos/sin(2 pi m / p) for the per-lane DFT lengths p (the odd primes 3..31, the odd
// composites 21, 25, 27, 33 and the even 18, 20, 22, 24, 26, 28, 30: the symmetric
// direct DFT-P below needs no prime), concatenated; exp(-2 pi i j / 32)
const int kPrimesW[] = {3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 33, 21, 25, 27, 26, 28, 30, 18, 20, 22, 24};
constexpr int kTrigW = 3 + 5 + 7 + 11 + 13 + 17 + 19 + 23 + 29 + 31 + 33 + 21 + 25 + 27 + 26 + 28 + 30 +
                       18 + 20 + 22 + 24;
__constant__ float2 c_trigw[kTrigW];
__constant__ float2 c_w32[32];

__host__ __device__ constexpr int toff(int p) {
    return p == 3 ? 0 : p == 5 ? 3 : p == 7 ? 8 : p == 11 ? 15 : p == 13 ? 26 : p == 17 ? 39
         : p == 19 ? 56 : p == 23 ? 75 : p == 29 ? 98 : p == 31 ? 127 : p == 33 ? 158
         : p == 21 ? 191 : p == 25 ? 212 : p == 27 ? 237 : p == 26 ? 264 : p == 28 ? 290
         : p == 30 ? 318 : p == 18 ? 348 : p == 20 ? 366 : p == 22 ? 386 : p == 24 ? 408 : -1;
}

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

// The per-lane DFT-P over a column (SIGN -1 forward, +1 inverse), in the symmetric
// direct form: x_j and x_{P-j} enter as s_j = x_j + x_{P-j} and d_j = x_j - x_{P-j},
// output k and P - k share A = x0 + sum_j s_j cos(2 pi j k / P) and
// B = sum_j d_j sin(2 pi j k / P), X[k] = A + SIGN i B and X[P-k] = A - SIGN i B.  For
// an even P the middle input x_{P/2} enters A with the sign (-1)^k (as e = x0 + x_{P/2}
// or o = x0 - x_{P/2}), and the outputs 0 and P/2 are e + sum_j s_j and
// (-1)^{P/2} part + sum_j (-1)^j s_j.  Inputs z[n2] at T[n2][n1]; with TW (inverse) the
// conjugate twiddles are applied as the inputs are loaded; with OTW (forward) the
// outputs are multiplied by the twiddles w_Lg^(n1 k2) as they are stored.
template <int N1, int P, int SIGN, bool TW, bool OTW>
__device__ __forceinline__ void dft_p_col(float2* __restrict__ T, int n1, const float2* __restrict__ tw2) {
    constexpr bool EVEN = (P % 2) == 0;
    constexpr int H = EVEN ? P / 2 - 1 : (P - 1) / 2;
    constexpr int OFF = toff(P);
    constexpr int RS = N1 + 1;
    float2 x0 = T[n1];
    if (TW) x0 = cmulc(x0, tw2[n1]);
    float2 e = x0, o = x0;
    if (EVEN) {
        float2 xh = T[(P / 2) * RS + n1];
        if (TW) xh = cmulc(xh, tw2[(P / 2) * N1 + n1]);
        e = cadd(x0, xh);
        o = csub(x0, xh);
    }
    float2 s[H], d[H];
    float2 y0 = e;
#pragma unroll
    for (int j = 1; j <= H; ++j) {
        float2 a = T[j * RS + n1], b = T[(P - j) * RS + n1];
        if (TW) {
            a = cmulc(a, tw2[j * N1 + n1]);
            b = cmulc(b, tw2[(P - j) * N1 + n1]);
        }
        s[j - 1] = cadd(a, b);
        d[j - 1] = csub(a, b);
        y0 = cadd(y0, s[j - 1]);
    }
    T[n1] = y0;
    if (EVEN) {
        float2 ym = ((P / 2) % 2 == 0) ? e : o;
#pragma unroll
        for (int j = 1; j <= H; ++j) ym = (j % 2) ? csub(ym, s[j - 1]) : cadd(ym, s[j - 1]);
        T[(P / 2) * RS + n1] = OTW ? cmul(ym, tw2[(P / 2) * N1 + n1]) : ym;
    }
#pragma unroll
    for (int k = 1; k <= H; ++k) {
        float2 A = (EVEN && (k % 2)) ? o : e, B = f2(0.f, 0.f);
#pragma unroll
        for (int j = 1; j <= H; ++j) {
            const float2 cs = c_trigw[OFF + (j * k) % P];
            A = rfma(s[j - 1], cs.x, A);
            B = rfma(d[j - 1], cs.y, B);
        }
        float2 ib = mul_i<SIGN>(B);
        if (OTW) {
            T[k * RS + n1] = cmul(cadd(A, ib), tw2[k * N1 + n1]);
            T[(P - k) * RS + n1] = cmul(csub(A, ib), tw2[(P - k) * N1 + n1]);
        } else {
            T[k * RS + n1] = cadd(A, ib);
            T[(P - k) * RS + n1] = csub(A, ib);
        }
    }
}

// Forward step 1, in place on this lane's column of the group buffer: inputs
// z[n2] at T[n2][n1], DFT-P over n2, twiddle by w_Lg^(n1 k2), outputs at T[k2][n1].
template <int N1, int P>
__device__ __forceinline__ void fwd_step1(float2* __restrict__ T, int n1,
                                          const float2* __restrict__ tw2) {
    dft_p_col<N1, P, -1, false, true>(T, n1, tw2);
}

// Inverse step 1, in place on this lane's column: inputs T[k2][n1] (already
// twiddled), inverse DFT-P over k2, outputs x[n1 + N1 n2] at T[n2][n1].
// With TW, the conjugate twiddles are applied here, as the inputs are loaded, instead
// of by inv_step2 (the same products, so the same bits).
template <int N1, int P, bool TW = false>
__device__ __forceinline__ void inv_step1(float2* __restrict__ T, int n1,
                                          const float2* __restrict__ tw2 = nullptr) {
    dft_p_col<N1, P, 1, TW, false>(T, n1, tw2);
}

// Forward step 2: rows of T -> DFT-N1 -> natural-order spectrum Z (same buffer).
template <int N1, int P>
__device__ __forceinline__ void fwd_step2(float2* __restrict__ buf, int j, bool active) {
    constexpr int RQ = (P + N1 - 1) / N1;
    constexpr int RS = N1 + 1;
    constexpr int LB = ilog2c(N1);
    float2 v[RQ][N1];
    // every lane loads (an idle lane reads row 0 and stores nothing), so that v is
    // defined on every path and not kept live around the callers' loops
#pragma unroll
    for (int q = 0; q < RQ; ++q) {
        const int r = j + N1 * q;
        const int rr = (active && r < P) ? r : 0;
#pragma unroll
        for (int t = 0; t < N1; ++t) v[q][t] = buf[rr * RS + t];
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
// With TW = false the conjugate twiddles are left to inv_step1<.., true>.
template <int N1, int P, bool TW = true>
__device__ __forceinline__ void inv_step2(float2* __restrict__ buf, int j, bool active,
                                          const float2* __restrict__ tw2) {
    constexpr int RQ = (P + N1 - 1) / N1;
    constexpr int RS = N1 + 1;
    constexpr int LB = ilog2c(N1);
    float2 v[RQ][N1];
#pragma unroll
    for (int q = 0; q < RQ; ++q) {
        const int r = j + N1 * q;
        const int rr = (active && r < P) ? r : 0;
#pragma unroll
        for (int k1 = 0; k1 < N1; ++k1) v[q][k1] = buf[rr + P * k1];
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
                buf[r * RS + n1] = TW ? cmulc(v[q][i], tw2[r * N1 + n1]) : v[q][i];
            }
        }
    }
    __syncwarp();
}

// shrink!, projectionX! and the dual updates of one entry (train.jl:12-14,
// csc_kernels.jl:53-82), returning V = (Y2 - y2') + (Y3 - y3') in na, nb, v:
//   Y2 = t - clamp(t, -lam, lam), t = X + y2 (= sign(t) max(|t| - lam, 0), the soft
//        threshold at lam -- not lam / rho, REF_QUIRK_Q4, csc_kernels.jl:61 -- up to the
//        sign of a zero result);  y2' = (y2 + X) - Y2;
//   on the rows projectionX! keeps (keep): Y3 = X + y3 and y3' = (y3 + X) - Y3 = +0;
//   elsewhere Y3 = 0 and y3' = y3 + X.
__device__ __forceinline__ void xprep1(float x, float a, float b, float lam, bool keep,
                                       float& na, float& nb, float& v) {
    const float t = x + a;
    const float Y2 = t - fminf(fmaxf(t, -lam), lam);
    na = t - Y2;
    const float u = x + b;
    nb = keep ? 0.f : u;
    const float w = Y2 - na;
    v = keep ? w + u : w - u;
}

// xprep1 for the two filters of a slot at once (packed FP32x2: the same operations
// on both halves, so the same bits); y2 and y3 are updated in place, V returned
__device__ __forceinline__ float2 xprep2(float2 x, float2& y2, float2& y3, float lam, bool keep) {
    const float2 t = cadd(x, y2);
    const float2 c = f2(fminf(fmaxf(t.x, -lam), lam), fminf(fmaxf(t.y, -lam), lam));
    const float2 Y2 = csub(t, c);
    const float2 na = csub(t, Y2);
    const float2 u = cadd(x, y3);
    const float2 w = csub(Y2, na);
    y2 = na;
    y3 = keep ? f2(0.f, 0.f) : u;
    return keep ? cadd(w, u) : csub(w, u);
}


// ---- cross-filter phases shared by the fused X-step kernels.  Slot sl of `bufs`
// (stride BUF) holds the packed spectrum Z = Vh[2 sl] + i Vh[2 sl + 1] of this CTA's
// filters 2 sl, 2 sl + 1 (the second absent when 2 sl + 1 == Mc); g1 is this CTA's
// [Mc][F] slice of G1h.  The loads of CH slots are issued together before their
// arithmetic, which stays in slot order (the same sums, the same bits).  Products that
// the compiler could fuse into a following add are written as separately rounded
// intrinsics, so that every kernel using these phases rounds identically.
constexpr int kSlotChunk = 4;

// this CTA's part of P = sum_m G1h[m] Vh[m] at bin f (train.jl:18-25, the RHS dot; the
// consensus dictionary's G1-hat, not the per-sequence d-hat: REF_QUIRK_Q5)
template <int Lg>
__device__ __forceinline__ float2 partial_P(const float2* __restrict__ bufs, int BUF, int B,
                                           int Mc, int F, int f, const float2* g1) {
    constexpr int half = Lg / 2;
    const bool edge = (f == 0) || (f == half);
    const int fr = edge ? f : Lg - f;
    float2 P_ = f2(0.f, 0.f);
    for (int s0 = 0; s0 < B; s0 += kSlotChunk) {
        float2 ga[kSlotChunk], gb[kSlotChunk], z1[kSlotChunk], z2[kSlotChunk];
#pragma unroll
        for (int u = 0; u < kSlotChunk; ++u) {
            const int sl = s0 + u;
            const int sa = sl < B ? sl : 0;
            const int mb = 2 * sl + 1 < Mc ? 2 * sl + 1 : 0;
            const float2* Z = bufs + (size_t)sa * BUF;
            z1[u] = Z[f];
            z2[u] = Z[fr];
            ga[u] = g1[(2 * sa) * F + f];
            gb[u] = g1[mb * F + f];
        }
#pragma unroll
        for (int u = 0; u < kSlotChunk; ++u) {
            const int sl = s0 + u;
            if (sl < B) {
                const float2 va = f2(z1[u].x + z2[u].x, z1[u].y - z2[u].y);     // 2 Vh[2 sl]
                const float2 vb = f2(z1[u].y + z2[u].y, z2[u].x - z1[u].x);     // 2 Vh[2 sl + 1]
                P_ = cfma(ga[u], va, P_);
                if (2 * sl + 1 < Mc) P_ = cfma(gb[u], vb, P_);
            }
        }
    }
    return f2(0.5f * P_.x, 0.5f * P_.y);      // every partial sum was exactly doubled
}

// P = sum over the cluster's CTAs of their parts at bin f, in rank order; the CS
// remote loads are issued before the sums
template <int CSMAX, class Cluster>
__device__ __forceinline__ float2 cluster_sum(Cluster& cluster, float2* Pp, int CS, int f) {
    float2 v[CSMAX];
#pragma unroll
    for (int r = 0; r < CSMAX; ++r) v[r] = r < CS ? cluster.map_shared_rank(Pp, r)[f] : f2(0.f, 0.f);
    float2 P_ = f2(0.f, 0.f);
#pragma unroll
    for (int r = 0; r < CSMAX; ++r)
        if (r < CS) P_ = cadd(P_, v[r]);
    return P_;
}

// Xh = (Vh + conj(G1h) W) * sc for this CTA's filters at bins f and Lg - f, packed back
// into the slots (sherman_CSC_combine!, csc_kernels.jl:38-49, and the inverse's input)
template <int Lg>
__device__ __forceinline__ void repack_X(float2* __restrict__ bufs, int BUF, int B, int Mc,
                                         int F, int f, const float2* g1, float2 W, float sc) {
    constexpr int half = Lg / 2;
    // with 2 Vh and 2 W every term is exactly doubled; the scale sc / 2 undoes it
    const float2 W2 = f2(W.x + W.x, W.y + W.y);
    const float sch = 0.5f * sc;
    const bool edge = (f == 0) || (f == half);
    const int fr = edge ? f : Lg - f;
    for (int s0 = 0; s0 < B; s0 += kSlotChunk) {
        float2 ga[kSlotChunk], gb[kSlotChunk], z1[kSlotChunk], z2[kSlotChunk];
#pragma unroll
        for (int u = 0; u < kSlotChunk; ++u) {
            const int sl = s0 + u;
            const int sa = sl < B ? sl : 0;
            const int mb = 2 * sl + 1 < Mc ? 2 * sl + 1 : 0;
            const float2* Z = bufs + (size_t)sa * BUF;
            z1[u] = Z[f];
            z2[u] = Z[fr];
            ga[u] = g1[(2 * sa) * F + f];
            gb[u] = g1[mb * F + f];
        }
#pragma unroll
        for (int u = 0; u < kSlotChunk; ++u) {
            const int sl = s0 + u;
            if (sl < B) {
                float2* Z = bufs + (size_t)sl * BUF;
                const bool hb = 2 * sl + 1 < Mc;
                const float2 va = f2(z1[u].x + z2[u].x, z1[u].y - z2[u].y);
                const float2 vb = f2(z1[u].y + z2[u].y, z2[u].x - z1[u].x);
                float2 xa = cjfma(ga[u], W2, va);
                float2 xb = hb ? cjfma(gb[u], W2, vb) : f2(0.f, 0.f);
                xa = f2(__fmul_rn(xa.x, sch), __fmul_rn(xa.y, sch));
                xb = f2(__fmul_rn(xb.x, sch), __fmul_rn(xb.y, sch));
                if (edge) {
                    Z[f] = f2(xa.x, xb.x);
                } else {
                    Z[f] = f2(xa.x - xb.y, xa.y + xb.x);
                    Z[Lg - f] = f2(xa.x + xb.y, xb.x - xa.y);
                }
            }
        }
    }
}

// Uploads this translation unit's trig tables, once per device: every context reads
// the same values, and a context's setup must not write them under another context's
// kernels.
inline cudaError_t regfft_upload_tables() {
    static std::mutex mu;
    static bool done[64];
    int dev = 0;
    cudaError_t e0 = cudaGetDevice(&dev);
    if (e0 != cudaSuccess) return e0;
    std::lock_guard<std::mutex> lk(mu);
    if (dev >= 0 && dev < 64 && done[dev]) return cudaSuccess;
    std::vector<float2> trig(kTrigW);
    for (int p : kPrimesW)
        for (int m = 0; m < p; ++m)
            trig[toff(p) + m] = make_float2((float)cos(2.0 * M_PI * m / p), (float)sin(2.0 * M_PI * m / p));
    std::vector<float2> w32(32);
    for (int j = 0; j < 32; ++j) w32[j] = make_float2((float)cos(2.0 * M_PI * j / 32), (float)-sin(2.0 * M_PI * j / 32));
    cudaError_t e = cudaMemcpyToSymbol(c_trigw, trig.data(), trig.size() * sizeof(float2));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_w32, w32.data(), 32 * sizeof(float2));
    // a copy from pageable memory may return before it lands, and the contexts' streams
    // do not wait on the legacy stream: wait for the copies there (not on other streams)
    if (e == cudaSuccess) e = cudaStreamSynchronize(0);
    if (e == cudaSuccess && dev >= 0 && dev < 64) done[dev] = true;
    return e;
}

// [P][N1] table exp(-2 pi i n1 k2 / Lg), Lg = N1 P
inline std::vector<float2> regfft_twiddles(int N1, int P) {
    const int Lg = N1 * P;
    std::vector<float2> tw2((size_t)P * N1);
    for (int k2 = 0; k2 < P; ++k2)
        for (int n1 = 0; n1 < N1; ++n1) {
            double a = 2.0 * M_PI * (double)((n1 * k2) % Lg) / Lg;
            tw2[(size_t)k2 * N1 + n1] = make_float2((float)cos(a), (float)-sin(a));
        }
    return tw2;
}

}  // namespace
