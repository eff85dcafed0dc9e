// The D-step's transforms (dict_update!, src/CDL/train.jl:52-62) as streaming kernels
// for the transform lengths with register-resident FFTs (regfft.cuh): k_dfwd (below)
// and the inverse k_dinv (further down, d = irfft(d-hat) per filter pair).
//
// For every (sequence n, filter pair a = 2s, b = 2s + 1) a lane group forms, straight
// from the state arrays, the three packed real pairs the D-step transforms (for an odd M
// the last pair has no filter b: that lane group reads and transforms filter a's row in
// its place and stores filter a's spectrum only) --
//   Y3 = projectionX!(X + y3)                 (X + y3 on the rows l % 4 == 0, else 0)
//   H  = (G1 - g1) + (G3 - g3)                (the filter-domain terms of sherman_CDL_RHS!)
//   d  (the previous iterate)
// -- runs the four-step FFT on each and writes the split half-spectra (f = 0..Lg/2) of
// both filters where the per-frequency solve expects them, (n, m, f).  It replaces a
// pass that wrote Y3 and H to HBM and three cuFFT R2C transforms (each a complex FFT
// and a post-processing pass over the spectra).
//
// This header holds the kernel templates; dstream_v*.cu instantiate them per length
// (one group per translation unit, so the build compiles them in parallel; every unit
// has its own copy of the register FFTs' constant tables and uploads it), and
// dstream.cu holds the host side.
#pragma once

#include "cdlgb_internal.h"
#include "regfft.cuh"

#include <stdlib.h>
#include <vector>

namespace dstream {

struct FArgs {
    const float* X;       // chunk (cn, M, Lg)
    const float* y3;
    const float* g1;
    const float* g3;
    const float* d;
    const float* G1;      // (M, Lg)
    const float* G3;
    float2* Yh;           // chunk (cn, M, F)
    float2* Hh;
    float2* Dh;
    const float2* tw2;    // [P][N1]
    int cn, M;
};

struct IArgsD {
    const float2* Dh;     // chunk (cn, M, F), unscaled
    float* d;             // chunk (cn, M, Lg)
    const float2* tw2;
    float scale;          // 1 / Lg, applied as the spectrum is read
    int cn, M;
};

typedef void (*kern_t)(FArgs);
typedef void (*kinv_t)(IArgsD);
typedef void (*kr2c_t)(const float*, float2*, const float2*, long, int);
typedef void (*kc2r_t)(const float2*, float*, const float2*, long, int);
// one transform length: the forward D-step transforms, their inverse, the row R2C and
// C2R; tables uploads the constant tables of the unit that instantiated them
struct Variant { int N1, P; kern_t k; kinv_t ki; kr2c_t kf; kc2r_t kb; cudaError_t (*tables)(); };

}  // namespace dstream

namespace {

using dstream::FArgs;
using dstream::IArgsD;

// split the packed spectrum Z = A + i B of two real sequences held in natural order in
// `buf` and store A[f], B[f] for f = 0..Lg/2 (lanes over f).  B is stored first: with
// ob == oa (a pair without a second sequence) A is what remains.
template <int Lg, int N1>
__device__ __forceinline__ void split_store(const float2* __restrict__ buf, int gl,
                                            float2* oa, float2* ob) {
    constexpr int F = Lg / 2 + 1;
    for (int f = gl; f < F; f += N1) {
        const float2 z1 = buf[f], z2 = buf[f == 0 ? 0 : Lg - f];
        ob[f] = f2(0.5f * (z1.y + z2.y), 0.5f * (z2.x - z1.x));
        oa[f] = f2(0.5f * (z1.x + z2.x), 0.5f * (z1.y - z2.y));
    }
}

// one of the three transforms of k_dfwd for the lane group's (sequence, filter pair):
// WHICH 0: Y3 = projectionX!(X + y3) (rows l % 4 == 0 only), 1: H = (G1 - g1) + (G3 - g3),
// 2: the previous d.  The state is read through the read-only path; P rows per column.
// bo: the offset of filter b's rows from filter a's (Lg; 0 for the last pair of an odd M,
// which has no filter b), fo the same for the spectra (F; 0).
template <int N1, int P, int WHICH>
__device__ __forceinline__ void dfwd_one(const FArgs& A, float2* sb, int gl, const float2* tw2,
                                         bool act, bool keep, int bo, int fo, size_t ra, size_t pa,
                                         size_t oa) {
    constexpr int Lg = N1 * P;
    constexpr int RS = N1 + 1;
    constexpr int F = Lg / 2 + 1;
    if (act) {
#pragma unroll 16
        for (int n2 = 0; n2 < P; ++n2) {
            const int o = N1 * n2;
            float2 v;
            if (WHICH == 0) {
                // Y3 = X + y3 on the kept rows.  Every X-step leaves y3 = +0 exactly there
                // (projectionX! keeps X + y3, so y3' = (y3 + X) - Y3 is set to +0, as
                // initialisation does), so X + 0 gives the same bits without reading y3.
                v = keep ? f2(__ldg(A.X + ra + o) + 0.f, __ldg(A.X + ra + bo + o) + 0.f)
                         : f2(0.f, 0.f);
            } else if (WHICH == 1) {
                v = f2((__ldg(A.G1 + pa + o) - __ldg(A.g1 + ra + o)) + (__ldg(A.G3 + pa + o) - __ldg(A.g3 + ra + o)),
                       (__ldg(A.G1 + pa + bo + o) - __ldg(A.g1 + ra + bo + o)) +
                           (__ldg(A.G3 + pa + bo + o) - __ldg(A.g3 + ra + bo + o)));
            } else {
                v = f2(__ldg(A.d + ra + o), __ldg(A.d + ra + bo + o));
            }
            sb[n2 * RS + gl] = v;
        }
        fwd_step1<N1, P>(sb, gl, tw2);
    }
    __syncwarp();
    fwd_step2<N1, P>(sb, gl, act);
    if (act) {
        float2* out = WHICH == 0 ? A.Yh : WHICH == 1 ? A.Hh : A.Dh;
        split_store<Lg, N1>(sb, gl, out + oa, out + oa + fo);
    }
    __syncwarp();
}

template <int N1, int P>
__global__ void __launch_bounds__(256, 2) k_dfwd(FArgs A) {
    constexpr int Lg = N1 * P;
    constexpr int G = 32 / N1;
    constexpr int RS = N1 + 1;
    constexpr int BUF = (P * RS + 1) & ~1;
    constexpr int F = Lg / 2 + 1;
    extern __shared__ float4 smem4[];
    float2* tw2 = reinterpret_cast<float2*>(smem4);        // [P][N1]
    float2* bufs = tw2 + P * N1;                           // [groups][BUF]
    for (int t = threadIdx.x; t < P * N1; t += blockDim.x) tw2[t] = A.tw2[t];
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const int gw = (threadIdx.x >> 5) * G + lane / N1;     // lane group in the CTA
    const int gl = lane % N1;
    const int groups = (blockDim.x >> 5) * G;
    const bool keep = (gl & 3) == 0;                       // l = gl + N1 n2, N1 % 4 == 0
    float2* sb = bufs + (size_t)gw * BUF;
    const int pairs = (A.M + 1) / 2;
    const long items = (long)A.cn * pairs;
    const long stride = (long)gridDim.x * groups;
    // every lane group of a warp runs the same number of rounds (the row DFT syncs the warp)
    const long rounds = (items + stride - 1) / stride;
    for (long r = 0; r < rounds; ++r) {
        const long item = r * stride + (long)blockIdx.x * groups + gw;
        const bool act = item < items;
        const long n = act ? item / pairs : 0;
        const int s = act ? (int)(item - n * pairs) : 0;
        const int ma = 2 * s;
        const size_t ra = ((size_t)n * A.M + ma) * Lg + gl;   // row of filter a at lane gl
        const size_t pa = (size_t)ma * Lg + gl;
        const size_t oa = ((size_t)n * A.M + ma) * F;
        const bool hb = ma + 1 < A.M;
        const int bo = hb ? Lg : 0, fo = hb ? F : 0;
        dfwd_one<N1, P, 0>(A, sb, gl, tw2, act, keep, bo, fo, ra, pa, oa);
        if (A.Hh) dfwd_one<N1, P, 1>(A, sb, gl, tw2, act, keep, bo, fo, ra, pa, oa);   // uniform
        if (A.Dh) dfwd_one<N1, P, 2>(A, sb, gl, tw2, act, keep, bo, fo, ra, pa, oa);
    }
}

// Inverse: for every (n, filter pair) the two half-spectra dh[a], dh[b] (scaled by 1/Lg
// as they are read) are packed into one full spectrum Z = Dh_a + i Dh_b (Z[f], and Z[Lg - f] =
// conj(Dh_a[f]) + i conj(Dh_b[f])), inverted with the register four-step FFT, and
// d[a] = Re, d[b] = Im written (as a C2R per filter, the imaginary parts of the
// half-spectrum's f = 0 and f = Lg/2 bins are dropped; for an odd M the last pair reads
// Dh_a for both halves and writes d[a] only: its Im store goes to d[a] first).

template <int N1, int P>
__global__ void __launch_bounds__(256, 2) k_dinv(IArgsD A) {
    constexpr int Lg = N1 * P;
    constexpr int G = 32 / N1;
    constexpr int RS = N1 + 1;
    constexpr int BUF = (P * RS + 1) & ~1;
    constexpr int F = Lg / 2 + 1;
    constexpr int half = Lg / 2;
    extern __shared__ float4 smem4[];
    float2* tw2 = reinterpret_cast<float2*>(smem4);
    float2* bufs = tw2 + P * N1;
    for (int t = threadIdx.x; t < P * N1; t += blockDim.x) tw2[t] = A.tw2[t];
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const int gw = (threadIdx.x >> 5) * G + lane / N1;
    const int gl = lane % N1;
    const int groups = (blockDim.x >> 5) * G;
    float2* sb = bufs + (size_t)gw * BUF;
    const int pairs = (A.M + 1) / 2;
    const long items = (long)A.cn * pairs;
    const long stride = (long)gridDim.x * groups;
    const long rounds = (items + stride - 1) / stride;
    for (long r = 0; r < rounds; ++r) {
        const long item = r * stride + (long)blockIdx.x * groups + gw;
        const bool act = item < items;
        const long n = act ? item / pairs : 0;
        const int s = act ? (int)(item - n * pairs) : 0;
        const size_t ia = ((size_t)n * A.M + 2 * s) * F;
        const bool hb = 2 * s + 1 < A.M;                   // false: the last pair of an odd M
        const size_t ib = ia + (hb ? F : 0);
        if (act) {
#pragma unroll 5
            for (int f = gl; f < F; f += N1) {
                float2 a = __ldg(A.Dh + ia + f), b = __ldg(A.Dh + ib + f);
                a = f2(a.x * A.scale, a.y * A.scale);
                b = f2(b.x * A.scale, b.y * A.scale);
                if (f == 0 || f == half) {
                    sb[f] = f2(a.x, b.x);
                } else {
                    sb[f] = f2(a.x - b.y, a.y + b.x);
                    sb[Lg - f] = f2(a.x + b.y, b.x - a.y);
                }
            }
        }
        __syncwarp();
        inv_step2<N1, P, false>(sb, gl, act, tw2);
        if (act) {
            inv_step1<N1, P, true>(sb, gl, tw2);
            const size_t ra = ((size_t)n * A.M + 2 * s) * Lg + gl;
            const size_t rb = ra + (hb ? Lg : 0);
#pragma unroll 4
            for (int n2 = 0; n2 < P; ++n2) {
                const float2 v = sb[n2 * RS + gl];
                A.d[rb + N1 * n2] = v.y;
                A.d[ra + N1 * n2] = v.x;
            }
        }
        __syncwarp();
    }
}

// Batched real transforms of R contiguous rows, in the layouts of the cuFFT batched plans
// they replace (rows of Lg floats; half-spectra of F = Lg/2 + 1 bins; unnormalised both
// ways, so C2R returns Lg times the input row).  The rows come in groups of grp
// consecutive rows (R a multiple of grp); inside a group, rows 2j and 2j + 1 form one
// complex transform of a lane group (the last row of an odd group is paired with zeros),
// so no row's rounding depends on a row of another group.  The forward split is
// split_store's; the inverse packs Z = A + i B from both half-spectra and drops the
// imaginary parts of bins 0 and Lg/2, as k_dinv does.
template <int N1, int P>
__global__ void __launch_bounds__(256, 2) k_rows_r2c(const float* __restrict__ x, float2* __restrict__ X,
                                                     const float2* __restrict__ tw2g, long R, int grp) {
    constexpr int Lg = N1 * P;
    constexpr int G = 32 / N1;
    constexpr int RS = N1 + 1;
    constexpr int BUF = (P * RS + 1) & ~1;
    constexpr int F = Lg / 2 + 1;
    extern __shared__ float4 smem4[];
    float2* tw2 = reinterpret_cast<float2*>(smem4);
    float2* bufs = tw2 + P * N1;
    for (int t = threadIdx.x; t < P * N1; t += blockDim.x) tw2[t] = tw2g[t];
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const int gw = (threadIdx.x >> 5) * G + lane / N1;
    const int gl = lane % N1;
    const int groups = (blockDim.x >> 5) * G;
    float2* sb = bufs + (size_t)gw * BUF;
    const int ppg = (grp + 1) / 2;                         // pairs per group
    const long items = (R / grp) * ppg;
    const long stride = (long)gridDim.x * groups;
    const long rounds = (items + stride - 1) / stride;
    for (long r = 0; r < rounds; ++r) {
        const long item = r * stride + (long)blockIdx.x * groups + gw;
        const bool act = item < items;
        const long g = act ? item / ppg : 0;
        const int j = act ? (int)(item - g * ppg) : 0;
        const long a = g * grp + 2 * j;
        const bool hb = 2 * j + 1 < grp;
        if (act) {
            const float* xa = x + (size_t)a * Lg + gl;
#pragma unroll 16
            for (int n2 = 0; n2 < P; ++n2) {
                const int o = N1 * n2;
                sb[n2 * RS + gl] = f2(__ldg(xa + o), hb ? __ldg(xa + Lg + o) : 0.f);
            }
            fwd_step1<N1, P>(sb, gl, tw2);
        }
        __syncwarp();
        fwd_step2<N1, P>(sb, gl, act);
        if (act) {
            float2* oa = X + (size_t)a * F;
            for (int f = gl; f < F; f += N1) {
                const float2 z1 = sb[f], z2 = sb[f == 0 ? 0 : Lg - f];
                oa[f] = f2(0.5f * (z1.x + z2.x), 0.5f * (z1.y - z2.y));
                if (hb) oa[F + f] = f2(0.5f * (z1.y + z2.y), 0.5f * (z2.x - z1.x));
            }
        }
        __syncwarp();
    }
}

template <int N1, int P>
__global__ void __launch_bounds__(256, 2) k_rows_c2r(const float2* __restrict__ X, float* __restrict__ x,
                                                     const float2* __restrict__ tw2g, long R, int grp) {
    constexpr int Lg = N1 * P;
    constexpr int G = 32 / N1;
    constexpr int RS = N1 + 1;
    constexpr int BUF = (P * RS + 1) & ~1;
    constexpr int F = Lg / 2 + 1;
    constexpr int half = Lg / 2;
    extern __shared__ float4 smem4[];
    float2* tw2 = reinterpret_cast<float2*>(smem4);
    float2* bufs = tw2 + P * N1;
    for (int t = threadIdx.x; t < P * N1; t += blockDim.x) tw2[t] = tw2g[t];
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const int gw = (threadIdx.x >> 5) * G + lane / N1;
    const int gl = lane % N1;
    const int groups = (blockDim.x >> 5) * G;
    float2* sb = bufs + (size_t)gw * BUF;
    const int ppg = (grp + 1) / 2;                         // pairs per group
    const long items = (R / grp) * ppg;
    const long stride = (long)gridDim.x * groups;
    const long rounds = (items + stride - 1) / stride;
    for (long r = 0; r < rounds; ++r) {
        const long item = r * stride + (long)blockIdx.x * groups + gw;
        const bool act = item < items;
        const long g = act ? item / ppg : 0;
        const int j = act ? (int)(item - g * ppg) : 0;
        const long a = g * grp + 2 * j;
        const bool hb = 2 * j + 1 < grp;
        if (act) {
            const float2* ia = X + (size_t)a * F;
#pragma unroll 5
            for (int f = gl; f < F; f += N1) {
                const float2 A = __ldg(ia + f), B = hb ? __ldg(ia + F + f) : f2(0.f, 0.f);
                if (f == 0 || f == half) {
                    sb[f] = f2(A.x, B.x);
                } else {
                    sb[f] = f2(A.x - B.y, A.y + B.x);
                    sb[Lg - f] = f2(A.x + B.y, B.x - A.y);
                }
            }
        }
        __syncwarp();
        inv_step2<N1, P, false>(sb, gl, act, tw2);
        if (act) {
            inv_step1<N1, P, true>(sb, gl, tw2);
            float* ra = x + (size_t)a * Lg + gl;
#pragma unroll 4
            for (int n2 = 0; n2 < P; ++n2) {
                const float2 v = sb[n2 * RS + gl];
                ra[N1 * n2] = v.x;
                if (hb) ra[Lg + N1 * n2] = v.y;
            }
        }
        __syncwarp();
    }
}

}  // namespace

#define DSTREAM_VARIANT(N1, P) \
    {N1, P, k_dfwd<N1, P>, k_dinv<N1, P>, k_rows_r2c<N1, P>, k_rows_c2r<N1, P>, regfft_upload_tables}
