// PWM scan and count kernels (src/SEARCH/scan.jl, src/SEARCH/helpers.jl).
//
// Scores are summed in float32 with one rounded multiply and one rounded add per
// term (__fmul_rn / __fadd_rn: no FMA contraction), in the order of the reference
// path being replaced, so positions and scores are bit-identical to it (REF_QUIRK_Q7):
//   greedy_search! (scan.jl:223-239): position-major, ind outer, nucleotide inner;
//   scan_n (scan.jl:10-21):           nucleotide-major, j outer, k inner.
#include "cdlgb_internal.h"

#include <math.h>
#include <vector>

namespace {

constexpr int kScanThreads = 256;

// order-preserving reduction of (value, index): larger value wins, ties -> lower index
struct VI { float v; int i; };
__device__ __forceinline__ VI vi_best(VI a, VI b) {
    bool take_b = (b.v > a.v) || (b.v == a.v && b.i < a.i);
    return take_b ? b : a;
}
__device__ VI block_argmax(VI x, VI* sh) {
    for (int o = 16; o > 0; o >>= 1) {
        VI y;
        y.v = __shfl_xor_sync(0xffffffffu, x.v, o);
        y.i = __shfl_xor_sync(0xffffffffu, x.i, o);
        x = vi_best(x, y);
    }
    int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) sh[w] = x;
    __syncthreads();
    if (w == 0) {
        x = lane < (int)(blockDim.x >> 5) ? sh[lane] : VI{-INFINITY, 0x7fffffff};
        for (int o = 16; o > 0; o >>= 1) {
            VI y;
            y.v = __shfl_xor_sync(0xffffffffu, x.v, o);
            y.i = __shfl_xor_sync(0xffffffffu, x.i, o);
            x = vi_best(x, y);
        }
        if (lane == 0) sh[0] = x;
    }
    __syncthreads();
    VI r = sh[0];
    __syncthreads();
    return r;
}

// one block per sequence n; loops over motifs k; threads over positions.
// pwms: (K, 4, maxlen) col-major; out pos: (K, N) col-major.
__global__ void k_scan_fwd(const float* __restrict__ data, const float* __restrict__ pwms,
                           const int32_t* __restrict__ lens, const float* __restrict__ thresh,
                           int K, int maxlen, int L, int32_t* __restrict__ pos) {
    extern __shared__ float xs[];      // one-hot column, 4L floats
    __shared__ VI red[32];
    const int n = blockIdx.x;
    const float* col = data + (size_t)n * 4 * L;
    for (int i = threadIdx.x; i < 4 * L; i += blockDim.x) xs[i] = col[i];
    __syncthreads();
    for (int k = 0; k < K; ++k) {
        const int w = lens[k];
        const float th = thresh[k];
        VI best{-INFINITY, 0x7fffffff};
        for (int l = threadIdx.x; l < L; l += blockDim.x) {
            float v = 0.f;
            if (l <= L - w) {
                float s = 0.f;
                for (int ind = 0; ind < w; ++ind)
#pragma unroll
                    for (int a = 0; a < 4; ++a)
                        s = __fadd_rn(s, __fmul_rn(pwms[k + K * (a + 4 * ind)], xs[(l + ind) * 4 + a]));
                v = s > th ? s : 0.f;
            }
            best = vi_best(best, VI{v, l});
        }
        VI r = block_argmax(best, red);
        // REF_QUIRK_Q3: a best hit at the first position reads as no hit (scan.jl:197)
        if (threadIdx.x == 0) pos[k + (size_t)K * n] = (r.i == 0) ? 0 : r.i + 1;
    }
}

// scan_n on both strands; complement pwm_c[j, kk] = pwm[3-j, w-1-kk] (reverse of the
// matrix).  Strict '>' from -Inf: NaN and -Inf never become the maximum.
__global__ void k_scan_both(const float* __restrict__ data, const float* __restrict__ pwms,
                            const int32_t* __restrict__ lens, const float* __restrict__ thresh,
                            int K, int maxlen, int L, int32_t* __restrict__ pos,
                            float* __restrict__ score, uint8_t* __restrict__ comp) {
    extern __shared__ float xs[];
    __shared__ VI red[32];
    const int n = blockIdx.x;
    const float* col = data + (size_t)n * 4 * L;
    for (int i = threadIdx.x; i < 4 * L; i += blockDim.x) xs[i] = col[i];
    __syncthreads();
    for (int k = 0; k < K; ++k) {
        const int w = lens[k];
        VI bf{-INFINITY, 0x7fffffff}, bc{-INFINITY, 0x7fffffff};
        for (int l = threadIdx.x; l <= L - w; l += blockDim.x) {
            float sf = 0.f, sc = 0.f;
            for (int j = 0; j < 4; ++j)
                for (int kk = 0; kk < w; ++kk) {
                    float x = xs[(l + kk) * 4 + j];
                    sf = __fadd_rn(sf, __fmul_rn(pwms[k + K * (j + 4 * kk)], x));
                    sc = __fadd_rn(sc, __fmul_rn(pwms[k + K * ((3 - j) + 4 * (w - 1 - kk))], x));
                }
            if (sf > -INFINITY) bf = vi_best(bf, VI{sf, l});
            if (sc > -INFINITY) bc = vi_best(bc, VI{sc, l});
        }
        VI rf = block_argmax(bf, red);
        VI rc = block_argmax(bc, red);
        if (threadIdx.x == 0) {
            // no candidate -> (-1, -Inf) as scan_n returns
            float sF = rf.i == 0x7fffffff ? -INFINITY : rf.v;
            float sC = rc.i == 0x7fffffff ? -INFINITY : rc.v;
            int iF = rf.i == 0x7fffffff ? -1 : rf.i + 1;
            int iC = rc.i == 0x7fffffff ? -1 : rc.i + 1;
            bool fwd = sF >= sC;
            float s = fwd ? sF : sC;
            bool keep = s > thresh[k];
            size_t o = k + (size_t)K * n;
            if (pos) pos[o] = keep ? (fwd ? iF : iC) : 0;
            if (score) score[o] = keep ? s : 0.f;
            if (comp) comp[o] = (keep && !fwd) ? 1 : 0;
        }
    }
}

// k_scan_both with the block's inputs staged once: the sequence base-major (xt[j][p],
// so consecutive positions are consecutive words), every PWM and its reverse complement
// as (fwd, comp) pairs in the order the sums consume them (pw[k][j][kk]), one position
// per thread, and the argmax of each motif reduced within each warp by shuffles (no
// barrier) and across the warps once, after the last motif.  The products and sums are
// k_scan_both's, in its order, and the (value, index) reduction is the same total order,
// so positions, scores and strands are bit-identical to it.
__global__ void k_scan_both_staged(const float* __restrict__ data, const float* __restrict__ pwms,
                                   const int32_t* __restrict__ lens, const float* __restrict__ thresh,
                                   int K, int maxlen, int L, int32_t* __restrict__ pos,
                                   float* __restrict__ score, uint8_t* __restrict__ comp) {
    extern __shared__ float4 sm4s[];
    const int nw = blockDim.x >> 5, lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    float2* pw = reinterpret_cast<float2*>(sm4s);                  // [K][4][maxlen]
    VI* wb = reinterpret_cast<VI*>(pw + (size_t)K * 4 * maxlen);     // [K][nw][2]
    float* xt = reinterpret_cast<float*>(wb + (size_t)K * nw * 2);  // [4][L]
    const int n = blockIdx.x;
    const float* col = data + (size_t)n * 4 * L;
    for (int i = threadIdx.x; i < 4 * L; i += blockDim.x) xt[(i & 3) * L + (i >> 2)] = col[i];
    const int per = 4 * maxlen;
    for (int i = threadIdx.x; i < K * per; i += blockDim.x) {
        const int k = i / per, r = i - k * per, j = r / maxlen, kk = r - j * maxlen;
        const int w = lens[k];
        float f = 0.f, cc = 0.f;
        if (kk < w) {
            f = pwms[k + K * (j + 4 * kk)];
            cc = pwms[k + K * ((3 - j) + 4 * (w - 1 - kk))];
        }
        pw[i] = make_float2(f, cc);
    }
    __syncthreads();
    const int l = threadIdx.x;
    for (int k = 0; k < K; ++k) {
        const int w = lens[k];
        VI bf{-INFINITY, 0x7fffffff}, bc{-INFINITY, 0x7fffffff};
        if (l <= L - w) {
            const float2* p = pw + (size_t)k * per;
            float sf = 0.f, sc = 0.f;
            for (int j = 0; j < 4; ++j) {
                const float* xr = xt + j * L + l;
                const float2* pj = p + j * maxlen;
#pragma unroll 4
                for (int kk = 0; kk < w; ++kk) {
                    const float x = xr[kk];
                    const float2 q = pj[kk];
                    sf = __fadd_rn(sf, __fmul_rn(q.x, x));
                    sc = __fadd_rn(sc, __fmul_rn(q.y, x));
                }
            }
            if (sf > -INFINITY) bf = VI{sf, l};
            if (sc > -INFINITY) bc = VI{sc, l};
        }
        for (int o = 16; o > 0; o >>= 1) {
            VI y;
            y.v = __shfl_xor_sync(0xffffffffu, bf.v, o);
            y.i = __shfl_xor_sync(0xffffffffu, bf.i, o);
            bf = vi_best(bf, y);
            y.v = __shfl_xor_sync(0xffffffffu, bc.v, o);
            y.i = __shfl_xor_sync(0xffffffffu, bc.i, o);
            bc = vi_best(bc, y);
        }
        if (lane == 0) {
            wb[((size_t)k * nw + wid) * 2] = bf;
            wb[((size_t)k * nw + wid) * 2 + 1] = bc;
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        VI rf{-INFINITY, 0x7fffffff}, rc{-INFINITY, 0x7fffffff};
        for (int v = 0; v < nw; ++v) {
            rf = vi_best(rf, wb[((size_t)k * nw + v) * 2]);
            rc = vi_best(rc, wb[((size_t)k * nw + v) * 2 + 1]);
        }
        const float sF = rf.i == 0x7fffffff ? -INFINITY : rf.v;
        const float sC = rc.i == 0x7fffffff ? -INFINITY : rc.v;
        const int iF = rf.i == 0x7fffffff ? -1 : rf.i + 1;
        const int iC = rc.i == 0x7fffffff ? -1 : rc.i + 1;
        const bool fwd = sF >= sC;
        const float sv = fwd ? sF : sC;
        const bool keep = sv > thresh[k];
        const size_t o = k + (size_t)K * n;
        if (pos) pos[o] = keep ? (fwd ? iF : iC) : 0;
        if (score) score[o] = keep ? sv : 0.f;
        if (comp) comp[o] = (keep && !fwd) ? 1 : 0;
    }
}

// ---------------------------------------------------------------- sparse scans
// On 0/1 data every term whose one-hot entry is 0 is pwm * 0 = +-0 for a finite pwm,
// and adding +-0 to a partial sum that starts at +0 leaves it unchanged (s + -0 = s for
// s != 0, +0 + -0 = +0, and the sum is never -0); a term whose entry is 1 is pwm * 1 =
// pwm.  So the sum of the nonzero terms alone, added in the reference's order, has the
// same bits: about w terms per window instead of 4 w products and sums.  Taken only
// when the data is exact 0/1 and every PWM entry finite (an infinite entry times 0 is
// NaN, which the dense kernels keep).

// the base bits of position p of the staged sequence: bit j set when entry j is 1
__device__ __forceinline__ uint32_t base_bits(const float* col, int p) {
    const float4 v = reinterpret_cast<const float4*>(col)[p];
    return (v.x != 0.f ? 1u : 0u) | (v.y != 0.f ? 2u : 0u) | (v.z != 0.f ? 4u : 0u) | (v.w != 0.f ? 8u : 0u);
}

// greedy_search! (scan.jl:223-239: position-major, nucleotide inner) on 0/1 data, one
// position per thread: for ind = 0 .. w-1 the entries of base(l + ind) in nucleotide
// order.  Same candidates and (value, index) order as k_scan_fwd.
__global__ void k_scan_fwd_sparse(const float* __restrict__ data, const float* __restrict__ pwms,
                                  const int32_t* __restrict__ lens, const float* __restrict__ thresh,
                                  int K, int maxlen, int L, int32_t* __restrict__ pos) {
    extern __shared__ float4 sm4f[];
    const int nw = blockDim.x >> 5, lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    float* pw = reinterpret_cast<float*>(sm4f);                    // [K][maxlen][4]
    VI* wb = reinterpret_cast<VI*>(pw + (size_t)K * 4 * maxlen);     // [K][nw]
    uint8_t* bb = reinterpret_cast<uint8_t*>(wb + (size_t)K * nw);  // [L] base bits
    const int n = blockIdx.x;
    const float* col = data + (size_t)n * 4 * L;
    for (int i = threadIdx.x; i < L; i += blockDim.x) bb[i] = (uint8_t)base_bits(col, i);
    for (int i = threadIdx.x; i < K * 4 * maxlen; i += blockDim.x) {
        const int k = i / (4 * maxlen), r = i - k * 4 * maxlen, ind = r >> 2, a = r & 3;
        pw[i] = pwms[k + K * (a + 4 * ind)];
    }
    __syncthreads();
    const int l = threadIdx.x;
    for (int k = 0; k < K; ++k) {
        const int w = lens[k];
        VI best{-INFINITY, 0x7fffffff};
        if (l < L) {
            float v = 0.f;
            if (l <= L - w) {
                const float* p = pw + (size_t)k * 4 * maxlen;
                float s = 0.f;
                for (int ind = 0; ind < w; ++ind) {
                    uint32_t b = bb[l + ind];
                    while (b) {
                        const int a = __ffs(b) - 1;
                        b &= b - 1;
                        s = __fadd_rn(s, p[4 * ind + a]);
                    }
                }
                v = s > thresh[k] ? s : 0.f;
            }
            best = VI{v, l};
        }
        for (int o = 16; o > 0; o >>= 1) {
            VI y;
            y.v = __shfl_xor_sync(0xffffffffu, best.v, o);
            y.i = __shfl_xor_sync(0xffffffffu, best.i, o);
            best = vi_best(best, y);
        }
        if (lane == 0) wb[(size_t)k * nw + wid] = best;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        VI r{-INFINITY, 0x7fffffff};
        for (int v = 0; v < nw; ++v) r = vi_best(r, wb[(size_t)k * nw + v]);
        // REF_QUIRK_Q3: a best hit at the first position reads as no hit (scan.jl:197)
        pos[k + (size_t)K * n] = (r.i == 0) ? 0 : r.i + 1;
    }
}

// scan_n on both strands (scan.jl:10-21: nucleotide-major) on 0/1 data, one position
// per thread, w <= 64 (MT = uint64_t) or <= 32 (MT = uint32_t): the window's positions
// of base j are the set bits of a mask cut from the sequence's bit plane of j (built
// with one ballot per base and warp of positions), so the nonzero terms are visited j by
// j, ind ascending -- the dense order -- in one loop of exactly that many steps.  The
// (forward, complement) coefficient pairs, the per-warp argmax and the final reduction
// are k_scan_both_staged's.
template <typename MT>
__global__ void k_scan_both_sparse(const float* __restrict__ data, const float* __restrict__ pwms,
                                   const int32_t* __restrict__ lens, const float* __restrict__ thresh,
                                   int K, int maxlen, int L, int32_t* __restrict__ pos,
                                   float* __restrict__ score, uint8_t* __restrict__ comp) {
    extern __shared__ float4 sm4p[];
    const int nw = blockDim.x >> 5, lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nwords = (L + 31) / 32 + 2;                           // two zero words of padding
    float2* pw = reinterpret_cast<float2*>(sm4p);                   // [K][4][maxlen]
    VI* wb = reinterpret_cast<VI*>(pw + (size_t)K * 4 * maxlen);     // [K][nw][2]
    uint32_t* planes = reinterpret_cast<uint32_t*>(wb + (size_t)K * nw * 2);   // [4][nwords]
    const int n = blockIdx.x;
    const float* col = data + (size_t)n * 4 * L;
    {
        // blockDim.x = 32 ceil(L / 32): warp w's ballots are word w of the planes
        const uint32_t bits = threadIdx.x < L ? base_bits(col, threadIdx.x) : 0u;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const uint32_t b = __ballot_sync(0xffffffffu, (bits >> j) & 1u);
            if (lane == 0) planes[j * nwords + wid] = b;
        }
        if (threadIdx.x < 8) planes[(threadIdx.x >> 1) * nwords + nw + (threadIdx.x & 1)] = 0u;
    }
    const int per = 4 * maxlen;
    for (int i = threadIdx.x; i < K * per; i += blockDim.x) {
        const int k = i / per, r = i - k * per, j = r / maxlen, kk = r - j * maxlen;
        const int w = lens[k];
        float f = 0.f, cc = 0.f;
        if (kk < w) {
            f = pwms[k + K * (j + 4 * kk)];
            cc = pwms[k + K * ((3 - j) + 4 * (w - 1 - kk))];
        }
        pw[i] = make_float2(f, cc);
    }
    __syncthreads();
    const int l = threadIdx.x;
    const int wi = l >> 5, sh = l & 31;
    constexpr int MB = 8 * (int)sizeof(MT);
    for (int k = 0; k < K; ++k) {
        const int w = lens[k];
        VI bf{-INFINITY, 0x7fffffff}, bc{-INFINITY, 0x7fffffff};
        if (l <= L - w) {
            const MT keep = w >= MB ? ~(MT)0 : (((MT)1 << w) - 1);
            MT mj[4];
            int cnt = 0;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const uint32_t* pl = planes + j * nwords + wi;
                MT m;
                if (MB == 32) {
                    m = (MT)__funnelshift_r(pl[0], pl[1], sh);
                } else {
                    const uint64_t lo = ((uint64_t)pl[1] << 32) | pl[0];
                    uint64_t m64 = lo >> sh;
                    if (sh) m64 |= (uint64_t)pl[2] << (64 - sh);
                    m = (MT)m64;
                }
                mj[j] = m & keep;
                cnt += MB == 32 ? __popc((uint32_t)mj[j]) : __popcll((unsigned long long)mj[j]);
            }
            const float2* p = pw + (size_t)k * per;
            float sf = 0.f, sc = 0.f;
            int j = 0;
            MT m = mj[0];
            for (int t = 0; t < cnt; ++t) {
                while (m == 0) {
                    ++j;
                    m = j == 1 ? mj[1] : (j == 2 ? mj[2] : mj[3]);
                }
                const int kk = (MB == 32 ? __ffs((int)(uint32_t)m) : __ffsll((long long)m)) - 1;
                m &= m - 1;
                const float2 q = p[j * maxlen + kk];
                sf = __fadd_rn(sf, q.x);
                sc = __fadd_rn(sc, q.y);
            }
            bf = VI{sf, l};
            bc = VI{sc, l};
        }
        for (int o = 16; o > 0; o >>= 1) {
            VI y;
            y.v = __shfl_xor_sync(0xffffffffu, bf.v, o);
            y.i = __shfl_xor_sync(0xffffffffu, bf.i, o);
            bf = vi_best(bf, y);
            y.v = __shfl_xor_sync(0xffffffffu, bc.v, o);
            y.i = __shfl_xor_sync(0xffffffffu, bc.i, o);
            bc = vi_best(bc, y);
        }
        if (lane == 0) {
            wb[((size_t)k * nw + wid) * 2] = bf;
            wb[((size_t)k * nw + wid) * 2 + 1] = bc;
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        VI rf{-INFINITY, 0x7fffffff}, rc{-INFINITY, 0x7fffffff};
        for (int v = 0; v < nw; ++v) {
            rf = vi_best(rf, wb[((size_t)k * nw + v) * 2]);
            rc = vi_best(rc, wb[((size_t)k * nw + v) * 2 + 1]);
        }
        const float sF = rf.i == 0x7fffffff ? -INFINITY : rf.v;
        const float sC = rc.i == 0x7fffffff ? -INFINITY : rc.v;
        const int iF = rf.i == 0x7fffffff ? -1 : rf.i + 1;
        const int iC = rc.i == 0x7fffffff ? -1 : rc.i + 1;
        const bool fwd = sF >= sC;
        const float sv = fwd ? sF : sC;
        const bool keepk = sv > thresh[k];
        const size_t o = k + (size_t)K * n;
        if (pos) pos[o] = keepk ? (fwd ? iF : iC) : 0;
        if (score) score[o] = keepk ? sv : 0.f;
        if (comp) comp[o] = (keepk && !fwd) ? 1 : 0;
    }
}

// k_scan_both_sparse for PWMs of at most 16 columns: the four bases' 16-bit window masks
// are packed into two words, lo = A | C << 16 and hi = G | T << 16, so that ascending bit
// order is the nucleotide-major order and bit b is the coefficient pair at row b of the
// staged table (rows of 16 columns per base): no per-base bookkeeping beyond one switch
// from lo to hi per window.
__global__ void k_scan_both_sparse16(const float* __restrict__ data, const float* __restrict__ pwms,
                                     const int32_t* __restrict__ lens, const float* __restrict__ thresh,
                                     int K, int maxlen, int L, int32_t* __restrict__ pos,
                                     float* __restrict__ score, uint8_t* __restrict__ comp) {
    extern __shared__ float4 sm4q[];
    const int nw = blockDim.x >> 5, lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nwords = (L + 31) / 32 + 2;
    float2* pw = reinterpret_cast<float2*>(sm4q);                   // [K][4][16]
    VI* wb = reinterpret_cast<VI*>(pw + (size_t)K * 64);             // [K][nw][2]
    uint32_t* planes = reinterpret_cast<uint32_t*>(wb + (size_t)K * nw * 2);   // [4][nwords]
    const int n = blockIdx.x;
    const float* col = data + (size_t)n * 4 * L;
    {
        const uint32_t bits = threadIdx.x < L ? base_bits(col, threadIdx.x) : 0u;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const uint32_t b = __ballot_sync(0xffffffffu, (bits >> j) & 1u);
            if (lane == 0) planes[j * nwords + wid] = b;
        }
        if (threadIdx.x < 8) planes[(threadIdx.x >> 1) * nwords + nw + (threadIdx.x & 1)] = 0u;
    }
    for (int i = threadIdx.x; i < K * 64; i += blockDim.x) {
        const int k = i >> 6, j = (i >> 4) & 3, kk = i & 15;
        const int w = lens[k];
        float f = 0.f, cc = 0.f;
        if (kk < w) {
            f = pwms[k + K * (j + 4 * kk)];
            cc = pwms[k + K * ((3 - j) + 4 * (w - 1 - kk))];
        }
        pw[i] = make_float2(f, cc);
    }
    __syncthreads();
    const int l = threadIdx.x;
    const int wi = l >> 5, sh = l & 31;
    uint32_t win[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const uint32_t* pl = planes + j * nwords + wi;
        win[j] = __funnelshift_r(pl[0], pl[1], sh);     // positions l .. l + 31 of base j
    }
    for (int k = 0; k < K; ++k) {
        const int w = lens[k];
        VI bf{-INFINITY, 0x7fffffff}, bc{-INFINITY, 0x7fffffff};
        if (l <= L - w) {
            const uint32_t keep = (1u << w) - 1u;         // w <= 16
            uint32_t lo = (win[0] & keep) | ((win[1] & keep) << 16);
            uint32_t hi = (win[2] & keep) | ((win[3] & keep) << 16);
            const int cnt = __popc(lo) + __popc(hi);
            const float2* p = pw + (size_t)k * 64;
            float sf = 0.f, sc = 0.f;
            for (int t = 0; t < cnt; ++t) {
                if (lo == 0) {
                    lo = hi;
                    hi = 0;
                    p += 32;
                }
                const int b = __ffs((int)lo) - 1;
                lo &= lo - 1;
                const float2 q = p[b];
                sf = __fadd_rn(sf, q.x);
                sc = __fadd_rn(sc, q.y);
            }
            bf = VI{sf, l};
            bc = VI{sc, l};
        }
        for (int o = 16; o > 0; o >>= 1) {
            VI y;
            y.v = __shfl_xor_sync(0xffffffffu, bf.v, o);
            y.i = __shfl_xor_sync(0xffffffffu, bf.i, o);
            bf = vi_best(bf, y);
            y.v = __shfl_xor_sync(0xffffffffu, bc.v, o);
            y.i = __shfl_xor_sync(0xffffffffu, bc.i, o);
            bc = vi_best(bc, y);
        }
        if (lane == 0) {
            wb[((size_t)k * nw + wid) * 2] = bf;
            wb[((size_t)k * nw + wid) * 2 + 1] = bc;
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        VI rf{-INFINITY, 0x7fffffff}, rc{-INFINITY, 0x7fffffff};
        for (int v = 0; v < nw; ++v) {
            rf = vi_best(rf, wb[((size_t)k * nw + v) * 2]);
            rc = vi_best(rc, wb[((size_t)k * nw + v) * 2 + 1]);
        }
        const float sF = rf.i == 0x7fffffff ? -INFINITY : rf.v;
        const float sC = rc.i == 0x7fffffff ? -INFINITY : rc.v;
        const int iF = rf.i == 0x7fffffff ? -1 : rf.i + 1;
        const int iC = rc.i == 0x7fffffff ? -1 : rc.i + 1;
        const bool fwd = sF >= sC;
        const float sv = fwd ? sF : sC;
        const bool keepk = sv > thresh[k];
        const size_t o = k + (size_t)K * n;
        if (pos) pos[o] = keepk ? (fwd ? iF : iC) : 0;
        if (score) score[o] = keepk ? sv : 0.f;
        if (comp) comp[o] = (keepk && !fwd) ? 1 : 0;
    }
}

// the sparse scans apply: exact 0/1 data, finite PWM entries (within each motif's
// length), not turned off by CDLGB_SCAN_DENSE
bool sparse_ok(const cdlgb_ctx* c, const float* pwms, const int32_t* lens, int K, int maxlen) {
    if (!c->onehot_exact) return false;
    if (const char* e = getenv("CDLGB_SCAN_DENSE"))
        if (atoi(e) != 0) return false;
    for (int k = 0; k < K; ++k)
        for (int kk = 0; kk < lens[k]; ++kk)
            for (int a = 0; a < 4; ++a)
                if (!isfinite(pwms[k + (size_t)K * (a + 4 * kk)])) return false;
    return true;
}

// integer count matrices: grid (K, chunks); counts (4, maxlen, K) col-major
__global__ void k_count(const float* __restrict__ data, const int32_t* __restrict__ pos,
                        const uint8_t* __restrict__ comp, const int32_t* __restrict__ lens, int K,
                        int maxlen, int L, int N, int32_t* __restrict__ counts,
                        int32_t* __restrict__ nseq) {
    extern __shared__ int cnt[];       // 4*maxlen + 1
    const int k = blockIdx.x;
    const int w = lens[k];
    for (int i = threadIdx.x; i < 4 * maxlen + 1; i += blockDim.x) cnt[i] = 0;
    __syncthreads();
    int per = (N + gridDim.y - 1) / gridDim.y;
    int n0 = blockIdx.y * per, n1 = min(N, n0 + per);
    for (int n = n0 + threadIdx.x; n < n1; n += blockDim.x) {
        int p = pos[k + (size_t)K * n];
        if (p <= 0) continue;
        bool rc = comp && comp[k + (size_t)K * n];
        const float* x = data + (size_t)n * 4 * L + (size_t)(p - 1) * 4;
        for (int i = 0; i < w; ++i)
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                int v = (int)(rc ? x[(w - 1 - i) * 4 + (3 - a)] : x[i * 4 + a]);
                if (v) atomicAdd(&cnt[a + 4 * i], v);
            }
        atomicAdd(&cnt[4 * maxlen], 1);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 4 * maxlen; i += blockDim.x)
        if (cnt[i]) atomicAdd(&counts[i + (size_t)4 * maxlen * k], cnt[i]);
    if (threadIdx.x == 0 && cnt[4 * maxlen]) atomicAdd(&nseq[k], cnt[4 * maxlen]);
}

int check_pwm_args(cdlgb_ctx* c, const float* pwms, const int32_t* lens, const float* thresh,
                   int K, int maxlen) {
    if (!c->loaded) return cdlgb_seterr(c, CDLGB_ESTATE, "no data loaded");
    if (K <= 0 || maxlen <= 0 || !pwms || !lens || !thresh)
        return cdlgb_seterr(c, CDLGB_EINVAL, "scan: bad K=%d / maxlen=%d / null input", K, maxlen);
    for (int k = 0; k < K; ++k)
        if (lens[k] < 1 || lens[k] > maxlen)
            return cdlgb_seterr(c, CDLGB_EINVAL, "scan: lens[%d]=%d outside 1..maxlen=%d", k,
                                lens[k], maxlen);
    return CDLGB_OK;
}

// device scratch layout: [pwms K*4*maxlen f32][thresh K f32] and [lens K i32][pos K*N i32]
int upload_pwms(cdlgb_ctx* c, const float* pwms, const int32_t* lens, const float* thresh, int K,
                int maxlen, size_t extra_i) {
    size_t nf = (size_t)K * 4 * maxlen + K;
    ST_TRY(ensure_scratch(c, &c->scan_f, &c->scan_f_cap, nf + (size_t)K * c->N));
    ST_TRY(ensure_scratch(c, &c->scan_i, &c->scan_i_cap, (size_t)K + extra_i));
    CU_TRY(c, cudaMemcpyAsync(c->scan_f, pwms, (size_t)K * 4 * maxlen * 4, cudaMemcpyHostToDevice,
                              c->stream));
    CU_TRY(c, cudaMemcpyAsync(c->scan_f + (size_t)K * 4 * maxlen, thresh, (size_t)K * 4,
                              cudaMemcpyHostToDevice, c->stream));
    CU_TRY(c, cudaMemcpyAsync(c->scan_i, lens, (size_t)K * 4, cudaMemcpyHostToDevice, c->stream));
    return CDLGB_OK;
}

}  // namespace

int scan_fwd(cdlgb_ctx* c, const float* pwms, const int32_t* lens, const float* thresh, int K,
             int maxlen, int32_t* pos_out) {
    ST_TRY(check_pwm_args(c, pwms, lens, thresh, K, maxlen));
    const int N = c->N, L = c->L4 / 4;
    cdlgb_phase_begin(c, PH_SCAN);
    ST_TRY(upload_pwms(c, pwms, lens, thresh, K, maxlen, (size_t)K * N));
    int32_t* dpos = c->scan_i + K;
    size_t shm = (size_t)4 * L * sizeof(float);
    if (shm > 200 * 1024) return cdlgb_seterr(c, CDLGB_ENOTSUP, "scan: L=%d too long", L);
    // one position per thread with the inputs staged, on exact one-hot data with finite
    // PWMs: the sparse sums (at most 1024 positions and 64 KB of staged inputs)
    const int nts = ((L + 31) / 32) * 32;
    const size_t shs = (size_t)K * 4 * maxlen * sizeof(float) + (size_t)K * (nts / 32) * sizeof(VI) +
                       (size_t)L;
    if (nts <= 1024 && shs <= 64 * 1024 && sparse_ok(c, pwms, lens, K, maxlen)) {
        if (shs > 48 * 1024)
            CU_TRY(c, cudaFuncSetAttribute(k_scan_fwd_sparse, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           64 * 1024));
        k_scan_fwd_sparse<<<N, nts, shs, c->stream>>>(scan_data(c), c->scan_f, c->scan_i,
                                                       c->scan_f + (size_t)K * 4 * maxlen, K, maxlen,
                                                       L, dpos);
        LAUNCH_CHECK(c, "k_scan_fwd_sparse");
    } else {
        if (shm > 48 * 1024)
            CU_TRY(c, cudaFuncSetAttribute(k_scan_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        k_scan_fwd<<<N, kScanThreads, shm, c->stream>>>(scan_data(c), c->scan_f, c->scan_i,
                                                         c->scan_f + (size_t)K * 4 * maxlen, K, maxlen,
                                                         L, dpos);
        LAUNCH_CHECK(c, "k_scan_fwd");
    }
    CU_TRY(c, cudaMemcpyAsync(pos_out, dpos, (size_t)K * N * 4, cudaMemcpyDeviceToHost, c->stream));
    cdlgb_phase_end(c, PH_SCAN);
    CU_TRY(c, cudaStreamSynchronize(c->stream));
    return CDLGB_OK;
}

int scan_both(cdlgb_ctx* c, const float* pwms, const int32_t* lens, const float* thresh, int K,
              int maxlen, int32_t* pos_out, float* score_out, uint8_t* comp_out) {
    ST_TRY(check_pwm_args(c, pwms, lens, thresh, K, maxlen));
    const int N = c->N, L = c->L4 / 4;
    cdlgb_phase_begin(c, PH_SCAN);
    ST_TRY(upload_pwms(c, pwms, lens, thresh, K, maxlen, (size_t)K * N));
    ST_TRY(ensure_scratch(c, &c->scan_u, &c->scan_u_cap, (size_t)K * N));
    int32_t* dpos = c->scan_i + K;
    float* dscore = c->scan_f + (size_t)K * 4 * maxlen + K;
    size_t shm = (size_t)4 * L * sizeof(float);
    if (shm > 200 * 1024) return cdlgb_seterr(c, CDLGB_ENOTSUP, "scan: L=%d too long", L);
    // one position per thread and the staged PWMs when they fit: at most 1024 positions
    // and 64 KB of staged inputs (several blocks per SM)
    const int nts = ((L + 31) / 32) * 32;
    const size_t shs = (size_t)K * 4 * maxlen * sizeof(float2) + (size_t)K * (nts / 32) * 2 * sizeof(VI) +
                       (size_t)4 * L * sizeof(float);
    const size_t shp = (size_t)K * 4 * maxlen * sizeof(float2) + (size_t)K * (nts / 32) * 2 * sizeof(VI) +
                       (size_t)4 * ((L + 31) / 32 + 2) * sizeof(uint32_t);
    const size_t shq = (size_t)K * 64 * sizeof(float2) + (size_t)K * (nts / 32) * 2 * sizeof(VI) +
                       (size_t)4 * ((L + 31) / 32 + 2) * sizeof(uint32_t);
    if (nts <= 1024 && maxlen <= 16 && shq <= 64 * 1024 && sparse_ok(c, pwms, lens, K, maxlen)) {
        if (shq > 48 * 1024)
            CU_TRY(c, cudaFuncSetAttribute(k_scan_both_sparse16, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           64 * 1024));
        k_scan_both_sparse16<<<N, nts, shq, c->stream>>>(scan_data(c), c->scan_f, c->scan_i,
                                                          c->scan_f + (size_t)K * 4 * maxlen, K, maxlen, L,
                                                          dpos, dscore, c->scan_u);
        LAUNCH_CHECK(c, "k_scan_both_sparse16");
    } else if (nts <= 1024 && maxlen <= 64 && shp <= 64 * 1024 && sparse_ok(c, pwms, lens, K, maxlen)) {
        auto kern = maxlen <= 32 ? k_scan_both_sparse<uint32_t> : k_scan_both_sparse<uint64_t>;
        if (shp > 48 * 1024)
            CU_TRY(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024));
        kern<<<N, nts, shp, c->stream>>>(scan_data(c), c->scan_f, c->scan_i,
                                         c->scan_f + (size_t)K * 4 * maxlen, K, maxlen, L,
                                         dpos, dscore, c->scan_u);
        LAUNCH_CHECK(c, "k_scan_both_sparse");
    } else if (nts <= 1024 && shs <= 64 * 1024) {
        if (shs > 48 * 1024)
            CU_TRY(c, cudaFuncSetAttribute(k_scan_both_staged, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           64 * 1024));
        k_scan_both_staged<<<N, nts, shs, c->stream>>>(scan_data(c), c->scan_f, c->scan_i,
                                                        c->scan_f + (size_t)K * 4 * maxlen, K, maxlen, L,
                                                        dpos, dscore, c->scan_u);
        LAUNCH_CHECK(c, "k_scan_both_staged");
    } else {
        if (shm > 48 * 1024)
            CU_TRY(c, cudaFuncSetAttribute(k_scan_both, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        k_scan_both<<<N, kScanThreads, shm, c->stream>>>(scan_data(c), c->scan_f, c->scan_i,
                                                          c->scan_f + (size_t)K * 4 * maxlen, K,
                                                          maxlen, L, dpos, dscore, c->scan_u);
        LAUNCH_CHECK(c, "k_scan_both");
    }
    if (pos_out)
        CU_TRY(c, cudaMemcpyAsync(pos_out, dpos, (size_t)K * N * 4, cudaMemcpyDeviceToHost, c->stream));
    if (score_out)
        CU_TRY(c, cudaMemcpyAsync(score_out, dscore, (size_t)K * N * 4, cudaMemcpyDeviceToHost, c->stream));
    if (comp_out)
        CU_TRY(c, cudaMemcpyAsync(comp_out, c->scan_u, (size_t)K * N, cudaMemcpyDeviceToHost, c->stream));
    cdlgb_phase_end(c, PH_SCAN);
    CU_TRY(c, cudaStreamSynchronize(c->stream));
    return CDLGB_OK;
}

int count_pfms(cdlgb_ctx* c, const int32_t* pos, const uint8_t* use_comp, const int32_t* lens,
               int K, int maxlen, int32_t* counts_out, int32_t* nseq_out) {
    if (!c->loaded) return cdlgb_seterr(c, CDLGB_ESTATE, "no data loaded");
    if (!c->onehot_exact)
        return cdlgb_seterr(c, CDLGB_ENOTSUP, "count_pfms needs 0/1 one-hot data");
    if (K <= 0 || maxlen <= 0 || !pos || !lens || !counts_out)
        return cdlgb_seterr(c, CDLGB_EINVAL, "count_pfms: bad arguments");
    const int N = c->N, L = c->L4 / 4;
    for (int k = 0; k < K; ++k)
        if (lens[k] < 1 || lens[k] > maxlen)
            return cdlgb_seterr(c, CDLGB_EINVAL, "count_pfms: lens[%d]=%d", k, lens[k]);
    if (const long long i = first_bad_position(pos, lens, K, (size_t)N, L); i >= 0) {
        const int k = (int)(i % K), n = (int)(i / K);
        return cdlgb_seterr(c, CDLGB_EINVAL,
                            "count_pfms: window at pos[%d,%d]=%d (len %d) leaves the sequence (L=%d)",
                            k, n, pos[i], lens[k], L);
    }
    size_t ncnt = (size_t)4 * maxlen * K;
    ST_TRY(ensure_scratch(c, &c->scan_i, &c->scan_i_cap, (size_t)K + (size_t)K * N + ncnt + K));
    ST_TRY(ensure_scratch(c, &c->scan_u, &c->scan_u_cap, (size_t)K * N));
    int32_t* dlens = c->scan_i;
    int32_t* dpos = c->scan_i + K;
    int32_t* dcnt = dpos + (size_t)K * N;
    int32_t* dnseq = dcnt + ncnt;
    CU_TRY(c, cudaMemcpyAsync(dlens, lens, (size_t)K * 4, cudaMemcpyHostToDevice, c->stream));
    CU_TRY(c, cudaMemcpyAsync(dpos, pos, (size_t)K * N * 4, cudaMemcpyHostToDevice, c->stream));
    if (use_comp)
        CU_TRY(c, cudaMemcpyAsync(c->scan_u, use_comp, (size_t)K * N, cudaMemcpyHostToDevice, c->stream));
    CU_TRY(c, cudaMemsetAsync(dcnt, 0, (ncnt + K) * 4, c->stream));
    int chunks = (N + 1023) / 1024;
    if (chunks > 64) chunks = 64;
    size_t shm = (size_t)(4 * maxlen + 1) * 4;
    k_count<<<dim3(K, chunks), 256, shm, c->stream>>>(scan_data(c), dpos, use_comp ? c->scan_u : nullptr,
                                                      dlens, K, maxlen, L, N, dcnt, dnseq);
    LAUNCH_CHECK(c, "k_count");
    CU_TRY(c, cudaMemcpyAsync(counts_out, dcnt, ncnt * 4, cudaMemcpyDeviceToHost, c->stream));
    if (nseq_out)
        CU_TRY(c, cudaMemcpyAsync(nseq_out, dnseq, (size_t)K * 4, cudaMemcpyDeviceToHost, c->stream));
    CU_TRY(c, cudaStreamSynchronize(c->stream));
    return CDLGB_OK;
}

namespace {
// non_overlap_scan! (scan.jl:123-174): one thread per sequence n over its K entries
// (k fastest).  sc is a scratch copy of the scores (taken entries are zeroed, as the
// reference zeroes scores_n), keep a scratch of flags; the intersection test walks the
// kept entries in the order they were taken.
__global__ void k_nonoverlap(int32_t* __restrict__ pos, float* __restrict__ score,
                             uint8_t* __restrict__ comp, const int32_t* __restrict__ lens,
                             int K, int N, float* __restrict__ sc, int32_t* __restrict__ order) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    int32_t* P = pos + (size_t)n * K;
    float* Sc = sc + (size_t)n * K;
    int32_t* ord = order + (size_t)n * K;         // kept entries in the order taken
    for (int k = 0; k < K; ++k) Sc[k] = P[k] != 0 ? score[(size_t)n * K + k] : 0.f;
    int nkept = 0;
    for (int iter = 0; iter < K; ++iter) {
        int best = 0;
        float bv = Sc[0];
        for (int k = 1; k < K; ++k)
            if (Sc[k] > bv) { bv = Sc[k]; best = k; }  // first maximum
        if (bv == 0.f) break;
        const int pm = P[best], pme = pm + lens[best] - 1;
        bool hit = false;
        for (int j = 0; j < nkept; ++j) {
            const int q = ord[j], p = P[q], pe = p + lens[q] - 1;
            if ((p <= pm && pm <= pe) || (p <= pme && pme <= pe) || (pm <= p && p <= pme) ||
                (pm <= pe && pe <= pme))
                hit = true;
        }
        if (!hit) ord[nkept++] = best;
        Sc[best] = 0.f;
    }
    // delete what was not kept: mark kept entries in sc (1), the rest (0)
    for (int k = 0; k < K; ++k) Sc[k] = 0.f;
    for (int j = 0; j < nkept; ++j) Sc[ord[j]] = 1.f;
    for (int k = 0; k < K; ++k)
        if (Sc[k] == 0.f && P[k] != 0) {
            P[k] = 0;
            score[(size_t)n * K + k] = 0.f;
            if (comp) comp[(size_t)n * K + k] = 0;
        }
}
}  // namespace

int nonoverlap_select(cdlgb_ctx* c, int32_t* pos, float* score, uint8_t* use_comp,
                      const int32_t* lens, int K) {
    if (!c->loaded) return cdlgb_seterr(c, CDLGB_ESTATE, "no data loaded");
    if (K <= 0 || !pos || !score || !lens)
        return cdlgb_seterr(c, CDLGB_EINVAL, "select_nonoverlapping: bad arguments");
    for (int k = 0; k < K; ++k)
        if (lens[k] < 1) return cdlgb_seterr(c, CDLGB_EINVAL, "select_nonoverlapping: lens[%d]=%d", k, lens[k]);
    const int N = c->N;
    const size_t KN = (size_t)K * N;
    ST_TRY(ensure_scratch(c, &c->scan_i, &c->scan_i_cap, (size_t)K + 2 * KN));
    ST_TRY(ensure_scratch(c, &c->scan_f, &c->scan_f_cap, 2 * KN));
    ST_TRY(ensure_scratch(c, &c->scan_u, &c->scan_u_cap, KN));
    int32_t* dlens = c->scan_i;
    int32_t* dpos = c->scan_i + K;
    int32_t* dord = dpos + KN;
    float* dscore = c->scan_f;
    float* dsc = c->scan_f + KN;
    CU_TRY(c, cudaMemcpyAsync(dlens, lens, (size_t)K * 4, cudaMemcpyHostToDevice, c->stream));
    CU_TRY(c, cudaMemcpyAsync(dpos, pos, KN * 4, cudaMemcpyHostToDevice, c->stream));
    CU_TRY(c, cudaMemcpyAsync(dscore, score, KN * 4, cudaMemcpyHostToDevice, c->stream));
    if (use_comp) CU_TRY(c, cudaMemcpyAsync(c->scan_u, use_comp, KN, cudaMemcpyHostToDevice, c->stream));
    cdlgb_phase_begin(c, PH_SCAN);
    k_nonoverlap<<<(N + 127) / 128, 128, 0, c->stream>>>(dpos, dscore, use_comp ? c->scan_u : nullptr,
                                                         dlens, K, N, dsc, dord);
    LAUNCH_CHECK(c, "k_nonoverlap");
    cdlgb_phase_end(c, PH_SCAN);
    CU_TRY(c, cudaMemcpyAsync(pos, dpos, KN * 4, cudaMemcpyDeviceToHost, c->stream));
    CU_TRY(c, cudaMemcpyAsync(score, dscore, KN * 4, cudaMemcpyDeviceToHost, c->stream));
    if (use_comp) CU_TRY(c, cudaMemcpyAsync(use_comp, c->scan_u, KN, cudaMemcpyDeviceToHost, c->stream));
    CU_TRY(c, cudaStreamSynchronize(c->stream));
    return CDLGB_OK;
}

namespace {
// pvalue2score (src/SEARCH/PWM_Touzet.jl:199-217) with the reference's granularity
// eps = 0.1 (a Float64) and flat background: the rounded entries floor(x / eps) eps are
// exact multiples k eps, every score reached is K eps for an integer K, and every
// probability is count / 4^m, so the reference's Double64 distribution Q[m]
// (score_distribution, :79-102) is the integer count table below, exactly.  One CTA per
// PWM: dense DP over K in shared memory, then find_largest_alpha (:130-142) over the
// reached keys in ascending order.
constexpr int kTouzetMaxR = 6144;     // score range per PWM (two uint64 tables in smem)

__global__ void k_touzet(const int32_t* __restrict__ kq, const int32_t* __restrict__ lens,
                         const int32_t* __restrict__ kmin, const int32_t* __restrict__ range,
                         int maxlen, const unsigned long long* __restrict__ thr_count,
                         int32_t* __restrict__ alpha_k, int32_t* __restrict__ status) {
    extern __shared__ unsigned long long tab[];
    const int p = blockIdx.x;
    const int m = lens[p], R = range[p];
    unsigned long long* Q0 = tab;
    unsigned long long* Q1 = tab + kTouzetMaxR;
    const int32_t* kp = kq + (size_t)p * 4 * maxlen;       // k[j][i] at j * maxlen + i
    for (int s = threadIdx.x; s < R; s += blockDim.x) Q0[s] = 0ull;
    __syncthreads();
    if (threadIdx.x == 0) Q0[0] = 1ull;
    __syncthreads();
    int lo = 0;      // sum of the column minima so far
    int width = 1;   // reached keys lie in [lo, lo + width)
    for (int i = 0; i < m; ++i) {
        int cmin = kp[i], cmax = kp[i];
        for (int j = 1; j < 4; ++j) {
            cmin = min(cmin, kp[j * maxlen + i]);
            cmax = max(cmax, kp[j * maxlen + i]);
        }
        const int nw = width + (cmax - cmin);
        for (int s = threadIdx.x; s < nw; s += blockDim.x) {
            unsigned long long acc = 0ull;
            for (int j = 0; j < 4; ++j) {
                const int src = s - (kp[j * maxlen + i] - cmin);
                if (src >= 0 && src < width) acc += Q0[src];
            }
            Q1[s] = acc;
        }
        __syncthreads();
        for (int s = threadIdx.x; s < nw; s += blockDim.x) Q0[s] = Q1[s];
        __syncthreads();
        lo += cmin;
        width = nw;
    }
    if (threadIdx.x == 0) {
        if (lo != kmin[p] || width != R) {
            status[p] = 1;
            return;
        }
        // find_largest_alpha: q_sum starts at the total (4^m counts), keys ascending;
        // q_sum >= pval  <=>  tail >= ceil(pval 4^m)  (integers, exact)
        unsigned long long tail = 0ull;
        for (int s = 0; s < width; ++s) tail += Q0[s];
        int best = -1;
        for (int s = 0; s < width; ++s) {
            const unsigned long long v = Q0[s];
            if (v == 0ull) continue;                       // keys never reached are absent
            best = s;
            if (tail < thr_count[p]) break;
            tail -= v;
        }
        alpha_k[p] = lo + best;
        status[p] = 0;
    }
}
}  // namespace

int touzet_thresholds(cdlgb_ctx* c, const float* pwms, const int32_t* lens, int K, int maxlen,
                      double pval, float* thresh_out) {
    if (K <= 0 || maxlen <= 0 || !pwms || !lens || !thresh_out)
        return cdlgb_seterr(c, CDLGB_EINVAL, "pvalue_thresholds: bad arguments");
    if (!(pval >= 0.0 && pval <= 1.0)) return cdlgb_seterr(c, CDLGB_EINVAL, "pvalue must be in [0,1]");
    const double eps = 1e-1;                                 // _granularity_
    const size_t nk = (size_t)K * 4 * maxlen;
    std::vector<int32_t> host((size_t)nk + 5 * (size_t)K, 0);
    int32_t* kq = host.data();
    int32_t* kmin = kq + nk;
    int32_t* range = kmin + K;
    int32_t* hl = range + K;
    std::vector<unsigned long long> thr(K);
    for (int p = 0; p < K; ++p) {
        const int m = lens[p];
        if (m < 1 || m > maxlen || m > 31)
            return cdlgb_seterr(c, CDLGB_EINVAL, "pvalue_thresholds: lens[%d]=%d (1..31, <= maxlen)", p, m);
        hl[p] = m;
        long lo = 0, hi = 0;
        for (int i = 0; i < m; ++i) {
            int cmin = 0, cmax = 0;
            for (int j = 0; j < 4; ++j) {
                // pwms (K, 4, maxlen) col-major: element (p, j, i) at p + K (j + 4 i)
                const double x = (double)pwms[p + (size_t)K * (j + 4 * (size_t)i)];
                if (!(fabs(x) < 1e6))
                    return cdlgb_seterr(c, CDLGB_EINVAL, "pvalue_thresholds: PWM entry %g", x);
                // exact floor(x / eps): the double quotient corrected by exact fma residuals
                double q = floor(x / eps);
                if (fma(q, eps, -x) > 0.0) q -= 1.0;
                else if (fma(q + 1.0, eps, -x) <= 0.0) q += 1.0;
                const int k = (int)q;
                kq[(size_t)p * 4 * maxlen + j * maxlen + i] = k;
                if (j == 0 || k < cmin) cmin = k;
                if (j == 0 || k > cmax) cmax = k;
            }
            lo += cmin;
            hi += cmax;
        }
        if (hi - lo + 1 > kTouzetMaxR)
            return cdlgb_seterr(c, CDLGB_ENOTSUP, "pvalue_thresholds: score range %ld of PWM %d exceeds %d",
                                hi - lo + 1, p, kTouzetMaxR);
        kmin[p] = (int32_t)lo;
        range[p] = (int32_t)(hi - lo + 1);
        thr[p] = (unsigned long long)ceil(ldexp(pval, 2 * m));   // pval 4^m is exact; <= 2^62
    }
    ST_TRY(ensure_scratch(c, &c->scan_i, &c->scan_i_cap, nk + 5 * (size_t)K));
    int32_t* d_kq = c->scan_i;
    int32_t* d_lens = d_kq + nk + 2 * (size_t)K;
    int32_t* d_alpha = d_lens + K;
    int32_t* d_status = d_alpha + K;
    unsigned long long* d_thr = nullptr;
    CU_TRY(c, cudaMallocAsync((void**)&d_thr, (size_t)K * sizeof(unsigned long long), c->stream));
    CU_TRY(c, cudaMemcpyAsync(d_kq, host.data(), (nk + 3 * (size_t)K) * 4, cudaMemcpyHostToDevice, c->stream));
    CU_TRY(c, cudaMemcpyAsync(d_thr, thr.data(), (size_t)K * sizeof(unsigned long long), cudaMemcpyHostToDevice,
                              c->stream));
    const int shm = (int)(2 * (size_t)kTouzetMaxR * sizeof(unsigned long long));
    CU_TRY(c, cudaFuncSetAttribute(k_touzet, cudaFuncAttributeMaxDynamicSharedMemorySize, shm));
    k_touzet<<<K, 256, shm, c->stream>>>(d_kq, d_lens, d_kq + nk, d_kq + nk + K, maxlen, d_thr, d_alpha,
                                         d_status);
    cudaError_t e = cudaGetLastError();
    cudaFreeAsync(d_thr, c->stream);
    if (e != cudaSuccess) return cdlgb_seterr(c, CDLGB_ECUDA, "k_touzet: %s", cudaGetErrorString(e));
    std::vector<int32_t> out(2 * (size_t)K);
    CU_TRY(c, cudaMemcpyAsync(out.data(), d_alpha, 2 * (size_t)K * 4, cudaMemcpyDeviceToHost, c->stream));
    CU_TRY(c, cudaStreamSynchronize(c->stream));
    for (int p = 0; p < K; ++p) {
        if (out[K + p] != 0) return cdlgb_seterr(c, CDLGB_ECUDA, "pvalue_thresholds: table mismatch for PWM %d", p);
        // the Double64 key K eps is exact; its high part rounded to float32 (get_thresh's
        // type_real conversion)
        thresh_out[p] = (float)((double)out[p] * eps);
    }
    return CDLGB_OK;
}

void scan_free(cdlgb_ctx* c) {
    dev_free(c, c->scan_i);
    dev_free(c, c->scan_f);
    dev_free(c, c->scan_u);
    c->scan_i = nullptr; c->scan_f = nullptr; c->scan_u = nullptr;
    c->scan_i_cap = c->scan_f_cap = c->scan_u_cap = 0;
}
