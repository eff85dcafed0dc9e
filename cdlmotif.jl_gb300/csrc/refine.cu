// Motif refinement on the device: the column-by-column motif extension of extend!
// (src/SEARCH/extend.jl:1-173) and the score re-evaluation scores_reevaluation
// (src/SEARCH/helpers.jl:151-172).
//
// extension! for one motif is a short sequential loop (one column on the left, one on
// the right, until the information content of a new column drops to the threshold),
// and every step is a sum of one-hot columns over the motif's sequences.  One CTA runs
// the loop of one motif; its threads sum the integer counts of a column over the
// sequences, thread 0 takes the decision.  A sequence whose new column would leave the
// sequence is dropped when that side's column is accepted (to_exclude!, extend.jl:118),
// so whether sequence n is still counted is a function of the accepted (dec, inc)
// alone: it is out as soon as any accepted column on either side fell outside 1..L.
// Evaluating that interval test replaces the reference's per-sequence `included` flags.
#include "cdlgb_internal.h"

#include <vector>

namespace {

struct ExtArgs {
    const float* S;          // one-hot (N, 4L) == Julia (4L, N)
    int32_t* pos;            // (N, K) == Julia (K, N), 1-based, 0 = no entry; in/out
    const uint8_t* comp;     // (N, K) or null: use_comp
    const int32_t* lens;     // K
    int2* list;              // scratch (K, N): per motif (n, p | rc << 30)
    int32_t* out;            // (K, 4): dec, inc, status, number of entries
    float bg0, bg1, bg2, bg3;
    float ps, perc, ic_thresh;
    int K, N, L;
};

enum { EXT_OK = 0, EXT_ENDLESS = 1, EXT_NOT_ONEHOT = 2 };

// get_ic_col_single (helpers.jl:127-133) in Float32, in the reference's order:
// s += p[i] * log2(p[i] / bg[i]).  log2 is evaluated in double and rounded to float,
// which is a correctly rounded Float32 log2 (the Float32 log2 of the reference's
// language evaluates in Float64 and rounds as well).
__device__ float ic_col(const float p[4], const float bg[4]) {
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float q = __fdiv_rn(p[i], bg[i]);
        const float lg = (float)log2((double)q);
        s = __fadd_rn(s, __fmul_rn(p[i], lg));
    }
    return s;
}

// is sequence (p, rc) still counted after the accepted dec left and inc right columns?
// Non-complemented entries take left columns p - o and right columns p + mlen - 1 + o;
// complemented ones the other way round (extend.jl:101-105).
__device__ __forceinline__ bool included(int p, bool rc, int mlen, int dec, int inc, int L) {
    const int nl = rc ? inc : dec;            // columns taken below p
    const int nh = rc ? dec : inc;            // columns taken above p + mlen - 1
    if (nl > 0 && (p - nl < 1 || p - 1 > L)) return false;
    if (nh > 0 && (p + mlen < 1 || p + mlen - 1 + nh > L)) return false;
    return true;
}

// counts of the next column of one side over the counted sequences; returns (in s_c)
// the four integer counts and sets *s_bad when a complemented column is not a one-hot
// vector (dummy_comp's Dict lookup fails there, helpers.jl:33-41)
__device__ void side_counts(const ExtArgs& A, const int2* lst, int nkeys, int mlen, int dec,
                            int inc, bool right, int* s_c, int* s_bad) {
    const int off = right ? inc + 1 : dec + 1;
    int c0 = 0, c1 = 0, c2 = 0, c3 = 0, bad = 0;
    const size_t L4 = (size_t)4 * A.L;
    for (int i = threadIdx.x; i < nkeys; i += blockDim.x) {
        const int2 e = lst[i];
        const int n = e.x, p = e.y & 0x3fffffff;
        const bool rc = (e.y >> 30) & 1;
        if (!included(p, rc, mlen, dec, inc, A.L)) continue;
        const int col = (right != rc) ? p + mlen - 1 + off : p - off;
        if (col < 1 || col > A.L) continue;
        const float4 v = *reinterpret_cast<const float4*>(A.S + (size_t)n * L4 + (size_t)4 * (col - 1));
        if (rc) {
            const bool onehot = (v.x == 0.f || v.x == 1.f) && (v.y == 0.f || v.y == 1.f) &&
                                (v.z == 0.f || v.z == 1.f) && (v.w == 0.f || v.w == 1.f) &&
                                (v.x + v.y + v.z + v.w == 1.f);
            if (!onehot) { bad = 1; continue; }
            c0 += (int)v.w; c1 += (int)v.z; c2 += (int)v.y; c3 += (int)v.x;
        } else {
            c0 += (int)v.x; c1 += (int)v.y; c2 += (int)v.z; c3 += (int)v.w;
        }
    }
    c0 = __reduce_add_sync(0xffffffffu, c0);
    c1 = __reduce_add_sync(0xffffffffu, c1);
    c2 = __reduce_add_sync(0xffffffffu, c2);
    c3 = __reduce_add_sync(0xffffffffu, c3);
    bad = __reduce_or_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31) == 0) {
        if (c0) atomicAdd(&s_c[0], c0);
        if (c1) atomicAdd(&s_c[1], c1);
        if (c2) atomicAdd(&s_c[2], c2);
        if (c3) atomicAdd(&s_c[3], c3);
        if (bad) atomicOr(s_bad, 1);
    }
}

// explore_sides!'s column (extend.jl:25-26 / 113-114): (counts + ps) / (n + 4 ps) in
// Float32, then its information content against the background
__device__ float column_ic(const int* c, const ExtArgs& A) {
    const float bg[4] = {A.bg0, A.bg1, A.bg2, A.bg3};
    // sum(this_col): ((c0 + c1) + c2) + c3 in Float32 (exact for integer counts < 2^24)
    const float tot = __fadd_rn(__fadd_rn(__fadd_rn((float)c[0], (float)c[1]), (float)c[2]), (float)c[3]);
    const float den = __fadd_rn(tot, __fmul_rn(4.f, A.ps));
    float p[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) p[i] = __fdiv_rn(__fadd_rn((float)c[i], A.ps), den);
    return ic_col(p, bg);
}

// extension! (extend.jl:31-81 without use_comp, 122-173 with it) for motif blockIdx.x
__global__ void __launch_bounds__(512) k_extend(ExtArgs A) {
    __shared__ int s_c[4], s_bad, s_cnt, s_acc;
    const int k = blockIdx.x;
    const int mlen = A.lens[k];
    int2* lst = A.list + (size_t)k * A.N;
    if (threadIdx.x == 0) s_cnt = 0;
    __syncthreads();
    // the motif's entries (the keys of positions[k]); their order does not matter
    for (int n = threadIdx.x; n < A.N; n += blockDim.x) {
        const int p = A.pos[(size_t)n * A.K + k];
        if (p <= 0) continue;
        const int rc = (A.comp && A.comp[(size_t)n * A.K + k]) ? 1 : 0;
        const int slot = atomicAdd(&s_cnt, 1);
        lst[slot] = make_int2(n, p | (rc << 30));
    }
    __syncthreads();
    const int nkeys = s_cnt;
    // usage_lowerbdd = floor(perc_no_less_than * len_pos) in Float32 (extend.jl:38).  The
    // reference compares it with num_included, which explore_sides! decrements only in
    // its own copy, so num_included stays len_pos.
    const int lowb = (int)floorf(__fmul_rn(A.perc, (float)nkeys));
    // A terminating loop takes at most L columns per side (past that no sequence has a
    // column in range); beyond 2L + 4 passes the reference would loop for ever.
    const int max_passes = 2 * A.L + 4;
    int dec = 0, inc = 0, status = EXT_OK;
    bool el = true, er = true;
    for (int pass = 0;; ++pass) {
        if (pass >= max_passes) { status = EXT_ENDLESS; break; }
        for (int side = 0; side < 2; ++side) {
            const bool right = side == 1;
            if (!(right ? er : el)) continue;
            if (threadIdx.x < 4) s_c[threadIdx.x] = 0;
            if (threadIdx.x == 0) s_bad = 0;
            __syncthreads();
            side_counts(A, lst, nkeys, mlen, dec, inc, right, s_c, &s_bad);
            __syncthreads();
            if (threadIdx.x == 0) {
                const float ic = column_ic(s_c, A);
                s_acc = s_bad ? -1 : (ic <= A.ic_thresh ? 0 : 1);   // NaN extends, as in the reference
            }
            __syncthreads();
            const int acc = s_acc;
            __syncthreads();
            if (acc < 0) { status = EXT_NOT_ONEHOT; break; }
            if (acc == 0) {
                if (right) er = false; else el = false;
            } else {
                if (right) ++inc; else ++dec;
            }
        }
        if (status != EXT_OK) break;
        if (!el && !er) break;
        if (nkeys <= lowb) break;
    }
    if (status == EXT_OK && (dec > 0 || inc > 0)) {
        for (int i = threadIdx.x; i < nkeys; i += blockDim.x) {
            const int2 e = lst[i];
            const int p = e.y & 0x3fffffff;
            const bool rc = (e.y >> 30) & 1;
            A.pos[(size_t)e.x * A.K + k] = included(p, rc, mlen, dec, inc, A.L) ? (rc ? p - inc : p - dec) : 0;
        }
    }
    if (threadIdx.x == 0) {
        A.out[4 * k + 0] = dec;
        A.out[4 * k + 1] = inc;
        A.out[4 * k + 2] = status;
        A.out[4 * k + 3] = nkeys;
    }
}

// scores_reevaluation (helpers.jl:151-172): for every entry the sum over the window of
// pwm .* data in Float32, in memory order (base-major, nucleotide inner), one rounded
// product and one rounded sum per term.  The reference reads the forward window even
// for reverse-complemented entries (it ignores use_comp here).  One thread per (k, n);
// grid (ceil(N / 256), K).
__global__ void k_rescore(const float* __restrict__ S, const float* __restrict__ pwms,
                          const int32_t* __restrict__ pos, const int32_t* __restrict__ lens,
                          int K, int maxlen, int N, int L, float* __restrict__ score) {
    const int k = blockIdx.y;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    const int p = pos[(size_t)n * K + k];
    if (p <= 0) { score[(size_t)n * K + k] = 0.f; return; }
    const int w = lens[k];
    const float* x = S + (size_t)n * 4 * L + (size_t)4 * (p - 1);
    float s = 0.f;
    for (int i = 0; i < w; ++i)
#pragma unroll
        for (int a = 0; a < 4; ++a)
            s = __fadd_rn(s, __fmul_rn(pwms[k + (size_t)K * (a + 4 * (size_t)i)], x[4 * i + a]));
    score[(size_t)n * K + k] = s;
}

}  // namespace

int extend_positions(cdlgb_ctx* c, int32_t* pos, const uint8_t* use_comp, int32_t* lens, int K,
                     const float* bg, float pseudocount, float perc_no_less_than,
                     float ic_extension_thresh, int32_t* dec_out, int32_t* inc_out) {
    if (!c->loaded) return cdlgb_seterr(c, CDLGB_ESTATE, "no data loaded");
    if (!c->onehot_exact)
        return cdlgb_seterr(c, CDLGB_ENOTSUP, "extend: needs 0/1 one-hot data");
    if (K <= 0 || !pos || !lens || !bg)
        return cdlgb_seterr(c, CDLGB_EINVAL, "extend: bad arguments");
    const int N = c->N, L = c->L4 / 4;
    if (L >= (1 << 29)) return cdlgb_seterr(c, CDLGB_EINVAL, "extend: L too large");
    for (int k = 0; k < K; ++k)
        if (lens[k] < 1 || lens[k] > L)
            return cdlgb_seterr(c, CDLGB_EINVAL, "extend: lens[%d]=%d outside 1..L=%d", k, lens[k], L);
    const size_t KN = (size_t)K * N;
    if (const long long i = first_bad_position(pos, nullptr, K, (size_t)N, L); i >= 0)
        return cdlgb_seterr(c, CDLGB_EINVAL, "extend: pos[%lld]=%d outside 0..L=%d", i, pos[i], L);
    // device scratch: lens (K) + out (4K) + pos (KN) ints, use_comp (KN) bytes, list (KN) int2
    ST_TRY(ensure_scratch(c, &c->scan_i, &c->scan_i_cap, (size_t)5 * K + KN));
    ST_TRY(ensure_scratch(c, &c->scan_u, &c->scan_u_cap, KN));
    ST_TRY(ensure_scratch(c, &c->scan_f, &c->scan_f_cap, 2 * KN));
    int32_t* dlens = c->scan_i;
    int32_t* dout = c->scan_i + K;
    int32_t* dpos = c->scan_i + 5 * K;
    ExtArgs a;
    a.S = scan_data(c); a.pos = dpos; a.comp = use_comp ? c->scan_u : nullptr; a.lens = dlens;
    a.list = reinterpret_cast<int2*>(c->scan_f); a.out = dout;
    a.bg0 = bg[0]; a.bg1 = bg[1]; a.bg2 = bg[2]; a.bg3 = bg[3];
    a.ps = pseudocount; a.perc = perc_no_less_than; a.ic_thresh = ic_extension_thresh;
    a.K = K; a.N = N; a.L = L;
    CU_TRY(c, cudaMemcpyAsync(dlens, lens, (size_t)K * 4, cudaMemcpyHostToDevice, c->stream));
    CU_TRY(c, cudaMemcpyAsync(dpos, pos, KN * 4, cudaMemcpyHostToDevice, c->stream));
    if (use_comp) CU_TRY(c, cudaMemcpyAsync(c->scan_u, use_comp, KN, cudaMemcpyHostToDevice, c->stream));
    cdlgb_phase_begin(c, PH_SCAN);
    k_extend<<<K, 512, 0, c->stream>>>(a);
    LAUNCH_CHECK(c, "k_extend");
    cdlgb_phase_end(c, PH_SCAN);
    std::vector<int32_t> out((size_t)4 * K);
    CU_TRY(c, cudaMemcpyAsync(out.data(), dout, (size_t)16 * K, cudaMemcpyDeviceToHost, c->stream));
    CU_TRY(c, cudaStreamSynchronize(c->stream));
    for (int k = 0; k < K; ++k) {
        if (out[4 * k + 2] == EXT_ENDLESS)
            return cdlgb_seterr(c, CDLGB_EINVAL,
                                "extend: motif %d keeps extending past both sequence ends (the "
                                "information content of an empty column, %g pseudocounts against the "
                                "background, exceeds the threshold; the reference never returns)",
                                k, (double)pseudocount);
        if (out[4 * k + 2] == EXT_NOT_ONEHOT)
            return cdlgb_seterr(c, CDLGB_EINVAL,
                                "extend: motif %d: a reverse-complemented column is not one-hot "
                                "(the reference's dummy_comp raises KeyError)", k);
    }
    CU_TRY(c, cudaMemcpyAsync(pos, dpos, KN * 4, cudaMemcpyDeviceToHost, c->stream));
    CU_TRY(c, cudaStreamSynchronize(c->stream));
    for (int k = 0; k < K; ++k) {
        lens[k] += out[4 * k] + out[4 * k + 1];
        if (dec_out) dec_out[k] = out[4 * k];
        if (inc_out) inc_out[k] = out[4 * k + 1];
    }
    return CDLGB_OK;
}

int rescore_positions(cdlgb_ctx* c, const float* pwms, const int32_t* pos, const int32_t* lens,
                      int K, int maxlen, float* score_out) {
    if (!c->loaded) return cdlgb_seterr(c, CDLGB_ESTATE, "no data loaded");
    if (K <= 0 || maxlen <= 0 || !pwms || !pos || !lens || !score_out)
        return cdlgb_seterr(c, CDLGB_EINVAL, "rescore: bad arguments");
    const int N = c->N, L = c->L4 / 4;
    const size_t KN = (size_t)K * N;
    for (int k = 0; k < K; ++k)
        if (lens[k] < 1 || lens[k] > maxlen)
            return cdlgb_seterr(c, CDLGB_EINVAL, "rescore: lens[%d]=%d outside 1..maxlen=%d", k, lens[k], maxlen);
    if (const long long i = first_bad_position(pos, lens, K, (size_t)N, L); i >= 0)
        return cdlgb_seterr(c, CDLGB_EINVAL, "rescore: window at pos[%lld]=%d (len %d) leaves the sequence (L=%d)",
                            i, pos[i], lens[i % K], L);
    const size_t npwm = (size_t)K * 4 * maxlen;
    ST_TRY(ensure_scratch(c, &c->scan_i, &c->scan_i_cap, (size_t)K + KN));
    ST_TRY(ensure_scratch(c, &c->scan_f, &c->scan_f_cap, npwm + KN));
    int32_t* dlens = c->scan_i;
    int32_t* dpos = c->scan_i + K;
    float* dpwm = c->scan_f;
    float* dsc = c->scan_f + npwm;
    CU_TRY(c, cudaMemcpyAsync(dlens, lens, (size_t)K * 4, cudaMemcpyHostToDevice, c->stream));
    CU_TRY(c, cudaMemcpyAsync(dpos, pos, KN * 4, cudaMemcpyHostToDevice, c->stream));
    CU_TRY(c, cudaMemcpyAsync(dpwm, pwms, npwm * 4, cudaMemcpyHostToDevice, c->stream));
    cdlgb_phase_begin(c, PH_SCAN);
    k_rescore<<<dim3((unsigned)((N + 255) / 256), (unsigned)K), 256, 0, c->stream>>>(
        scan_data(c), dpwm, dpos, dlens, K, maxlen, N, L, dsc);
    LAUNCH_CHECK(c, "k_rescore");
    cdlgb_phase_end(c, PH_SCAN);
    CU_TRY(c, cudaMemcpyAsync(score_out, dsc, KN * 4, cudaMemcpyDeviceToHost, c->stream));
    CU_TRY(c, cudaStreamSynchronize(c->stream));
    return CDLGB_OK;
}
