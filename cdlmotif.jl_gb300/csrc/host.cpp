// Host-only parts of the C ABI: the posdicts2pfms normalisation and the transfac
// writer.  Both are CPU code in the reference too (src/SEARCH/helpers.jl:59-96,
// src/SAVE/save_learned_results.jl:184-217); they take a few hundred numbers.
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "cdlgb.h"

namespace {

// Shortest decimal digits that read back to the same float32 (the digit string
// Julia's Ryu-based `string(::Float32)` prints), as (digits, exponent) with
// value = 0.d1d2...dk * 10^pt.
struct Dec { std::string digits; int pt; };

bool roundtrips(const std::string& digits, int pt, float x) {
    std::string s = "0." + digits + "e" + std::to_string(pt);
    return strtof(s.c_str(), nullptr) == x;
}

Dec shortest(float x) {
    // x > 0, finite
    for (int prec = 1; prec <= 9; ++prec) {
        char buf[64];
        snprintf(buf, sizeof(buf), "%.*e", prec - 1, (double)x);
        // buf: d.ddddde[+-]XX
        std::string s(buf);
        size_t epos = s.find('e');
        std::string mant = s.substr(0, epos);
        int e10 = atoi(s.c_str() + epos + 1);
        std::string digits;
        for (char ch : mant) if (ch != '.') digits += ch;
        int pt = e10 + 1;
        if (roundtrips(digits, pt, x)) {
            // an equally short neighbour may be closer to x only if printf's choice
            // is the nearest; it is, so keep it
            return {digits, pt};
        }
        // the nearest p-digit decimal is outside the rounding interval; the other
        // neighbour (one unit in the last digit, towards x) may still be inside it
        // (asymmetric intervals at powers of two)
        long long v = atoll(digits.c_str());
        double approx = strtod((("0." + digits + "e" + std::to_string(pt))).c_str(), nullptr);
        long long w = approx < (double)x ? v + 1 : v - 1;
        if (w > 0) {
            std::string wd = std::to_string(w);
            int wpt = pt;
            if ((int)wd.size() > prec) { wd = wd.substr(0, prec); wpt += 1; }
            while ((int)wd.size() < prec) { wd = "0" + wd; }
            if (wd[0] != '0' && roundtrips(wd, wpt, x)) return {wd, wpt};
        }
    }
    char buf[64];
    snprintf(buf, sizeof(buf), "%.8e", (double)x);
    std::string s(buf);
    size_t epos = s.find('e');
    std::string digits;
    for (char ch : s.substr(0, epos)) if (ch != '.') digits += ch;
    return {digits, atoi(s.c_str() + epos + 1) + 1};
}

// Julia's Float32 `string`: positional when -4 < pt <= 6, else d.ddde[-]X
std::string julia_f32(float x) {
    if (isnan(x)) return "NaN";
    if (isinf(x)) return x > 0 ? "Inf" : "-Inf";
    if (x == 0.f) return signbit(x) ? "-0.0" : "0.0";
    std::string sign = x < 0 ? "-" : "";
    Dec d = shortest(fabsf(x));
    while (d.digits.size() > 1 && d.digits.back() == '0') d.digits.pop_back();
    int k = (int)d.digits.size(), pt = d.pt;
    std::string out;
    if (pt > -4 && pt <= 6) {
        if (pt <= 0) out = "0." + std::string(-pt, '0') + d.digits;
        else if (pt < k) out = d.digits.substr(0, pt) + "." + d.digits.substr(pt);
        else out = d.digits + std::string(pt - k, '0') + ".0";
    } else {
        std::string frac = k > 1 ? d.digits.substr(1) : "0";
        out = d.digits.substr(0, 1) + "." + frac + "e" + std::to_string(pt - 1);
    }
    return sign + out;
}

}  // namespace

extern "C" {

int cdlgb_counts_to_pfms(const int32_t* counts, const int32_t* nseq, const int32_t* lens,
                         int32_t K, int32_t maxlen, float pseudocounts_r, float pseudo_count,
                         int32_t smoothing, int32_t less_pseudocount, float* pfm_out) {
    if (!counts || !nseq || !lens || !pfm_out || K <= 0 || maxlen <= 0) return CDLGB_EINVAL;
    for (int k = 0; k < K; ++k) {
        if (lens[k] < 1 || lens[k] > maxlen) return CDLGB_EINVAL;
        volatile float n = (float)nseq[k];
        volatile float ps = smoothing ? pseudocounts_r * n
                                      : (less_pseudocount ? 0.1f : pseudo_count);
        volatile float four_ps = 4.f * ps;
        volatile float den = n + four_ps;
        for (int i = 0; i < maxlen; ++i)
            for (int a = 0; a < 4; ++a) {
                size_t o = (size_t)a + 4 * ((size_t)i + (size_t)maxlen * k);
                if (i >= lens[k]) { pfm_out[o] = 0.f; continue; }
                volatile float num = (float)counts[o] + ps;
                pfm_out[o] = num / den;
            }
    }
    return CDLGB_OK;
}

int64_t cdlgb_transfac_format(const float* pfm, int32_t w, int32_t reverse_complement, char* out,
                              size_t cap) {
    if (!pfm || w <= 0) return CDLGB_EINVAL;
    std::string s = "ID\t\nXX\t\nBF\t\nXX\t\nP0\tA\tC\tG\tT\n";
    for (int j = 0; j < w; ++j) {
        std::string row = (j + 1 < 10) ? "0" + std::to_string(j + 1) : std::to_string(j + 1);
        s += row;
        for (int a = 0; a < 4; ++a) {
            // reverse(pfm) reverses both dims: (a, j) <- (3-a, w-1-j)
            float v = reverse_complement ? pfm[(3 - a) + 4 * (w - 1 - j)] : pfm[a + 4 * j];
            volatile float q = v * 1000.f;
            s += "\t" + julia_f32(q);
        }
        s += "\n";
    }
    s += "XX\t\n";
    if (out && cap > 0) {
        size_t n = s.size() < cap - 1 ? s.size() : cap - 1;
        memcpy(out, s.data(), n);
        out[n] = 0;
    }
    return (int64_t)s.size();
}

namespace {
// median of a Float32 window as the reference's median computes it: NaN if any entry is
// NaN, else the middle of the sorted values, middle(a, b) = a/2 + b/2 for an even count
float median_f32(std::vector<float> v) {
    for (float x : v)
        if (x != x) return x;
    std::sort(v.begin(), v.end());
    const size_t n = v.size();
    if (n & 1) return v[n / 2];
    volatile float a = v[n / 2 - 1] / 2.f;
    volatile float b = v[n / 2] / 2.f;
    return a + b;
}
}  // namespace

int cdlgb_trim_pfms(const float* pfms, const int32_t* lens, int32_t K, int32_t maxlen,
                    const float* bg, const int32_t* mask_len, const float* mask_thresh,
                    int32_t nmask, int32_t* front_out, int32_t* back_out) {
    if (!pfms || !lens || !bg || !front_out || !back_out || K <= 0 || maxlen <= 0 || nmask < 0 ||
        (nmask > 0 && (!mask_len || !mask_thresh)))
        return CDLGB_EINVAL;
    for (int k = 0; k < K; ++k) {
        const int w = lens[k];
        if (w < 0 || w > maxlen) return CDLGB_EINVAL;
        // get_ic_col_multiple (helpers.jl:135-138): per column, in Float32,
        // ((s1 + s2) + s3) + s4 with s_a = p * log2(p / bg[a]) (log2 rounded from double)
        std::vector<float> ic((size_t)w);
        for (int j = 0; j < w; ++j) {
            volatile float acc = 0.f;
            for (int a = 0; a < 4; ++a) {
                volatile float p = pfms[(size_t)a + 4 * ((size_t)j + (size_t)maxlen * k)];
                volatile float q = p / bg[a];
                volatile float lg = (float)log2((double)q);
                volatile float t = p * lg;
                acc = acc + t;
            }
            ic[j] = acc;
        }
        // trim_this_pfm_by_masking! (trim.jl:1-36): for each mask, mark window starts
        // from the front while the window's median IC is below the mask threshold, and
        // window ends from the back likewise; already marked columns are skipped.
        std::vector<char> trim((size_t)w, 0);
        for (int m = 0; m < nmask; ++m) {
            const int ml = mask_len[m];
            const float mt = mask_thresh[m];
            if (ml < 1) return CDLGB_EINVAL;
            for (int i = 0; i + ml <= w; ++i) {
                if (trim[i]) continue;
                if (median_f32(std::vector<float>(ic.begin() + i, ic.begin() + i + ml)) < mt)
                    trim[i] = 1;
                else
                    break;
            }
            for (int j = w - 1; j >= ml - 1; --j) {
                if (trim[j]) continue;
                if (median_f32(std::vector<float>(ic.begin() + (j - ml + 1), ic.begin() + j + 1)) < mt)
                    trim[j] = 1;
                else
                    break;
            }
        }
        int front = 0, back = 0;
        for (int j = 0; j < w && trim[j]; ++j) ++front;
        for (int j = w - 1; j >= 0 && trim[j]; --j) ++back;
        front_out[k] = front;
        back_out[k] = back;
    }
    return CDLGB_OK;
}

int cdlgb_fisher_evalues(const int32_t* hits, const int32_t* hits_bg, int32_t K, int32_t N,
                         double* evalues_out) {
    if (!hits || !hits_bg || !evalues_out || K <= 0 || N < 0) return CDLGB_EINVAL;
    for (int i = 0; i < K; ++i) {
        const long a = hits[i], b = hits_bg[i];
        if (a < 0 || a > N || b < 0 || b > N) return CDLGB_EINVAL;
        // table [a N; b N]: X ~ Hypergeometric(r1 = a + N successes, r2 = b + N failures,
        // c1 = a + b draws), observed a; P(X = j) = C(r1, j) C(r2, c1 - j) / C(r1 + r2, c1)
        const double r1 = (double)(a + N), r2 = (double)(b + N), c1 = (double)(a + b);
        const long lo = (long)std::max(0.0, c1 - r2), hi = (long)std::min(c1, r1);
        auto lp = [&](long j) {
            return -lgamma((double)j + 1.0) - lgamma(r1 - (double)j + 1.0) -
                   lgamma(c1 - (double)j + 1.0) - lgamma(r2 - c1 + (double)j + 1.0);
        };
        double mx = -INFINITY;
        for (long j = lo; j <= hi; ++j) mx = std::max(mx, lp(j));
        double left = 0.0, right = 0.0, total = 0.0;
        for (long j = lo; j <= hi; ++j) {
            const double t = exp(lp(j) - mx);
            total += t;
            if (j <= a) left += t;
            if (j >= a) right += t;
        }
        double p = 2.0 * std::min(left, right) / total;
        if (p > 1.0) p = 1.0;
        evalues_out[i] = p * (double)K;
    }
    return CDLGB_OK;
}

}  // extern "C"
