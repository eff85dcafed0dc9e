// Code -> activations -> filter-pair topology -> pair count matrices
// (src/SEARCH/store.jl:1-144, src/SEARCH/extractions.jl:18-190), device resident.
//
// The activation record keeps, for each training t, the codes
//   codes[t][n][m][c] = X_best[gamma + 4c, m, n]   (store.jl:15, c = 0..L-1)
// and its threshold; a filter k of the record is (t, m) for every m of training t with
// at least one activation (the reference's uinds, store.jl:22).  Activations are
// codes > thresh[t] (store.jl:17), evaluated on the fly.
//
// topology_at_nth_pt! (store.jl:64-107) launches a thread per (r, c, n) over
// (C*K)^2 * N; here one CTA per sequence compacts its active (k, position) entries
// and loops over pairs of them only, with the reference's conditions and integer
// atomics (counts are exact and order-independent).
#include "cdlgb_internal.h"

#include <algorithm>
#include <new>
#include <string>
#include <vector>

struct cdlgb_ar {
    int dev = 0;
    cudaStream_t stream = nullptr;
    char err[512];
    int N = 0, C = 0, M = 0, T = 0;
    std::vector<int> uinds, training_num, filter_lengths;   // per registered filter (1-based)
    std::vector<float> thresh;                               // per training
    std::vector<int> recorded;                               // training recorded?
    float* codes = nullptr;                                  // (T, N, M, C)
    int* anym = nullptr;                                     // (M) scratch
    int* kmap = nullptr;                                     // (Kcap) t*M + m
    int* klen = nullptr;                                     // (Kcap) filter length (bases)
    int* ktrain = nullptr;                                   // (Kcap) training number
    float* dthresh = nullptr;                                // (T)
    int* list = nullptr;                                     // per-CTA compaction space
    int list_ctas = 0;
    int* dcount = nullptr;                                   // topology outputs (device)
    size_t dcount_cap = 0;
    float* msa = nullptr;                                    // pair MSA partials
    size_t msa_cap = 0;
};

namespace {

int ar_err(cdlgb_ar* a, int code, const char* fmt, ...) {
    if (a) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(a->err, sizeof(a->err), fmt, ap);
        va_end(ap);
    }
    return code;
}

#define AR_CU(a, call)                                                                   \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess)                                                           \
            return ar_err((a), CDLGB_ECUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

// codes[t] <- X_best rows gamma, gamma+4, ...; anym[m] |= any(code > thresh)
__global__ void k_record(const float* __restrict__ Xb, float* __restrict__ codes, int N, int M,
                         int C, int Lg, int gamma, float thresh, int* __restrict__ anym) {
    const size_t total = (size_t)N * M * C;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
         i += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const size_t nm = i / C;                 // n * M + m
        const int m = (int)(nm % M);
        const float v = Xb[nm * Lg + gamma + 4 * (size_t)c];
        codes[i] = v;
        if (v > thresh && !anym[m]) atomicOr(&anym[m], 1);
    }
}

// One CTA per sequence (persistent over sequences): compact the active (k, pos)
// entries, then count every ordered pair as topology_at_nth_pt! does.
// over (K, K, maxlen), non_over (K, K, CmFm1), next_to (K, K), all col-major int32.
__global__ void k_topology(const float* __restrict__ codes, const int* __restrict__ kmap,
                           const int* __restrict__ klen, const int* __restrict__ ktrain,
                           const float* __restrict__ thresh, int N, int M, int C, int K,
                           int maxlen, int CmFm1, int* __restrict__ list, int* __restrict__ over,
                           int* __restrict__ non_over, int* __restrict__ next_to) {
    __shared__ int cnt;
    int* my = list + (size_t)blockIdx.x * K * C;
    for (int n = blockIdx.x; n < N; n += gridDim.x) {
        if (threadIdx.x == 0) cnt = 0;
        __syncthreads();
        for (int e = threadIdx.x; e < K * C; e += blockDim.x) {
            const int k = e / C, p = e - k * C;
            const int tm = kmap[k];
            const int t = tm / M, m = tm - t * M;
            const float v = codes[(((size_t)t * N + n) * M + m) * C + p];
            if (v > thresh[t]) {
                const int slot = atomicAdd(&cnt, 1);
                my[slot] = (k << 16) | p;
            }
        }
        __syncthreads();
        const int ne = cnt;
        const long long np = (long long)ne * ne;
        for (long long q = threadIdx.x; q < np; q += blockDim.x) {
            const int a = my[q / ne], b = my[q % ne];
            const int fr = a >> 16, pr = (a & 0xffff) + 1;     // 1-based start positions
            const int fc = b >> 16, pc = (b & 0xffff) + 1;
            if (fr == fc || pr > pc || ktrain[fr] == ktrain[fc]) continue;
            const int lr = klen[fr];
            if (lr == klen[fc] && pr == pc) continue;           // exact matches excluded
            const int dist = pc - (pr + lr - 1) - 1;
            if (dist < 0) {
                atomicAdd(&over[fr + (size_t)K * (fc + (size_t)K * (-dist - 1))], 1);
            } else if (dist > 0 && dist <= CmFm1) {
                atomicAdd(&non_over[fr + (size_t)K * (fc + (size_t)K * (dist - 1))], 1);
            } else {
                atomicAdd(&next_to[fr + (size_t)K * fc], 1);
            }
        }
        __syncthreads();
    }
}

// Pair MSAs (get_f_pair_starts + msa_fill, extractions.jl:116-181): grid (P, chunks);
// each block accumulates its sequences' code-weighted one-hot windows for pair p in
// shared memory and writes one partial per chunk (summed in order afterwards).
__global__ void k_pair_msa(const float* __restrict__ codes, const float* __restrict__ S,
                           const int* __restrict__ pairs, const int* __restrict__ kmap,
                           const int* __restrict__ klen, const float* __restrict__ thresh,
                           int N, int M, int C, int max_span, float* __restrict__ part) {
    extern __shared__ float acc[];                            // 4 * max_span
    const int p = blockIdx.x, ch = blockIdx.y, nch = gridDim.y;
    const int fr = pairs[3 * p] - 1, fc = pairs[3 * p + 1] - 1, o_len = pairs[3 * p + 2];
    const int fl1 = klen[fr], fl2 = klen[fc];
    const int span = o_len >= fl2 ? o_len : fl1 - o_len + fl2;   // get_span_len
    const int t1 = kmap[fr] / M, f1 = kmap[fr] % M;
    const int t2 = kmap[fc] / M, f2 = kmap[fc] % M;
    const float th1 = thresh[t1], th2 = thresh[t2];
    for (int i = threadIdx.x; i < 4 * max_span; i += blockDim.x) acc[i] = 0.f;
    __syncthreads();
    const int n0 = (int)((long long)N * ch / nch), n1 = (int)((long long)N * (ch + 1) / nch);
    const int nl = 4 * span;
    for (int n = n0; n < n1; ++n) {
        const float* c1 = codes + (((size_t)t1 * N + n) * M + f1) * C;
        const float* c2 = codes + (((size_t)t2 * N + n) * M + f2) * C;
        const float* x = S + (size_t)n * 4 * C;
        // s: 1-based start of filter fr; fc starts at s + fl1 - o_len
        for (int s = 1; s <= C - span + 1; ++s) {
            const int s2 = s + fl1 - o_len;
            if (s2 < 1 || s2 > C) continue;
            const float a = c1[s - 1], b = c2[s2 - 1];
            if (!(a > th1) || !(b > th2)) continue;
            const float avg = (a + b) / 2;
            for (int l = threadIdx.x; l < nl; l += blockDim.x)
                acc[l] += avg * x[(s - 1) * 4 + l];
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 4 * max_span; i += blockDim.x)
        part[((size_t)p * nch + ch) * 4 * max_span + i] = acc[i];
}

// sum the chunk partials in order, + 0.1 inside the span (msa_pseudocount), normalise
// by the first column's total; pfms (P, 4, max_span) col-major
__global__ void k_pair_finish(const float* __restrict__ part, const int* __restrict__ pairs,
                              const int* __restrict__ klen, int P, int nch, int max_span,
                              float* __restrict__ pfm, int* __restrict__ spans) {
    extern __shared__ double col[];                           // 4 * max_span
    const int p = blockIdx.x;
    const int fr = pairs[3 * p] - 1, fc = pairs[3 * p + 1] - 1, o_len = pairs[3 * p + 2];
    const int fl1 = klen[fr], fl2 = klen[fc];
    const int span = o_len >= fl2 ? o_len : fl1 - o_len + fl2;
    for (int i = threadIdx.x; i < 4 * max_span; i += blockDim.x) {
        double s = 0.0;
        for (int ch = 0; ch < nch; ++ch) s += part[((size_t)p * nch + ch) * 4 * max_span + i];
        float v = (float)s;
        if (i < 4 * span) v += 0.1f;
        col[i] = v;
    }
    __syncthreads();
    const double tot = col[0] + col[1] + col[2] + col[3];
    for (int i = threadIdx.x; i < 4 * max_span; i += blockDim.x) {
        const int a = i % 4, j = i / 4;
        pfm[p + (size_t)P * (a + 4 * (size_t)j)] = (float)(col[i] / tot);
    }
    if (threadIdx.x == 0) spans[p] = span;
}

}  // namespace

extern "C" {

int cdlgb_ar_create(int32_t N, int32_t L, int32_t M, int32_t T, int32_t device, cdlgb_ar** out) {
    if (!out || N <= 0 || L <= 0 || M <= 0 || T <= 0 || L > 65535)
        return noctx_seterr(CDLGB_EINVAL, "cdlgb_ar_create: N=%d, L=%d, M=%d, T=%d (L <= 65535)",
                            N, L, M, T);
    *out = nullptr;
    cdlgb_ar* a = new (std::nothrow) cdlgb_ar();
    if (!a) return noctx_seterr(CDLGB_EINVAL, "cdlgb_ar_create: out of host memory");
    a->err[0] = 0;
    a->dev = device;
    a->N = N; a->C = L; a->M = M; a->T = T;
    a->thresh.assign(T, 0.f);
    a->recorded.assign(T, 0);
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking);
    size_t kcap = (size_t)T * M;
    if (e == cudaSuccess) e = cudaMalloc((void**)&a->codes, (size_t)T * N * M * L * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void**)&a->anym, M * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc((void**)&a->kmap, kcap * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc((void**)&a->klen, kcap * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc((void**)&a->ktrain, kcap * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc((void**)&a->dthresh, T * sizeof(float));
    if (e != cudaSuccess) {
        noctx_seterr(CDLGB_ECUDA, "cdlgb_ar_create: %s", cudaGetErrorString(e));
        cdlgb_ar_destroy(a);
        return CDLGB_ECUDA;
    }
    *out = a;
    return CDLGB_OK;
}

int cdlgb_ar_destroy(cdlgb_ar* a) {
    if (!a) return CDLGB_OK;
    cudaSetDevice(a->dev);
    if (a->stream) cudaStreamSynchronize(a->stream);
    void* ptrs[] = {a->codes, a->anym, a->kmap, a->klen, a->ktrain, a->dthresh, a->list,
                    a->dcount, a->msa};
    for (void* p : ptrs) if (p) cudaFree(p);
    if (a->stream) cudaStreamDestroy(a->stream);
    delete a;
    return CDLGB_OK;
}

const char* cdlgb_ar_last_error(const cdlgb_ar* a) {
    if (a) return a->err;
    const char* m = noctx_err();
    return m ? m : "null record";
}

int cdlgb_ar_record(cdlgb_ar* a, cdlgb_ctx* c, double thresh, int32_t train_num,
                    int32_t filter_size, int32_t* added) {
    if (!a || !c) return CDLGB_EINVAL;
    // store.jl:8
    if (!(thresh > 0)) return ar_err(a, CDLGB_EINVAL, "threshold must be greater than 0");
    if (train_num < 1 || train_num > a->T || a->recorded[train_num - 1])
        return ar_err(a, CDLGB_EINVAL, "train_num %d outside 1..%d or already recorded", train_num, a->T);
    if (!c->initialized || c->N != a->N || c->L4 != 4 * a->C || c->M != a->M)
        return ar_err(a, CDLGB_EINVAL, "context does not hold an initialised N=%d, L=%d, M=%d problem",
                      a->N, a->C, a->M);
    if (filter_size < 1 || filter_size > a->C) return ar_err(a, CDLGB_EINVAL, "bad filter_size");
    AR_CU(a, cudaSetDevice(a->dev));
    AR_CU(a, cudaStreamSynchronize(c->stream));     // X_best is final
    const int t = train_num - 1;
    const float th = (float)thresh;                 // activations compare Float32 codes
    const float* Xb = c->best_is_cur ? c->Xb[c->xcur] : c->Xb[1 - c->xcur];
    AR_CU(a, cudaMemsetAsync(a->anym, 0, a->M * sizeof(int), a->stream));
    size_t total = (size_t)a->N * a->M * a->C;
    k_record<<<grid_for(total, 256), 256, 0, a->stream>>>(
        Xb, a->codes + (size_t)t * a->N * a->M * a->C, a->N, a->M, a->C, c->Lg, c->gamma, th, a->anym);
    AR_CU(a, cudaGetLastError());
    std::vector<int> any(a->M);
    AR_CU(a, cudaMemcpyAsync(any.data(), a->anym, a->M * sizeof(int), cudaMemcpyDeviceToHost, a->stream));
    AR_CU(a, cudaStreamSynchronize(a->stream));
    int cnt = 0;
    for (int m = 0; m < a->M; ++m)
        if (any[m]) {
            a->uinds.push_back(m + 1);
            a->training_num.push_back(train_num);
            a->filter_lengths.push_back(filter_size);
            ++cnt;
        }
    a->thresh[t] = th;
    a->recorded[t] = 1;
    const int K = (int)a->uinds.size();
    std::vector<int> km(K), kl(K), kt(K);
    for (int k = 0; k < K; ++k) {
        km[k] = (a->training_num[k] - 1) * a->M + (a->uinds[k] - 1);
        kl[k] = a->filter_lengths[k];
        kt[k] = a->training_num[k];
    }
    // on the record's stream, ahead of the kernels that read them (a blocking copy from
    // pageable memory may return before it lands, and that stream does not wait on the
    // legacy stream); each call returns once its host bytes are staged
    AR_CU(a, cudaMemcpyAsync(a->kmap, km.data(), K * sizeof(int), cudaMemcpyHostToDevice, a->stream));
    AR_CU(a, cudaMemcpyAsync(a->klen, kl.data(), K * sizeof(int), cudaMemcpyHostToDevice, a->stream));
    AR_CU(a, cudaMemcpyAsync(a->ktrain, kt.data(), K * sizeof(int), cudaMemcpyHostToDevice, a->stream));
    AR_CU(a, cudaMemcpyAsync(a->dthresh, a->thresh.data(), a->T * sizeof(float), cudaMemcpyHostToDevice,
                             a->stream));
    if (added) *added = cnt;
    return CDLGB_OK;
}

int cdlgb_ar_info(const cdlgb_ar* a, int32_t* K, int32_t* uinds, int32_t* training_num,
                  int32_t* filter_lengths, int32_t cap) {
    if (!a || !K) return CDLGB_EINVAL;
    const int k = (int)a->uinds.size();
    *K = k;
    if (cap < k && (uinds || training_num || filter_lengths)) return CDLGB_EINVAL;
    for (int i = 0; i < k; ++i) {
        if (uinds) uinds[i] = a->uinds[i];
        if (training_num) training_num[i] = a->training_num[i];
        if (filter_lengths) filter_lengths[i] = a->filter_lengths[i];
    }
    return CDLGB_OK;
}

int cdlgb_ar_topology(cdlgb_ar* a, int32_t* over, int32_t* non_over, int32_t* next_to) {
    if (!a || !over || !non_over || !next_to) return CDLGB_EINVAL;
    const int K = (int)a->uinds.size();
    if (K == 0) return ar_err(a, CDLGB_ESTATE, "no filters recorded");
    AR_CU(a, cudaSetDevice(a->dev));
    int maxlen = *std::max_element(a->filter_lengths.begin(), a->filter_lengths.end());
    int minlen = *std::min_element(a->filter_lengths.begin(), a->filter_lengths.end());
    const int CmFm1 = a->C - minlen - 1;       // maximum_apart_length (helpers.jl:11)
    if (CmFm1 < 0) return ar_err(a, CDLGB_EINVAL, "filters longer than the sequences");
    const size_t n_over = (size_t)K * K * maxlen, n_non = (size_t)K * K * CmFm1, n_next = (size_t)K * K;
    const size_t need = n_over + n_non + n_next;
    if (a->dcount_cap < need) {
        if (a->dcount) cudaFree(a->dcount);
        a->dcount = nullptr;
        AR_CU(a, cudaMalloc((void**)&a->dcount, need * sizeof(int)));
        a->dcount_cap = need;
    }
    const int ctas = std::min(a->N, 152 * 4);
    if (a->list_ctas < ctas || !a->list) {
        if (a->list) cudaFree(a->list);
        a->list = nullptr;
        AR_CU(a, cudaMalloc((void**)&a->list, (size_t)ctas * a->T * a->M * a->C * sizeof(int)));
        a->list_ctas = ctas;
    }
    AR_CU(a, cudaMemsetAsync(a->dcount, 0, need * sizeof(int), a->stream));
    k_topology<<<ctas, 256, 0, a->stream>>>(a->codes, a->kmap, a->klen, a->ktrain, a->dthresh,
                                            a->N, a->M, a->C, K, maxlen, CmFm1, a->list, a->dcount,
                                            a->dcount + n_over, a->dcount + n_over + n_non);
    AR_CU(a, cudaGetLastError());
    AR_CU(a, cudaMemcpyAsync(over, a->dcount, n_over * sizeof(int), cudaMemcpyDeviceToHost, a->stream));
    AR_CU(a, cudaMemcpyAsync(non_over, a->dcount + n_over, n_non * sizeof(int), cudaMemcpyDeviceToHost, a->stream));
    AR_CU(a, cudaMemcpyAsync(next_to, a->dcount + n_over + n_non, n_next * sizeof(int), cudaMemcpyDeviceToHost, a->stream));
    AR_CU(a, cudaStreamSynchronize(a->stream));
    return CDLGB_OK;
}

int cdlgb_ar_pair_pfms(cdlgb_ar* a, cdlgb_ctx* c, const int32_t* pairs, int32_t P,
                       int32_t filter_size, float* pfms, int32_t* span_lens) {
    if (!a || !c || !pairs || !pfms || !span_lens || P <= 0 || filter_size < 1) return CDLGB_EINVAL;
    if (!c->loaded || c->N != a->N || c->L4 != 4 * a->C)
        return ar_err(a, CDLGB_EINVAL, "context does not hold the record's data");
    const int K = (int)a->uinds.size();
    const int max_span = 2 * filter_size - 1;   // extractions.jl:22
    for (int p = 0; p < P; ++p) {
        const int fr = pairs[3 * p], fc = pairs[3 * p + 1], o = pairs[3 * p + 2];
        if (fr < 1 || fr > K || fc < 1 || fc > K || o < 1 || o > a->filter_lengths[fr - 1])
            return ar_err(a, CDLGB_EINVAL, "pair %d = (%d, %d, %d) out of range (K=%d)", p, fr, fc, o, K);
        const int fl1 = a->filter_lengths[fr - 1], fl2 = a->filter_lengths[fc - 1];
        const int span = o >= fl2 ? o : fl1 - o + fl2;
        if (span > max_span || span > a->C)
            return ar_err(a, CDLGB_EINVAL, "pair %d spans %d bases (> %d)", p, span, max_span);
    }
    AR_CU(a, cudaSetDevice(a->dev));
    AR_CU(a, cudaStreamSynchronize(c->stream));
    const int nch = std::max(1, std::min(64, a->N / 64));
    const size_t npart = (size_t)P * nch * 4 * max_span;
    const size_t need = npart + (size_t)P * 4 * max_span + 3 * (size_t)P + P;
    if (a->msa_cap < need) {
        if (a->msa) cudaFree(a->msa);
        a->msa = nullptr;
        AR_CU(a, cudaMalloc((void**)&a->msa, need * sizeof(float)));
        a->msa_cap = need;
    }
    float* part = a->msa;
    float* dpfm = part + npart;
    int* dpairs = (int*)(dpfm + (size_t)P * 4 * max_span);
    int* dspan = dpairs + 3 * P;
    AR_CU(a, cudaMemcpyAsync(dpairs, pairs, 3 * (size_t)P * sizeof(int), cudaMemcpyHostToDevice, a->stream));
    k_pair_msa<<<dim3(P, nch), 128, 4 * max_span * sizeof(float), a->stream>>>(
        a->codes, c->S, dpairs, a->kmap, a->klen, a->dthresh, a->N, a->M, a->C, max_span, part);
    AR_CU(a, cudaGetLastError());
    k_pair_finish<<<P, 128, 4 * max_span * sizeof(double), a->stream>>>(part, dpairs, a->klen, P, nch,
                                                                       max_span, dpfm, dspan);
    AR_CU(a, cudaGetLastError());
    AR_CU(a, cudaMemcpyAsync(pfms, dpfm, (size_t)P * 4 * max_span * sizeof(float), cudaMemcpyDeviceToHost, a->stream));
    AR_CU(a, cudaMemcpyAsync(span_lens, dspan, P * sizeof(int), cudaMemcpyDeviceToHost, a->stream));
    AR_CU(a, cudaStreamSynchronize(a->stream));
    return CDLGB_OK;
}

}  // extern "C"
