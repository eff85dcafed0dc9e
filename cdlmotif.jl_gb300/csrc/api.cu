// C ABI entry points of libcdlgb (declared in include/cdlgb.h).
#include "cdlgb_internal.h"

#include <math.h>
#include <stdlib.h>
#include <algorithm>
#include <new>
#include <string>
#include <vector>

namespace {
thread_local char t_noctx_err[512];
}

int noctx_seterr(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(t_noctx_err, sizeof(t_noctx_err), fmt, ap);
    va_end(ap);
    return code;
}

const char* noctx_err() { return t_noctx_err[0] ? t_noctx_err : nullptr; }

int cdlgb_seterr(cdlgb_ctx* c, int code, const char* fmt, ...) {
    if (c) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(c->err, sizeof(c->err), fmt, ap);
        va_end(ap);
    }
    return code;
}

int cdlgb_after_launch(cdlgb_ctx* c, const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return cdlgb_seterr(c, CDLGB_ECUDA, "launch of %s failed: %s", what, cudaGetErrorString(e));
    c->launches++;
    return CDLGB_OK;
}

// ---- phase timers: a ring of event pairs, read back (and synchronised) on demand
namespace {
constexpr int kRing = 4096;
struct Ring {
    cudaEvent_t ev[2 * kRing];
    int ph[kRing];
    int w[kRing];           // units the interval covers (X-step iterations for PH_XSTEP)
    int used = 0;
    int open[PH_COUNT];
};
}  // namespace

static void ring_collect(cdlgb_ctx* c) {
    Ring* r = (Ring*)c->ring;
    if (!r) return;
    cudaStreamSynchronize(c->stream);
    for (int k = 0; k < r->used; ++k) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, r->ev[2 * k], r->ev[2 * k + 1]) == cudaSuccess) {
            c->ph_ms[r->ph[k]] += ms;
            c->ph_n[r->ph[k]] += r->w[k];
        }
    }
    r->used = 0;
}

void cdlgb_phase_begin(cdlgb_ctx* c, int ph) {
    Ring* r = (Ring*)c->ring;
    if (!c->profile || !r) return;
    if (r->used >= kRing) ring_collect(c);
    int k = r->used++;
    r->ph[k] = ph;
    r->w[k] = 1;
    r->open[ph] = k;
    cudaEventRecord(r->ev[2 * k], c->stream);
}

void cdlgb_phase_end_n(cdlgb_ctx* c, int ph, int units) {
    Ring* r = (Ring*)c->ring;
    if (!c->profile || !r) return;
    int k = r->open[ph];
    if (k < 0 || k >= r->used) return;
    r->w[k] = units;
    cudaEventRecord(r->ev[2 * k + 1], c->stream);
    r->open[ph] = -1;
}

void cdlgb_phase_end(cdlgb_ctx* c, int ph) { cdlgb_phase_end_n(c, ph, 1); }

// one-hot validation on the device: every entry must be 0 or 1 (the integer count
// kernels rely on it).  Sets c->onehot_exact; synchronises the stream.
__global__ void k_check_onehot(const float4* __restrict__ S, size_t n4, int* __restrict__ bad) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4;
         i += (size_t)gridDim.x * blockDim.x) {
        float4 v = S[i];
        bool ok = (v.x == 0.f || v.x == 1.f) && (v.y == 0.f || v.y == 1.f) &&
                  (v.z == 0.f || v.z == 1.f) && (v.w == 0.f || v.w == 1.f);
        if (!ok) *bad = 1;
    }
}

static int check_onehot(cdlgb_ctx* c) {
    int* flag = (int*)c->dscalar;      // 8 doubles of device scratch, first int used here
    CU_TRY(c, cudaMemsetAsync(flag, 0, sizeof(int), c->stream));
    size_t n4 = (size_t)c->L4 * c->N / 4;
    k_check_onehot<<<grid_for(n4, 256), 256, 0, c->stream>>>((const float4*)c->S, n4, flag);
    LAUNCH_CHECK(c, "k_check_onehot");
    int hbad = 0;
    CU_TRY(c, cudaMemcpyAsync(&hbad, flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CU_TRY(c, cudaStreamSynchronize(c->stream));
    c->onehot_exact = hbad == 0;
    return CDLGB_OK;
}

// read_fasta + data_2_dummy's rules (src/LOAD/read.jl:2-28, src/LOAD/to_dummy.jl:27-38)
// on the host: '>'-records, header line dropped, lines joined, records with 'N'/'n'
// dropped, the first max_entries kept, upper-cased; one byte per base (A C G T = 0..3;
// 4 for every base of a record whose length differs from the first one's).
int fasta_codes(const char* text, size_t nbytes, int32_t max_entries, std::vector<uint8_t>& codes,
                int32_t* N_out, int32_t* L_out, int32_t* wrong_out, char* err, size_t errlen) {
    if (!text || max_entries <= 0) {
        snprintf(err, errlen, "load_fasta: null text or max_entries <= 0");
        return CDLGB_EINVAL;
    }
    std::vector<std::string> reads;
    size_t i = 0;
    while (i < nbytes && (int)reads.size() < max_entries) {
        size_t j = i;
        while (j < nbytes && text[j] != '>') ++j;            // chunk [i, j)
        if (j > i) {
            size_t k = i;
            while (k < j && text[k] != '\n') ++k;           // header line
            std::string r;
            bool has_n = false;
            for (size_t t = k; t < j; ++t) {
                const char ch = text[t];
                if (ch == '\n') continue;
                if (ch == 'N' || ch == 'n') has_n = true;
                r.push_back(ch);
            }
            if (!has_n) reads.push_back(std::move(r));
        }
        i = j + 1;
    }
    if (reads.empty()) { snprintf(err, errlen, "load_fasta: no sequences"); return CDLGB_EINVAL; }
    const size_t L = reads[0].size();
    if (L == 0) { snprintf(err, errlen, "load_fasta: the first sequence is empty"); return CDLGB_EINVAL; }
    if (L > (size_t)(1 << 28) / 4) { snprintf(err, errlen, "load_fasta: sequences too long"); return CDLGB_EINVAL; }
    const int32_t N = (int32_t)reads.size();
    codes.assign((size_t)N * L, 0);
    int32_t wrong = 0;
    for (int32_t n = 0; n < N; ++n) {
        const std::string& r = reads[n];
        uint8_t* o = codes.data() + (size_t)n * L;
        if (r.size() != L) {           // left uninitialised by the reference; zeros here
            ++wrong;
            memset(o, 4, L);
            continue;
        }
        for (size_t l = 0; l < L; ++l) {
            const char u = (char)toupper((unsigned char)r[l]);
            const uint8_t b = u == 'A' ? 0 : u == 'C' ? 1 : u == 'G' ? 2 : u == 'T' ? 3 : 255;
            if (b == 255) {   // dummy[uppercase(c)] raises a KeyError in the reference
                snprintf(err, errlen, "load_fasta: record %d has character 0x%02x at %zu", n,
                         (unsigned)(unsigned char)r[l], l);
                return CDLGB_EINVAL;
            }
            o[l] = b;
        }
    }
    *N_out = N;
    *L_out = (int32_t)L;
    *wrong_out = wrong;
    return CDLGB_OK;
}

extern "C" {
static int load_impl(cdlgb_ctx* c, const float* onehot, const uint8_t* codes, int32_t L4, int32_t N);
}

// the context loaded from one byte per base (fasta_codes' output)
int load_codes(cdlgb_ctx* c, const uint8_t* codes, int32_t L, int32_t N) {
    return load_impl(c, nullptr, codes, 4 * L, N);
}

extern "C" {

int cdlgb_params_default(cdlgb_params* p) {
    if (!p) return CDLGB_EINVAL;
    memset(p, 0, sizeof(*p));
    p->M = 10;
    p->filter_size = 4;
    p->rho = 100.f;
    p->sigma = 100.f;
    p->lambda = 0.01f;
    p->csc_iter_num = 15;
    p->cdl_iter_num = 1;
    p->iter_num = 10;
    p->std_threshold_multiplier = 1.f;
    p->sherman_const_csc = 2.f;
    p->sherman_const_cdl = 2.f;
    p->device = 0;
    p->init_mode = 0;
    p->fft_mode = 0;
    p->hbm_budget_bytes = 0;
    p->stop_tol = 0.f;
    p->track_residuals = 0;
    return CDLGB_OK;
}

static int check_params(cdlgb_ctx* c, const cdlgb_params* p) {
    if (p->M < 1 || p->M > 4096) return cdlgb_seterr(c, CDLGB_EINVAL, "M=%d out of range", p->M);
    if (p->filter_size < 1 || p->filter_size > 1024)
        return cdlgb_seterr(c, CDLGB_EINVAL, "filter_size=%d out of range", p->filter_size);
    if (!(p->rho > 0) || !(p->sigma > 0) || !(p->lambda >= 0))
        return cdlgb_seterr(c, CDLGB_EINVAL, "rho, sigma must be > 0 and lambda >= 0");
    if (!(p->sherman_const_csc > 0) || !(p->sherman_const_cdl > 0))
        return cdlgb_seterr(c, CDLGB_EINVAL, "sherman constants must be > 0");
    if (p->fft_mode < 0 || p->fft_mode > 2)
        return cdlgb_seterr(c, CDLGB_EINVAL, "fft_mode=%d (0 auto, 1 cuFFT, 2 fused)", p->fft_mode);
    if (!(p->stop_tol >= 0.f))
        return cdlgb_seterr(c, CDLGB_EINVAL, "stop_tol must be >= 0 (0 = fixed iteration count)");
    return CDLGB_OK;
}

int cdlgb_create(const cdlgb_params* p, cdlgb_ctx** out) {
    if (!p || !out) return noctx_seterr(CDLGB_EINVAL, "cdlgb_create: null argument");
    *out = nullptr;
    cdlgb_ctx* c = new (std::nothrow) cdlgb_ctx();
    if (!c) return noctx_seterr(CDLGB_EINVAL, "cdlgb_create: out of host memory");
    c->err[0] = 0;
    c->p = *p;
    int st = check_params(c, p);
    if (st) {
        noctx_seterr(st, "cdlgb_create: %s", c->err);
        delete c;
        return st;
    }
    c->dev = p->device;
    c->res_on = p->track_residuals != 0 || p->stop_tol > 0.f;
    cudaError_t e = cudaSetDevice(c->dev);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        noctx_seterr(CDLGB_ECUDA, "cdlgb_create: device %d: %s", c->dev, cudaGetErrorString(e));
        delete c;
        return CDLGB_ECUDA;
    }
    c->own_stream = true;
    // load the allocation-free objective's module and look up its scratch on this
    // device now, while the caller's memory is still free (lazy module loading would
    // otherwise do it at the first cdlgb_objective_noalloc call); a failure here only
    // leaves that lookup to the first call
    (void)noalloc_warm_current_device();
    Ring* r = new (std::nothrow) Ring();
    if (r) {
        bool ok = true;
        for (int i = 0; i < 2 * kRing && ok; ++i) ok = cudaEventCreate(&r->ev[i]) == cudaSuccess;
        for (int i = 0; i < PH_COUNT; ++i) r->open[i] = -1;
        if (!ok) { delete r; r = nullptr; }
    }
    c->ring = r;
    *out = c;
    return CDLGB_OK;
}

int cdlgb_destroy(cdlgb_ctx* c) {
    if (!c) return CDLGB_OK;
    cudaSetDevice(c->dev);
    if (c->stream) cudaStreamSynchronize(c->stream);
    admm_free(c);
    fused_free(c);
    scan_free(c);
    dev_free(c, c->S);
    dev_free(c, c->S_bg);
    Ring* r = (Ring*)c->ring;
    if (r) {
        for (int i = 0; i < 2 * kRing; ++i) cudaEventDestroy(r->ev[i]);
        delete r;
    }
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return CDLGB_OK;
}

const char* cdlgb_last_error(const cdlgb_ctx* c) {
    if (c) return c->err;
    const char* m = noctx_err();
    return m ? m : "null context";
}

static int pick_fused(const cdlgb_params* p, int Lg) {
    if (p->fft_mode == 1) return 0;
    int ok = fused_supported(Lg, p->M, Lg - 8 * p->filter_size);
    if (p->fft_mode == 2) return ok ? 1 : -1;
    return ok;
}

int cdlgb_footprint(const cdlgb_params* p, int32_t L, int32_t N, uint64_t* bytes) {
    if (!p || !bytes || L <= 0 || N <= 0) return CDLGB_EINVAL;
    int L4 = 4 * L, Lg = L4 + 8 * p->filter_size;
    int f = pick_fused(p, Lg);
    *bytes = admm_footprint(p, L4, N, f > 0);
    return CDLGB_OK;
}

// one thread per base: code 0..3 -> the one-hot column (A, C, G, T); any other code
// (a record whose length differs from the first) -> zeros
__global__ void k_encode_onehot(const uint8_t* __restrict__ codes, float4* __restrict__ S, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const unsigned b = codes[i];
        S[i] = make_float4(b == 0 ? 1.f : 0.f, b == 1 ? 1.f : 0.f, b == 2 ? 1.f : 0.f, b == 3 ? 1.f : 0.f);
    }
}

// Uploads the data: the float one-hot matrix as given, or (codes != NULL) one byte per
// base, expanded on the device (timed as part of the set-up phase).
static int upload_data_timed(cdlgb_ctx* c, const float* onehot, const uint8_t* codes, size_t n);
static int upload_data(cdlgb_ctx* c, const float* onehot, const uint8_t* codes, size_t n) {
    cdlgb_phase_begin(c, PH_SETUP);
    const int st = upload_data_timed(c, onehot, codes, n);
    cdlgb_phase_end(c, PH_SETUP);
    return st;
}

static int upload_data_timed(cdlgb_ctx* c, const float* onehot, const uint8_t* codes, size_t n) {
    if (onehot) {
        CU_TRY(c, cudaMemcpyAsync(c->S, onehot, n * 4, cudaMemcpyHostToDevice, c->stream));
        return check_onehot(c);
    }
    uint8_t* d = nullptr;
    CU_TRY(c, dev_copy_in(c, (void**)&d, codes, n / 4));
    k_encode_onehot<<<grid_for(n / 4, 256), 256, 0, c->stream>>>(d, (float4*)c->S, n / 4);
    cudaError_t e = cudaGetLastError();
    dev_free(c, d);
    if (e != cudaSuccess) return cdlgb_seterr(c, CDLGB_ECUDA, "k_encode_onehot: %s", cudaGetErrorString(e));
    CU_TRY(c, cudaStreamSynchronize(c->stream));
    c->onehot_exact = true;      // 0/1 by construction
    return CDLGB_OK;
}


int cdlgb_load_data(cdlgb_ctx* c, const float* onehot, int32_t L4, int32_t N) {
    if (!c) return CDLGB_EINVAL;
    if (!onehot || L4 <= 0 || N <= 0)
        return cdlgb_seterr(c, CDLGB_EINVAL, "load_data: null data or bad size (4L=%d, N=%d)", L4, N);
    return load_impl(c, onehot, nullptr, L4, N);
}

static int load_impl(cdlgb_ctx* c, const float* onehot, const uint8_t* codes, int32_t L4, int32_t N) {
    // CDL_setup.jl:174
    if (L4 % 4) return cdlgb_seterr(c, CDLGB_EINVAL, "first dimension of dat must be multiple of 4s (got %d)", L4);
    CU_TRY(c, cudaSetDevice(c->dev));
    if (c->loaded && c->L4 == L4 && c->N == N) {
        // same shape as the resident dataset: keep every buffer and plan, replace the data
        c->initialized = false;
        c->bg_valid = c->use_bg = 0;
        return upload_data(c, onehot, codes, (size_t)L4 * N);
    }
    if (c->loaded) {
        CU_TRY(c, cudaStreamSynchronize(c->stream));
        admm_free(c);
        fused_free(c);
        dev_free(c, c->S);
        dev_free(c, c->S_bg);
        c->S = c->S_bg = nullptr;
        c->bg_valid = c->use_bg = 0;
        c->loaded = c->initialized = false;
    }
    const cdlgb_params& p = c->p;
    c->L4 = L4;
    c->N = N;
    c->M = p.M;
    c->gamma = 4 * p.filter_size;
    c->Lg = L4 + 2 * c->gamma;
    c->F = c->Lg / 2 + 1;
    c->LMN = (size_t)c->Lg * c->M * N;
    c->LN = (size_t)c->Lg * N;
    c->LM = (size_t)c->Lg * c->M;
    int f = pick_fused(&p, c->Lg);
    if (f < 0)
        return cdlgb_seterr(c, CDLGB_ENOTSUP, "fused path does not support Lg=%d, M=%d", c->Lg, c->M);
    c->fused = f;
    if (const char* e = getenv("CDLGB_ROWFFT")) c->rows_cufft = atoi(e) == 0;
    // admission by HBM footprint
    size_t need = admm_footprint(&p, L4, N, c->fused);
    size_t freeb = 0, total = 0;
    CU_TRY(c, cudaMemGetInfo(&freeb, &total));
    freeb += devmem_reusable(c->dev);      // held by the library's pool, free for reuse
    size_t budget = p.hbm_budget_bytes ? (size_t)p.hbm_budget_bytes
                                       : (freeb > (1ull << 30) ? freeb - (1ull << 30) : 0);
    if (need > budget)
        return cdlgb_seterr(c, CDLGB_ENOMEM_BUDGET,
                            "dataset needs %.2f GB of device memory, budget is %.2f GB (N=%d, 4L=%d, M=%d)",
                            need / 1e9, budget / 1e9, N, L4, c->M);
    size_t n = (size_t)L4 * N;
    ST_TRY(dev_alloc(c, (void**)&c->S, n * 4));
    int st = admm_alloc(c);
    if (st == CDLGB_OK && c->fused) st = fused_setup(c);
    if (st != CDLGB_OK) {
        std::string msg = c->err;
        cudaGetLastError();
        admm_free(c);
        fused_free(c);
        dev_free(c, c->S);
        c->S = nullptr;
        return cdlgb_seterr(c, st, "%s", msg.c_str());
    }
    c->loaded = true;
    return upload_data(c, onehot, codes, n);
}

// read_fasta (src/LOAD/read.jl:2-28) and data_2_dummy (src/LOAD/to_dummy.jl:27-38):
// records are the '>'-separated chunks of the text; in each, the first line (header)
// is dropped and the remaining lines are joined (only '\n' is removed); records that
// contain 'N' or 'n' are dropped; the first max_entries are kept and upper-cased.
int cdlgb_load_fasta(cdlgb_ctx* c, const char* text, size_t nbytes, int32_t max_entries,
                     int32_t* N_out, int32_t* L_out, int32_t* n_wrong_len) {
    if (!c) return CDLGB_EINVAL;
    std::vector<uint8_t> codes;
    int32_t N = 0, L = 0, wrong = 0;
    char err[256];
    int st = fasta_codes(text, nbytes, max_entries, codes, &N, &L, &wrong, err, sizeof(err));
    if (st != CDLGB_OK) return cdlgb_seterr(c, st, "%s", err);
    st = load_impl(c, nullptr, codes.data(), 4 * L, N);
    if (st != CDLGB_OK) return st;
    if (N_out) *N_out = N;
    if (L_out) *L_out = L;
    if (n_wrong_len) *n_wrong_len = wrong;
    return CDLGB_OK;
}

int cdlgb_dims(const cdlgb_ctx* c, int32_t* L4, int32_t* N, int32_t* M, int32_t* gamma, int32_t* Lg) {
    if (!c) return CDLGB_EINVAL;
    if (!c->loaded) return CDLGB_ESTATE;
    if (L4) *L4 = c->L4;
    if (N) *N = c->N;
    if (M) *M = c->M;
    if (gamma) *gamma = c->gamma;
    if (Lg) *Lg = c->Lg;
    return CDLGB_OK;
}

#define NEED_LOADED(c)                                                                   \
    do {                                                                                 \
        if (!(c)) return CDLGB_EINVAL;                                                   \
        if (!(c)->loaded) return cdlgb_seterr((c), CDLGB_ESTATE, "no data loaded");      \
        CU_TRY((c), cudaSetDevice((c)->dev));                                            \
    } while (0)
#define NEED_INIT(c)                                                                     \
    do {                                                                                 \
        NEED_LOADED(c);                                                                  \
        if (!(c)->initialized) return cdlgb_seterr((c), CDLGB_ESTATE, "state not initialised"); \
    } while (0)

int cdlgb_init_state(cdlgb_ctx* c, const float* X0, const float* D0, uint64_t seed) {
    NEED_LOADED(c);
    c->initialized = false;
    cdlgb_phase_begin(c, PH_SETUP);
    const int st = admm_init(c, X0, D0, seed);
    cdlgb_phase_end(c, PH_SETUP);
    return st;
}

int cdlgb_code_update(cdlgb_ctx* c, int32_t num_iter) {
    NEED_INIT(c);
    if (num_iter < 0) return cdlgb_seterr(c, CDLGB_EINVAL, "num_iter < 0");
    return admm_code_update(c, num_iter);
}

int cdlgb_dict_update(cdlgb_ctx* c, int32_t num_iter) {
    NEED_INIT(c);
    if (num_iter < 0) return cdlgb_seterr(c, CDLGB_EINVAL, "num_iter < 0");
    return admm_dict_update(c, num_iter);
}

int cdlgb_objective(cdlgb_ctx* c, double* obj) {
    NEED_INIT(c);
    if (!obj) return cdlgb_seterr(c, CDLGB_EINVAL, "obj is NULL");
    return admm_objective(c, obj);
}

int cdlgb_update_best(cdlgb_ctx* c, double* obj, int32_t* improved) {
    NEED_INIT(c);
    int imp = 0;
    ST_TRY(admm_update_best(c, obj, &imp));
    if (improved) *improved = imp;
    return CDLGB_OK;
}

int cdlgb_run_outer(cdlgb_ctx* c, int32_t iter_num, double* objs) {
    NEED_INIT(c);
    if (iter_num < 0) return cdlgb_seterr(c, CDLGB_EINVAL, "iter_num < 0");
    c->outer_done = 0;
    for (int it = 0; it < iter_num; ++it) {
        ST_TRY(admm_code_update(c, c->p.csc_iter_num));
        double o = 0;
        int imp = 0;
        ST_TRY(admm_update_best(c, &o, &imp));
        ST_TRY(admm_dict_update(c, c->p.cdl_iter_num));
        if (objs) objs[it] = o;
        c->outer_done = it + 1;
        if (c->p.stop_tol > 0.f) {
            // the stopping test: the largest relative residual (float64, on the device)
            CU_TRY(c, cudaMemcpyAsync(c->hscalar + 7, c->dres + RESIDUAL_REL_MAX, sizeof(double),
                                      cudaMemcpyDeviceToHost, c->stream));
            CU_TRY(c, cudaStreamSynchronize(c->stream));
            if (c->hscalar[7] <= (double)c->p.stop_tol) break;
        }
    }
    return CDLGB_OK;
}

int cdlgb_code_threshold(cdlgb_ctx* c, double* thresh) {
    NEED_INIT(c);
    if (!thresh) return cdlgb_seterr(c, CDLGB_EINVAL, "thresh is NULL");
    cdlgb_phase_begin(c, PH_THRESH);
    const int st = admm_code_threshold(c, thresh);
    cdlgb_phase_end(c, PH_THRESH);
    return st;
}

int cdlgb_get(cdlgb_ctx* c, int32_t field, void* dst, size_t bytes) {
    if (field == CDLGB_FIELD_DATA || field == CDLGB_FIELD_BACKGROUND) {
        NEED_LOADED(c);
        if (!dst || bytes != (size_t)c->L4 * c->N * 4)
            return cdlgb_seterr(c, CDLGB_EINVAL, "data is (4L, N) float32");
        if (field == CDLGB_FIELD_BACKGROUND && !c->bg_valid)
            return cdlgb_seterr(c, CDLGB_ESTATE, "no background made (cdlgb_make_background)");
        CU_TRY(c, cudaMemcpyAsync(dst, field == CDLGB_FIELD_DATA ? c->S : c->S_bg, bytes,
                                  cudaMemcpyDeviceToHost, c->stream));
        CU_TRY(c, cudaStreamSynchronize(c->stream));
        return CDLGB_OK;
    }
    NEED_INIT(c);
    if (!dst) return cdlgb_seterr(c, CDLGB_EINVAL, "dst is NULL");
    if (field == CDLGB_FIELD_D || field == CDLGB_FIELD_G1_DUAL || field == CDLGB_FIELD_G3_DUAL)
        ST_TRY(admm_sync_time_state(c));
    const void* src = nullptr;
    size_t want = 0;
    const size_t LMN = c->LMN * 4, LN = c->LN * 4, LM = c->LM * 4;
    switch (field) {
        case CDLGB_FIELD_X: src = c->Xb[c->xcur]; want = LMN; break;
        case CDLGB_FIELD_X_BEST: src = c->best_is_cur ? c->Xb[c->xcur] : c->Xb[1 - c->xcur]; want = LMN; break;
        case CDLGB_FIELD_D: src = c->d; want = LMN; break;
        case CDLGB_FIELD_D_BEST: src = c->Dbest; want = LM; break;
        case CDLGB_FIELD_G1: src = c->G1; want = LM; break;
        case CDLGB_FIELD_G3: src = c->G3; want = LM; break;
        case CDLGB_FIELD_DX: src = c->DX; want = LN; break;
        case CDLGB_FIELD_Y1: src = c->Y1; want = LN; break;
        case CDLGB_FIELD_Y2_DUAL: src = c->y2; want = LMN; break;
        case CDLGB_FIELD_Y3_DUAL: src = c->y3; want = LMN; break;
        case CDLGB_FIELD_G1_DUAL: src = c->g1; want = LMN; break;
        case CDLGB_FIELD_G3_DUAL: src = c->g3; want = LMN; break;
        case CDLGB_FIELD_TD: src = c->Td; want = LN; break;
        case CDLGB_FIELD_G2: src = c->G2; want = LN; break;
        case CDLGB_FIELD_G2_DUAL: src = c->g2; want = LN; break;
        case CDLGB_FIELD_Y1_DUAL: src = c->y1; want = LN; break;
        case CDLGB_FIELD_OBJ_BEST:
            if (bytes != sizeof(double)) return cdlgb_seterr(c, CDLGB_EINVAL, "obj_best is one float64");
            *(double*)dst = c->obj_best;
            return CDLGB_OK;
        case CDLGB_FIELD_RESIDUALS: src = c->dres; want = RESIDUAL_COUNT * sizeof(double); break;
        case CDLGB_FIELD_OUTER_DONE:
            if (bytes != sizeof(int32_t)) return cdlgb_seterr(c, CDLGB_EINVAL, "outer_done is one int32");
            *(int32_t*)dst = c->outer_done;
            return CDLGB_OK;
        default: return cdlgb_seterr(c, CDLGB_EINVAL, "unknown field %d", field);
    }
    if (bytes != want)
        return cdlgb_seterr(c, CDLGB_EINVAL, "field %d is %zu bytes, got %zu", field, want, bytes);
    CU_TRY(c, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream));
    CU_TRY(c, cudaStreamSynchronize(c->stream));
    return CDLGB_OK;
}

int cdlgb_scan_fwd(cdlgb_ctx* c, const float* pwms, const int32_t* lens, const float* thresh,
                   int32_t K, int32_t maxlen, int32_t* pos_out) {
    NEED_LOADED(c);
    if (!pos_out) return cdlgb_seterr(c, CDLGB_EINVAL, "pos_out is NULL");
    return scan_fwd(c, pwms, lens, thresh, K, maxlen, pos_out);
}

int cdlgb_autotune(cdlgb_ctx* c, int32_t max_candidates, double* ms_per_xstep, int32_t* kind,
                   int32_t* cluster, int32_t* filters, int32_t* n_candidates, int32_t* chosen) {
    NEED_INIT(c);
    if (!ms_per_xstep || !kind || !cluster || !filters || !n_candidates || !chosen || max_candidates <= 0)
        return cdlgb_seterr(c, CDLGB_EINVAL, "autotune: bad arguments");
    if (!c->fused) return cdlgb_seterr(c, CDLGB_ENOTSUP, "autotune: the cuFFT path has no variants");
    return fused_autotune(c, max_candidates, ms_per_xstep, kind, cluster, filters, n_candidates, chosen);
}

int cdlgb_pvalue_thresholds(cdlgb_ctx* c, const float* pwms, const int32_t* lens, int32_t K,
                            int32_t maxlen, double pval, float* thresh_out) {
    if (!c) return CDLGB_EINVAL;
    CU_TRY(c, cudaSetDevice(c->dev));
    return touzet_thresholds(c, pwms, lens, K, maxlen, pval, thresh_out);
}

int cdlgb_select_nonoverlapping(cdlgb_ctx* c, int32_t* pos, float* score, uint8_t* use_comp,
                                const int32_t* lens, int32_t K) {
    if (!c) return CDLGB_EINVAL;
    return nonoverlap_select(c, pos, score, use_comp, lens, K);
}

int cdlgb_scan_both(cdlgb_ctx* c, const float* pwms, const int32_t* lens, const float* thresh,
                    int32_t K, int32_t maxlen, int32_t* pos_out, float* score_out,
                    uint8_t* use_comp_out) {
    NEED_LOADED(c);
    return scan_both(c, pwms, lens, thresh, K, maxlen, pos_out, score_out, use_comp_out);
}

int cdlgb_count_pfms(cdlgb_ctx* c, const int32_t* pos, const uint8_t* use_comp,
                     const int32_t* lens, int32_t K, int32_t maxlen, int32_t* counts_out,
                     int32_t* nseq_out) {
    NEED_LOADED(c);
    return count_pfms(c, pos, use_comp, lens, K, maxlen, counts_out, nseq_out);
}

int cdlgb_extend_positions(cdlgb_ctx* c, int32_t* pos, const uint8_t* use_comp, int32_t* lens,
                           int32_t K, const float* bg, float pseudocount, float perc_no_less_than,
                           float ic_extension_thresh, int32_t* dec_out, int32_t* inc_out) {
    NEED_LOADED(c);
    return extend_positions(c, pos, use_comp, lens, K, bg, pseudocount, perc_no_less_than,
                            ic_extension_thresh, dec_out, inc_out);
}

int cdlgb_rescore_positions(cdlgb_ctx* c, const float* pwms, const int32_t* pos,
                            const int32_t* lens, int32_t K, int32_t maxlen, float* score_out) {
    NEED_LOADED(c);
    return rescore_positions(c, pwms, pos, lens, K, maxlen, score_out);
}

int cdlgb_make_background(cdlgb_ctx* c, int32_t k, uint64_t seed) {
    NEED_LOADED(c);
    return make_background(c, k, (unsigned long long)seed);
}

int cdlgb_select_data(cdlgb_ctx* c, int32_t which) {
    NEED_LOADED(c);
    if (which != 0 && which != 1) return cdlgb_seterr(c, CDLGB_EINVAL, "select_data: which=%d", which);
    if (which == 1 && !c->bg_valid)
        return cdlgb_seterr(c, CDLGB_ESTATE, "no background made (cdlgb_make_background)");
    c->use_bg = which;
    return CDLGB_OK;
}

// ------------------------------------------------------------------ instrumentation
int cdlgb_set_stream(cdlgb_ctx* c, void* stream) {
    if (!c) return CDLGB_EINVAL;
    CU_TRY(c, cudaSetDevice(c->dev));
    if (c->stream) CU_TRY(c, cudaStreamSynchronize(c->stream));
    if (stream) {
        if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
        c->own_stream = false;
        c->stream = (cudaStream_t)stream;
    } else if (!c->own_stream) {
        CU_TRY(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        c->own_stream = true;
    }
    return cdlgb_set_plan_streams(c);
}

int cdlgb_profile(cdlgb_ctx* c, int32_t enable) {
    if (!c) return CDLGB_EINVAL;
    if (!c->ring) return cdlgb_seterr(c, CDLGB_ECUDA, "no timing events available");
    ring_collect(c);
    c->profile = enable ? 1 : 0;
    return CDLGB_OK;
}

int cdlgb_profile_read(cdlgb_ctx* c, double* ms, int64_t* counts, int64_t* launches,
                       int64_t* fft_calls, int32_t reset) {
    if (!c) return CDLGB_EINVAL;
    ring_collect(c);
    for (int i = 0; i < PH_COUNT; ++i) {
        if (ms) ms[i] = c->ph_ms[i];
        if (counts) counts[i] = c->ph_n[i];
    }
    if (launches) *launches = c->launches;
    if (fft_calls) *fft_calls = c->fft_calls;
    if (reset) {
        for (int i = 0; i < PH_COUNT; ++i) { c->ph_ms[i] = 0; c->ph_n[i] = 0; }
        c->launches = 0;
        c->fft_calls = 0;
    }
    return CDLGB_OK;
}

}  // extern "C"
