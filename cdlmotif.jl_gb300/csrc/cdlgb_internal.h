// Internal declarations shared by the libcdlgb translation units.
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>
#include <stdint.h>
#include <stddef.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include "cdlgb.h"

// Per-phase timers (CUDA events on the context's stream), enabled on demand.
enum cdlgb_phase {
    PH_XSTEP = 0,     // one whole X-step iteration
    PH_DSTEP,         // one whole D-step iteration
    PH_OBJ,           // objective / update_best
    PH_XFUSED,        // the fused X-step kernel alone
    PH_SETUP,         // the data upload's copy and kernels, and the state initialisation
    PH_THRESH,        // the code threshold
    PH_SCAN,
    PH_COUNT
};

// The residual record (float64 on the device, resid.cu), in order; read with
// cdlgb_get(CDLGB_FIELD_RESIDUALS).
enum cdlgb_residual {
    RESIDUAL_X_Y2 = 0,        // sum (X - shrink(X + y2))^2        after a code update
    RESIDUAL_X_Y3,            // sum (X - projectionX(X + y3))^2
    RESIDUAL_X_Y1,            // sum (DX - Y1)^2
    RESIDUAL_X_NORM,          // sum X^2
    RESIDUAL_DX_NORM,         // sum DX^2
    RESIDUAL_D_G1,            // sum (d - G1_old)^2               after a D-step
    RESIDUAL_D_G3,            // sum (d - G3_old)^2
    RESIDUAL_D_G2,            // sum (Td - G2)^2
    RESIDUAL_D_NORM,          // sum d^2
    RESIDUAL_TD_NORM,         // sum Td^2
    RESIDUAL_DUAL_G1,         // N sum (G1 - G1_old)^2
    RESIDUAL_DUAL_G3,         // N sum (G3 - G3_old)^2
    RESIDUAL_G_NORM,          // N (sum G1^2 + sum G3^2)
    RESIDUAL_REL_PRIMAL_X,    // sqrt((X_Y2 + X_Y3) / X_NORM)
    RESIDUAL_REL_PRIMAL_DX,   // sqrt(X_Y1 / DX_NORM)
    RESIDUAL_REL_PRIMAL_D,    // sqrt((D_G1 + D_G3) / (2 D_NORM))
    RESIDUAL_REL_PRIMAL_TD,   // sqrt(D_G2 / TD_NORM)
    RESIDUAL_REL_DUAL_D,      // sqrt((DUAL_G1 + DUAL_G3) / G_NORM)
    RESIDUAL_REL_MAX,         // the largest of the five: the stopping test's value
    RESIDUAL_COUNT
};

struct cdlgb_ctx {
    cdlgb_params p;
    int dev = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    char err[1024];

    bool loaded = false, initialized = false;
    int L4 = 0, N = 0, M = 0, gamma = 0, Lg = 0, F = 0;
    size_t LMN = 0, LN = 0, LM = 0;
    int fused = 0;                  // 1 when the fused in-kernel-FFT X-step is used
    int absx_fused = 0;             // sum |X| partials of the last fused X-step are current

    // one-hot data, (N, L4) == Julia (4L, N)
    float* S = nullptr;
    int onehot_exact = 0;
    // k-let shuffled background of S (same layout) and which of the two the scan family
    // reads (the ADMM always reads S)
    float* S_bg = nullptr;
    int bg_valid = 0, use_bg = 0;

    // LMN state
    float* Xb[2] = {nullptr, nullptr};
    int xcur = 0;                   // Xb[xcur] holds X
    int best_is_cur = 1;            // X_best aliases Xb[xcur] (else Xb[1-xcur])
    float *y2 = nullptr, *y3 = nullptr, *d = nullptr, *g1 = nullptr, *g3 = nullptr;
    // fused path: the last D-step's d-hat (N, M, F), rfft(d) for the next D-step's Td sum,
    // valid while dh_valid is set (a D-step through the streaming transforms sets it;
    // initialisation and the other D-step paths clear it)
    float2* Dhs = nullptr;
    int dh_valid = 0;
    // spectral D-step state (dspec.cu): with dspec set, d-hat (Dhs), g1-hat (N, M, F) and
    // Dg = g1-hat - g3-hat (M, F, the same for every sequence) are the dictionary state
    // and d, g1, g3 are refreshed from them on demand (time_stale); G3-hat, the per-range
    // sums and their total are scratch
    float2 *g1h = nullptr, *Dg = nullptr, *G3h = nullptr, *spart = nullptr, *sumspec = nullptr;
    int dspec = 0, time_stale = 0;
    // with dspec: d, g1, g3 still to receive their initial values (d = G1 broadcast,
    // g1 = g3 = 0), written when first read, unless a D-step comes first
    int time_init = 0;
    int absx_init = 0;              // dred[0, 304) holds sum |X| of the initial X
    // LN state
    float *Y1 = nullptr, *y1 = nullptr, *DX = nullptr, *Td = nullptr, *G2 = nullptr, *g2 = nullptr;
    // LM state
    float *G1 = nullptr, *G3 = nullptr, *dsum = nullptr, *Dbest = nullptr, *vbar = nullptr;
    float2* G1h = nullptr;          // (M, F) rfft of G1
    float* Ah = nullptr;            // (F) sum_m |G1h|^2

    // scratch (cuFFT path)
    float *sA = nullptr, *sB = nullptr;              // LMN real
    float2 *sAh = nullptr, *sBh = nullptr, *sCh = nullptr;   // (N, M, F) spectra
    float* sU = nullptr;                              // LN real
    float2 *sUh = nullptr, *sVh = nullptr;            // (N, F)
    float* part = nullptr;                            // D-step partial sums
    int nchunk = 0;
    double* dred = nullptr;                           // reduction partials (float64)
    int nred = 0;
    double* dscalar = nullptr;                        // device scalars
    double* hscalar = nullptr;                        // pinned host mirror
    bool hscalar_own = false;                         // from cudaMallocHost, not the slab
    double obj_best = 0.0;
    // residual record (RESIDUAL_COUNT float64), its per-block partials, G1 and G3 of
    // the D-step before their update (2 LM), outer iterations of the last run_outer
    double* dres = nullptr;
    double* rpart = nullptr;
    float* Gprev = nullptr;
    int outer_done = 0;
    int res_on = 0;                 // residual record kept (params.track_residuals or stop_tol > 0)

    // fused path twiddles / plan
    void* fplan = nullptr;

    void* plans = nullptr;          // cuFFT plan cache keyed by (direction, batch)
    int chunk = 0;                  // sequences per chunk of the cuFFT-transform passes
    int schunk = 0;                 // sequences per chunk of the spectral D-step
    int dslots = 0;                 // its partial-sum slots over all chunks
    int nsm = 0;                    // SMs of the device

    // scan scratch
    int32_t* scan_i = nullptr; size_t scan_i_cap = 0;
    float* scan_f = nullptr; size_t scan_f_cap = 0;
    uint8_t* scan_u = nullptr; size_t scan_u_cap = 0;

    // instrumentation
    int profile = 0;
    void* ring = nullptr;           // event ring for the phase timers
    double ph_ms[PH_COUNT] = {};
    int64_t ph_n[PH_COUNT] = {};
    int64_t launches = 0;           // our own kernel launches
    int64_t fft_calls = 0;          // cuFFT exec calls
    bool rows_cufft = false;        // CDLGB_ROWFFT=0: row transforms on cuFFT even where
                                    // the register-FFT row kernels exist
};

int cdlgb_seterr(cdlgb_ctx* c, int code, const char* fmt, ...);
// the calling thread's message for a failure with no handle to hold it (creating a
// context, record or server; the allocation-free objective), returned by the
// *_last_error calls given a null handle; nullptr when there is none
int noctx_seterr(int code, const char* fmt, ...);
const char* noctx_err();

#define CU_TRY(c, call)                                                                 \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess)                                                          \
            return cdlgb_seterr((c), CDLGB_ECUDA, "%s failed: %s (%s:%d)", #call,        \
                                cudaGetErrorString(e_), __FILE__, __LINE__);            \
    } while (0)

#define FFT_TRY(c, call)                                                                \
    do {                                                                                \
        cufftResult r_ = (call);                                                        \
        if (r_ != CUFFT_SUCCESS)                                                        \
            return cdlgb_seterr((c), CDLGB_ECUDA, "%s failed: cufft status %d (%s:%d)",  \
                                #call, (int)r_, __FILE__, __LINE__);                    \
    } while (0)

#define ST_TRY(call)                                                                    \
    do {                                                                                \
        int s_ = (call);                                                                \
        if (s_ != CDLGB_OK) return s_;                                                  \
    } while (0)

// launch bookkeeping: checks the launch error of the kernel just issued
int cdlgb_after_launch(cdlgb_ctx* c, const char* what);
#define LAUNCH_CHECK(c, what) ST_TRY(cdlgb_after_launch((c), (what)))

// phase timers
void cdlgb_phase_begin(cdlgb_ctx* c, int ph);
void cdlgb_phase_end(cdlgb_ctx* c, int ph);
void cdlgb_phase_end_n(cdlgb_ctx* c, int ph, int units);   // interval covering `units` steps

// ---- devmem.cpp: stream-ordered device memory of a context (its device's pool, its
// stream) and pinned host scalars ----
cudaError_t dev_malloc(cdlgb_ctx* c, void** p, size_t bytes);
cudaError_t dev_copy_in(cdlgb_ctx* c, void** p, const void* host, size_t bytes);   // alloc + copy
int dev_alloc(cdlgb_ctx* c, void** p, size_t bytes);      // dev_malloc with the error recorded
void dev_free(cdlgb_ctx* c, void* p);
size_t devmem_reusable(int dev);          // reserved by the pool and not in use
int devmem_hold(int dev, int delta);      // > 0 holds: the pool keeps what is freed
double* host_scalars_get();               // 8 pinned doubles, nullptr when none is left
void host_scalars_put(double* p);

// ---- admm.cu ----
int admm_alloc(cdlgb_ctx* c);
void admm_free(cdlgb_ctx* c);
int admm_init(cdlgb_ctx* c, const float* X0, const float* D0, uint64_t seed);
int admm_code_update(cdlgb_ctx* c, int iters);
int admm_dict_update(cdlgb_ctx* c, int iters);
int admm_objective(cdlgb_ctx* c, double* obj);      // synchronous: result on host
int admm_update_best(cdlgb_ctx* c, double* obj, int* improved);
int admm_code_threshold(cdlgb_ctx* c, double* thr);
size_t admm_footprint(const cdlgb_params* p, int L4, int N, int fused);
int cdlgb_set_plan_streams(cdlgb_ctx* c);

// ---- fused.cu ----
int fused_supported(int Lg, int M, int L4);
int iter_variant_fits(int Lg, int M, int L4);
int fused_setup(cdlgb_ctx* c);
void fused_free(cdlgb_ctx* c);
int fused_xstep(cdlgb_ctx* c, const float* Xin, float* Xout, int accum_abs);
int fused_absx(cdlgb_ctx* c, const double** part, int* n);
size_t fused_scratch_bytes(int Lg, int M, int N);

// ---- xwarp.cu (register-FFT variant of the fused X-step) ----
void* warp_plan_create(cdlgb_ctx* c, int* status);
void warp_plan_free(cdlgb_ctx* c, void* p);
int warp_xstep(cdlgb_ctx* c, void* p, const float* Xin, float* Xout);
int warp_absx(void* p, const double** part, int* n);
int warp_variant_exists(int Lg, int M);
// multi-iteration fused X-step (xiter.cu): all iterations of one code update per launch
void* iter_plan_create(cdlgb_ctx* c, int* status);
void iter_plan_free(cdlgb_ctx* c, void* p);
int iter_xsteps(cdlgb_ctx* c, void* p, const float* Xin, float* Xout, int iters);
int iter_absx(void* p, const double** part, int* n);
int iter_plan_cluster(void* p);
int iter_plan_filters(void* p);
int iter_plan_grid(void* p);
void* iter_plan_create_nth(cdlgb_ctx* c, int nth, int want_cs, int* status);
int iter_xsteps_n(cdlgb_ctx* c, void* p, const float* Xin, float* Xout, int iters, int Nlim);
int warp_xstep_n(cdlgb_ctx* c, void* p, const float* Xin, float* Xout, int Nlim);
int warp_plan_cluster(void* p);
int warp_plan_filters(void* p);
int fused_autotune(cdlgb_ctx* c, int maxc, double* ms, int32_t* kind, int32_t* cs, int32_t* mc,
                   int32_t* n_out, int32_t* chosen);
int fused_has_multi(cdlgb_ctx* c);
// api.cu: FASTA text -> one byte per base (the reference's parsing rules), and a load
// from those bytes
#include <vector>
int fasta_codes(const char* text, size_t nbytes, int32_t max_entries, std::vector<uint8_t>& codes,
                int32_t* N, int32_t* L, int32_t* wrong, char* err, size_t errlen);
int load_codes(cdlgb_ctx* c, const uint8_t* codes, int32_t L, int32_t N);
// resid.cu: residual norms and the stopping test
size_t resid_part_doubles(int N, int F, int slots);
int resid_finish(cdlgb_ctx* c);
int resid_x_from_parts(cdlgb_ctx* c, const double* part, int nb);
int resid_x_from_arrays(cdlgb_ctx* c, const float* X);
int resid_d_from_spec_parts(cdlgb_ctx* c, int nb);
int resid_d_from_arrays(cdlgb_ctx* c);
int resid_td(cdlgb_ctx* c);
int resid_save_G(cdlgb_ctx* c);
int resid_dual_and_finish(cdlgb_ctx* c);
int iter_resid(void* p, const double** part, int* n);
int fused_resid(cdlgb_ctx* c, const double** part, int* n);
// noalloc.cu: scratch lookup of the allocation-free objective on the current device
int noalloc_warm_current_device();
// streaming forward transforms of the D-step (dstream.cu)
void* dfwd_plan_create(cdlgb_ctx* c, int* status);
void dfwd_plan_free(cdlgb_ctx* c, void* p);
int dfwd_run(cdlgb_ctx* c, void* p, const float* X, int n0, int cn, float2* Yh, float2* Hh, float2* Dh);
int dinv_run(cdlgb_ctx* c, void* p, const float2* Dh, int n0, int cn, float scale);
// batched R2C / C2R of R contiguous rows on the register FFT (cuFFT's layouts and
// scaling); two rows share a transform only inside a group of grp consecutive rows
int rows_r2c(cdlgb_ctx* c, void* p, long R, const float* in, float2* out, int grp);
int rows_c2r(cdlgb_ctx* c, void* p, long R, const float2* in, float* out, int grp);
void* fused_dfwd(cdlgb_ctx* c);
int fused_xsteps(cdlgb_ctx* c, const float* Xin, float* Xout, int iters);

// a scan-family scratch buffer of at least n elements (reallocated when too small)
template <typename T>
inline int ensure_scratch(cdlgb_ctx* c, T** p, size_t* cap, size_t n) {
    if (*cap >= n) return CDLGB_OK;
    dev_free(c, *p);
    *p = nullptr;
    *cap = 0;
    ST_TRY(dev_alloc(c, (void**)p, n * sizeof(T)));
    *cap = n;
    return CDLGB_OK;
}
// The first entry i of pos (n-major, k fastest: K entries per sequence, 1-based, 0 =
// none) that is negative or, with lens, whose window of lens[k] bases leaves a sequence
// of L bases (without lens: that exceeds L); -1 when every entry is valid.  A
// branch-free pass over all entries first (the compiler vectorises it), the search for
// the index only when that pass finds one.
inline long long first_bad_position(const int32_t* pos, const int32_t* lens, int K, size_t N, int L) {
    int bad = 0;
    for (size_t n = 0; n < N; ++n) {
        const int32_t* pr = pos + n * (size_t)K;
        for (int k = 0; k < K; ++k) {
            const int p = pr[k];
            const int lim = lens ? L + 1 - lens[k] : L;
            bad |= (p < 0) | ((p > 0) & (p > lim));
        }
    }
    if (!bad) return -1;
    for (size_t i = 0; i < N * (size_t)K; ++i) {
        const int p = pos[i];
        const int lim = lens ? L + 1 - lens[i % K] : L;
        if (p < 0 || (p > 0 && p > lim)) return (long long)i;
    }
    return -1;
}
// ---- scan.cu ----
int scan_fwd(cdlgb_ctx* c, const float* pwms, const int32_t* lens, const float* thresh,
             int K, int maxlen, int32_t* pos_out);
int scan_both(cdlgb_ctx* c, const float* pwms, const int32_t* lens, const float* thresh,
              int K, int maxlen, int32_t* pos_out, float* score_out, uint8_t* comp_out);
int count_pfms(cdlgb_ctx* c, const int32_t* pos, const uint8_t* use_comp,
               const int32_t* lens, int K, int maxlen, int32_t* counts_out, int32_t* nseq_out);
int nonoverlap_select(cdlgb_ctx* c, int32_t* pos, float* score, uint8_t* use_comp,
                      const int32_t* lens, int K);
int touzet_thresholds(cdlgb_ctx* c, const float* pwms, const int32_t* lens, int K, int maxlen,
                      double pval, float* thresh_out);
void scan_free(cdlgb_ctx* c);
// ---- dspec.cu ----
int dspec_max_m();
size_t dspec_part_bytes(int M, int F, int slots);
int dspec_nsub(int cn, int F, int nsm);
int dspec_slots(int N, int chunk, int F, int nsm);
int dspec_launch(cdlgb_ctx* c, const float2* Yh, const float2* G3h, int c0, int c1, int slot0);
int dspec_sums(cdlgb_ctx* c, const float2* G3h, float2* out);
int dspec_g3(cdlgb_ctx* c, float2* dst, const float2* g1h, size_t rows);
int dspec_bcast(cdlgb_ctx* c, float2* dst, const float2* plane);
int dspec_scale(cdlgb_ctx* c, float* x, size_t n, float s);
int admm_sync_time_state(cdlgb_ctx* c);
// ---- background.cu ----
int make_background(cdlgb_ctx* c, int k, unsigned long long seed);
// the one-hot data the scans, counts and motif refinement read
static inline const float* scan_data(const cdlgb_ctx* c) { return c->use_bg ? c->S_bg : c->S; }
// ---- refine.cu ----
int extend_positions(cdlgb_ctx* c, int32_t* pos, const uint8_t* use_comp, int32_t* lens, int K,
                     const float* bg, float pseudocount, float perc_no_less_than,
                     float ic_extension_thresh, int32_t* dec_out, int32_t* inc_out);
int rescore_positions(cdlgb_ctx* c, const float* pwms, const int32_t* pos, const int32_t* lens,
                      int K, int maxlen, float* score_out);

static inline unsigned grid_for(size_t n, int block, unsigned cap = 152u * 32u) {
    size_t g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (unsigned)g;
}
