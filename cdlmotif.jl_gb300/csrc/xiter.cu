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
// Host side: the variants instantiated in xiter_v*.cu, the plan, the launch.
#include "xiter.cuh"

namespace xiter {
const Variant* variants_1(int* n);
const Variant* variants_2(int* n);
const Variant* variants_3(int* n);
const Variant* variants_4(int* n);
const Variant* variants_5(int* n);
const Variant* variants_6(int* n);
const Variant* variants_7(int* n);
const Variant* variants_8(int* n);
}  // namespace xiter

namespace {

using xiter::Variant;
using xiter::kern_t;

constexpr size_t kCap2 = 115200;       // two CTAs per SM (2 x (this + 1 KB reserved) <= 228 KB)
constexpr size_t kCap1 = 220 * 1024;   // one CTA per SM

// in order of preference (measured at L=200, K=64: 16 filters per CTA, one CTA per SM,
// 6.7 ms per X-step; 8 filters per CTA, two CTAs per SM, 7.6 ms).  Lg = 16 P and 32 P
// for per-lane lengths P from 17 to 33 (Lg = 4L + 8W), listed in xiter_v*.cu.
const std::vector<Variant>& all_variants() {
    static const std::vector<Variant> all = [] {
        std::vector<Variant> v;
        for (auto f : {xiter::variants_1, xiter::variants_2, xiter::variants_3, xiter::variants_4,
                       xiter::variants_5, xiter::variants_6, xiter::variants_7, xiter::variants_8}) {
            int n = 0;
            const Variant* p = f(&n);
            v.insert(v.end(), p, p + n);
        }
        return v;
    }();
    return all;
}

// bytes of shared memory: slot buffers, P parts, twiddles, the interleaved y2 / y3
// pair rows (ld, ld3 pairs each), y1, A, the W'S window
size_t iter_smem(int N1, int P, int slots, int Mc, int ld, int ld3, int L4) {
    const int Lg = N1 * P, F = Lg / 2 + 1, Fp = (F + 1) & ~1;
    const size_t buf = ((size_t)P * (N1 + 1) + 1) & ~(size_t)1;
    return ((size_t)slots * buf + 2 * (size_t)Fp + (size_t)P * N1 +
            (size_t)(Mc / 2) * (ld + ld3)) * sizeof(float2) +
           ((size_t)Lg + Fp + L4) * sizeof(float);
}

// the static checks of a variant for Lg, M and the window length L4: its transform
// length, an even M (filters are transformed in pairs) on ceil(M / MC) <= 8 CTAs (exactly
// want_cs when that is set), and its shared memory
bool variant_fits(const Variant& v, int Lg, int M, int L4, int want_cs, int* cs, size_t* smem) {
    if (v.N1 * v.P != Lg || M < 2 || M % 2) return false;
    *cs = (M + v.MC - 1) / v.MC;
    if (*cs > 8 || (want_cs && *cs != want_cs)) return false;
    *smem = iter_smem(v.N1, v.P, (v.MC + 1) / 2 + 1, v.MC, Lg, 3 * v.N1 / 4 * v.P, L4);
    return *smem <= (v.minb == 2 ? kCap2 : kCap1);
}

bool xiter_off() {
    if (getenv("CDLGB_GENERIC_FFT")) return true;
    const char* e = getenv("CDLGB_XITER");
    return e && atoi(e) == 0;
}

int env_cluster() {
    const char* e = getenv("CDLGB_CLUSTER");
    return e ? atoi(e) : 0;
}

struct IterPlan {
    kern_t k, kr;
    int CS, Mc, ld, ld3, threads, grid;
    size_t smem;
    float2* tw2;
    double* absx_part;
    double* res_part;
};

}  // namespace

// The first variant (in all_variants() order) whose transform length is Lg, for an even M
// on ceil(M / filters per CTA) <= 8 CTAs (the last one may hold fewer real filters);
// CDLGB_CLUSTER forces a cluster size and CDLGB_XITER=0 turns the multi-iteration kernel
// off.  Returns nullptr when the size has no variant.
void* iter_plan_create(cdlgb_ctx* c, int* status) {
    *status = CDLGB_OK;
    if (xiter_off()) return nullptr;
    return iter_plan_create_nth(c, 0, env_cluster(), status);
}

// Whether iter_plan_create would find a variant for Lg, M and L4 (the checks that need
// no device: the cluster's occupancy is checked when the plan is made).
int iter_variant_fits(int Lg, int M, int L4) {
    if (xiter_off()) return 0;
    int cs = 0;
    size_t sm = 0;
    for (const Variant& v : all_variants())
        if (variant_fits(v, Lg, M, L4, env_cluster(), &cs, &sm)) return 1;
    return 0;
}

// The nth variant (in all_variants() order) that fits Lg and M, optionally only with
// cluster size want_cs; nullptr when there is none.
void* iter_plan_create_nth(cdlgb_ctx* c, int nth, int want_cs, int* status) {
    *status = CDLGB_OK;
    IterPlan* P = nullptr;
    const Variant* v = nullptr;
    for (const Variant& cand : all_variants()) {
        // the last CTA of a cluster may hold fewer than MC filters
        int cs = 0;
        size_t sm = 0;
        if (!variant_fits(cand, c->Lg, c->M, c->L4, want_cs, &cs, &sm)) continue;
        const int ld = c->Lg;
        const int ld3 = 3 * cand.N1 / 4 * cand.P;
        if (nth-- > 0) continue;
        v = &cand;
        P = new IterPlan();
        P->k = cand.k; P->kr = cand.kr; P->CS = cs; P->Mc = cand.MC; P->ld = ld; P->ld3 = ld3;
        P->threads = cand.threads; P->smem = sm;
        break;
    }
    if (!P) return nullptr;
    std::vector<float2> tw2 = regfft_twiddles(v->N1, v->P);
    cudaError_t e = v->tables();
    if (e == cudaSuccess) e = dev_copy_in(c, (void**)&P->tw2, tw2.data(), tw2.size() * sizeof(float2));
    // process-wide per kernel: the same cap for every context
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(P->k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(v->minb == 2 ? kCap2 : kCap1));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(P->kr, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(v->minb == 2 ? kCap2 : kCap1));
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
    if (e == cudaSuccess && nclusters >= 1) {
        if (nclusters > c->N) nclusters = c->N;
        P->grid = nclusters * P->CS;
        e = dev_malloc(c, (void**)&P->absx_part, (size_t)P->grid * sizeof(double));
        if (e == cudaSuccess) e = dev_malloc(c, (void**)&P->res_part, (size_t)P->grid * 5 * sizeof(double));
    }
    if (e != cudaSuccess || nclusters < 1) {
        *status = cdlgb_seterr(c, CDLGB_ECUDA, "multi-iteration X-step setup failed: %s",
                               e != cudaSuccess ? cudaGetErrorString(e) : "no cluster fits");
        dev_free(c, P->tw2);
        dev_free(c, P->absx_part);
        dev_free(c, P->res_part);
        delete P;
        return nullptr;
    }
    return P;
}

void iter_plan_free(cdlgb_ctx* c, void* p) {
    IterPlan* P = (IterPlan*)p;
    if (!P) return;
    dev_free(c, P->tw2);
    dev_free(c, P->absx_part);
    dev_free(c, P->res_part);
    delete P;
}

int iter_plan_cluster(void* p) { return p ? ((IterPlan*)p)->CS : 0; }
int iter_plan_filters(void* p) { return p ? ((IterPlan*)p)->Mc : 0; }
int iter_plan_grid(void* p) { return p ? ((IterPlan*)p)->grid : 0; }

int iter_xsteps(cdlgb_ctx* c, void* p, const float* Xin, float* Xout, int iters) {
    return iter_xsteps_n(c, p, Xin, Xout, iters, c->N);
}

// `iters` X-steps over the first Nlim sequences (the autotuner times on a prefix)
int iter_xsteps_n(cdlgb_ctx* c, void* p, const float* Xin, float* Xout, int iters, int Nlim) {
    IterPlan* P = (IterPlan*)p;
    IArgs a;
    a.Xin = Xin; a.Xout = Xout; a.y2 = c->y2; a.y3 = c->y3;
    a.Y1 = c->Y1; a.y1 = c->y1; a.DX = c->DX; a.S = c->S;
    a.G1h = c->G1h; a.Ah = c->Ah; a.tw2 = P->tw2; a.absx_part = P->absx_part;
    a.res_part = P->res_part;
    a.N = Nlim; a.M = c->M; a.L4 = c->L4; a.gamma = c->gamma; a.iters = iters;
    a.lam = c->p.lambda; a.rho = c->p.rho; a.kc = c->p.sherman_const_csc;
    a.ld = P->ld; a.ld3 = P->ld3;
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
    CU_TRY(c, cudaLaunchKernelEx(&cfg, c->res_on ? P->kr : P->k, a));
    LAUNCH_CHECK(c, "k_xiter");
    cdlgb_phase_end(c, PH_XFUSED);
    return CDLGB_OK;
}

int iter_absx(void* p, const double** part, int* n) {
    IterPlan* P = (IterPlan*)p;
    if (!P) return 0;
    *part = P->absx_part;
    *n = P->grid;
    return 1;
}

int iter_resid(void* p, const double** part, int* n) {
    IterPlan* P = (IterPlan*)p;
    if (!P) return 0;
    *part = P->res_part;
    *n = P->grid;
    return 1;
}
