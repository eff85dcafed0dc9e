// The D-step's transforms (dict_update!, src/CDL/train.jl:52-62) as streaming kernels
// for the transform lengths with register-resident FFTs (regfft.cuh): k_dfwd (below)
// and the inverse k_dinv (further down, d = irfft(d-hat) per filter pair).
//
// For every (sequence n, filter pair a = 2s, b = 2s + 1) a lane group forms, straight
// from the state arrays, the three packed real pairs the D-step transforms --
//   Y3 = projectionX!(X + y3)                 (X + y3 on the rows l % 4 == 0, else 0)
//   H  = (G1 - g1) + (G3 - g3)                (the filter-domain terms of sherman_CDL_RHS!)
//   d  (the previous iterate)
// -- runs the four-step FFT on each and writes the split half-spectra (f = 0..Lg/2) of
// both filters where the per-frequency solve expects them, (n, m, f).  It replaces a
// pass that wrote Y3 and H to HBM and three cuFFT R2C transforms (each a complex FFT
// and a post-processing pass over the spectra).
//
// Host side: the lengths instantiated in dstream_v*.cu, the plan, the launches.
#include "dstream.cuh"

namespace dstream {
const Variant* variants_1(int* n);
const Variant* variants_2(int* n);
const Variant* variants_3(int* n);
const Variant* variants_4(int* n);
const Variant* variants_5(int* n);
const Variant* variants_6(int* n);
}  // namespace dstream

namespace {

using dstream::FArgs;
using dstream::IArgsD;
using dstream::Variant;
using dstream::kern_t;
using dstream::kinv_t;
using dstream::kr2c_t;
using dstream::kc2r_t;

const std::vector<Variant>& all_variants() {
    static const std::vector<Variant> all = [] {
        std::vector<Variant> v;
        for (auto f : {dstream::variants_1, dstream::variants_2, dstream::variants_3, dstream::variants_4,
                       dstream::variants_5, dstream::variants_6}) {
            int n = 0;
            const Variant* p = f(&n);
            v.insert(v.end(), p, p + n);
        }
        return v;
    }();
    return all;
}

struct FwdPlan {
    kern_t k;
    kinv_t ki;
    kr2c_t kf;
    kc2r_t kb;
    int N1, P;
    size_t smem;
    int grid, grid_inv, grid_rows_f, grid_rows_b;
    float2* tw2;
};

}  // namespace

// Returns nullptr when Lg has no register-FFT variant (or CDLGB_DSTREAM=0).
void* dfwd_plan_create(cdlgb_ctx* c, int* status) {
    *status = CDLGB_OK;
    if (const char* e = getenv("CDLGB_DSTREAM"))
        if (atoi(e) == 0) return nullptr;
    const Variant* v = nullptr;
    for (const Variant& cand : all_variants())
        if (cand.N1 * cand.P == c->Lg) v = &cand;
    if (!v) return nullptr;
    FwdPlan* P = new FwdPlan();
    P->k = v->k; P->ki = v->ki; P->kf = v->kf; P->kb = v->kb; P->N1 = v->N1; P->P = v->P;
    const int threads = 256, groups = (threads / 32) * (32 / v->N1);
    const size_t buf = ((size_t)v->P * (v->N1 + 1) + 1) & ~(size_t)1;
    P->smem = ((size_t)v->P * v->N1 + (size_t)groups * buf) * sizeof(float2);
    std::vector<float2> tw2 = regfft_twiddles(v->N1, v->P);
    cudaError_t e = v->tables();
    if (e == cudaSuccess) e = dev_copy_in(c, (void**)&P->tw2, tw2.data(), tw2.size() * sizeof(float2));
    if (e == cudaSuccess) e = cudaFuncSetAttribute(P->k, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(P->ki, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(P->kf, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(P->kb, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
    int per_sm = 0, per_sm_inv = 0, per_sm_f = 0, per_sm_b = 0;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, P->k, threads, P->smem);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_inv, P->ki, threads, P->smem);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_f, P->kf, threads, P->smem);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_b, P->kb, threads, P->smem);
    if (e != cudaSuccess || per_sm < 1 || per_sm_inv < 1 || per_sm_f < 1 || per_sm_b < 1) {
        *status = cdlgb_seterr(c, CDLGB_ECUDA, "D-step transform setup failed: %s",
                               e != cudaSuccess ? cudaGetErrorString(e) : "no CTA fits");
        dev_free(c, P->tw2);
        delete P;
        return nullptr;
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    P->grid = per_sm * sms;
    P->grid_inv = per_sm_inv * sms;
    P->grid_rows_f = per_sm_f * sms;
    P->grid_rows_b = per_sm_b * sms;
    return P;
}

void dfwd_plan_free(cdlgb_ctx* c, void* p) {
    FwdPlan* P = (FwdPlan*)p;
    if (!P) return;
    dev_free(c, P->tw2);
    delete P;
}

// Y3-hat, H-hat and d-hat of sequences [n0, n0 + cn) into Yh, Hh, Dh (chunk layout); a
// null Hh or Dh skips that transform.
int dfwd_run(cdlgb_ctx* c, void* p, const float* X, int n0, int cn, float2* Yh, float2* Hh, float2* Dh) {
    FwdPlan* P = (FwdPlan*)p;
    const size_t off = (size_t)n0 * c->M * c->Lg;
    FArgs a;
    // g1, g3, d are read only for H-hat and d-hat (the time-domain D-step, where they exist)
    a.X = X + off; a.y3 = c->y3 + off;
    a.g1 = c->g1 ? c->g1 + off : nullptr;
    a.g3 = c->g3 ? c->g3 + off : nullptr;
    a.d = c->d ? c->d + off : nullptr;
    a.G1 = c->G1; a.G3 = c->G3; a.Yh = Yh; a.Hh = Hh; a.Dh = Dh; a.tw2 = P->tw2;
    a.cn = cn; a.M = c->M;
    P->k<<<P->grid, 256, P->smem, c->stream>>>(a);
    LAUNCH_CHECK(c, "k_dfwd");
    return CDLGB_OK;
}

// d of sequences [n0, n0 + cn) from the half-spectra Dh (chunk layout), as C2R would.
int dinv_run(cdlgb_ctx* c, void* p, const float2* Dh, int n0, int cn, float scale) {
    FwdPlan* P = (FwdPlan*)p;
    IArgsD a;
    a.Dh = Dh; a.d = c->d + (size_t)n0 * c->M * c->Lg; a.tw2 = P->tw2; a.cn = cn; a.M = c->M;
    a.scale = scale;
    P->ki<<<P->grid_inv, 256, P->smem, c->stream>>>(a);
    LAUNCH_CHECK(c, "k_dinv");
    return CDLGB_OK;
}

// R2C / C2R of R contiguous rows with the register FFT (the cuFFT batched plans' layouts)
static unsigned rows_grid(long R, int grp, int cap, int N1) {
    const long lane_groups = (256 / 32) * (32 / N1);
    const long items = (R / grp) * ((grp + 1) / 2);
    const long need = (items + lane_groups - 1) / lane_groups;
    return (unsigned)(need < cap ? (need > 0 ? need : 1) : cap);
}

int rows_r2c(cdlgb_ctx* c, void* p, long R, const float* in, float2* out, int grp) {
    FwdPlan* P = (FwdPlan*)p;
    if (grp < 1 || R % grp)
        return cdlgb_seterr(c, CDLGB_EINVAL, "row transform: %ld rows in groups of %d", R, grp);
    P->kf<<<rows_grid(R, grp, P->grid_rows_f, P->N1), 256, P->smem, c->stream>>>(in, out, P->tw2, R, grp);
    LAUNCH_CHECK(c, "k_rows_r2c");
    return CDLGB_OK;
}

int rows_c2r(cdlgb_ctx* c, void* p, long R, const float2* in, float* out, int grp) {
    FwdPlan* P = (FwdPlan*)p;
    if (grp < 1 || R % grp)
        return cdlgb_seterr(c, CDLGB_EINVAL, "row transform: %ld rows in groups of %d", R, grp);
    P->kb<<<rows_grid(R, grp, P->grid_rows_b, P->N1), 256, P->smem, c->stream>>>(in, out, P->tw2, R, grp);
    LAUNCH_CHECK(c, "k_rows_c2r");
    return CDLGB_OK;
}
