/* A plain C host of the library's C ABI (include/cdlgb.h), used the way a Julia
 * `ccall` shim or any other non-Python caller would use it: no Python, no torch.
 *
 *   abi_driver cpu   host-only calls (defaults, count normalisation, transfac text,
 *                    Fisher e-values, trimming); prints their results
 *   abi_driver gpu   one training on a small deterministic dataset (create, load,
 *                    init from a seed, run_outer, code threshold, D_best, residual
 *                    record) and a two-strand scan; prints every value in hex-float
 *                    form so the caller can compare bit for bit
 * Exit code 0 on success; on a failed call it prints the library's message. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "cdlgb.h"

#define CHECK(ctx, call)                                                              \
    do {                                                                              \
        int st_ = (call);                                                             \
        if (st_ != CDLGB_OK) {                                                        \
            fprintf(stderr, "%s -> %d: %s\n", #call, st_, (ctx) ? cdlgb_last_error(ctx) : ""); \
            return 1;                                                                 \
        }                                                                             \
    } while (0)

static uint32_t lcg(uint32_t* s) { *s = *s * 1664525u + 1013904223u; return *s >> 8; }

static int run_cpu(void) {
    cdlgb_params p;
    if (cdlgb_params_default(&p) != CDLGB_OK) return 1;
    printf("defaults %d %d %a %a %a %d %d %d\n", p.M, p.filter_size, p.rho, p.sigma, p.lambda,
           p.csc_iter_num, p.cdl_iter_num, p.iter_num);
    /* counts (4, 3, 1) of 10 sequences -> PFM with the fixed pseudocount 5 */
    const int32_t counts[12] = {7, 1, 1, 1, 0, 10, 0, 0, 2, 2, 3, 3};
    const int32_t nseq[1] = {10}, lens[1] = {3};
    float pfm[12];
    if (cdlgb_counts_to_pfms(counts, nseq, lens, 1, 3, 0.0295f, 5.f, 0, 0, pfm) != CDLGB_OK) return 1;
    printf("pfm");
    for (int i = 0; i < 12; ++i) printf(" %a", pfm[i]);
    printf("\n");
    char buf[4096];
    const int64_t n = cdlgb_transfac_format(pfm, 3, 0, buf, sizeof(buf));
    if (n < 0 || n >= (int64_t)sizeof(buf)) return 1;
    printf("transfac %lld\n%s", (long long)n, buf);
    const int32_t hits[2] = {40, 3}, hits_bg[2] = {5, 3};
    double ev[2];
    if (cdlgb_fisher_evalues(hits, hits_bg, 2, 100, ev) != CDLGB_OK) return 1;
    printf("evalues %a %a\n", ev[0], ev[1]);
    return 0;
}

static int run_gpu(void) {
    const int N = 24, L = 40, M = 4, fs = 3;
    cdlgb_params p;
    cdlgb_params_default(&p);
    p.M = M; p.filter_size = fs; p.rho = 1.f; p.sigma = 100.f; p.lambda = 0.1f;
    p.track_residuals = 1;
    cdlgb_ctx* c = NULL;
    CHECK(NULL, cdlgb_create(&p, &c));
    /* (4L, N) column-major one-hot from a fixed generator */
    float* S = calloc((size_t)4 * L * N, sizeof(float));
    uint32_t s = 12345u;
    for (int n = 0; n < N; ++n)
        for (int l = 0; l < L; ++l) S[(size_t)n * 4 * L + 4 * l + (lcg(&s) & 3u)] = 1.f;
    CHECK(c, cdlgb_load_data(c, S, 4 * L, N));
    CHECK(c, cdlgb_init_state(c, NULL, NULL, 7));
    double objs[3];
    CHECK(c, cdlgb_run_outer(c, 3, objs));
    double th = 0;
    CHECK(c, cdlgb_code_threshold(c, &th));
    int32_t L4, Nn, Mm, g, Lg;
    CHECK(c, cdlgb_dims(c, &L4, &Nn, &Mm, &g, &Lg));
    float* Db = malloc((size_t)Lg * M * sizeof(float));
    CHECK(c, cdlgb_get(c, CDLGB_FIELD_D_BEST, Db, (size_t)Lg * M * sizeof(float)));
    double res[19];
    CHECK(c, cdlgb_get(c, CDLGB_FIELD_RESIDUALS, res, sizeof(res)));
    printf("objs %a %a %a\nthresh %a\nLg %d\n", objs[0], objs[1], objs[2], th, Lg);
    printf("D_best");
    for (int i = 0; i < Lg * M; ++i) printf(" %a", Db[i]);
    printf("\nresiduals");
    for (int i = 0; i < 19; ++i) printf(" %a", res[i]);
    printf("\n");
    /* a two-strand scan with one PWM of width 5: (K=1, 4, 5) */
    float pwm[20];
    for (int i = 0; i < 20; ++i) pwm[i] = (float)((int)(lcg(&s) % 21) - 10) / 4.f;
    const int32_t lens[1] = {5};
    const float thresh[1] = {0.5f};
    int32_t pos[24];
    float score[24];
    uint8_t comp[24];
    CHECK(c, cdlgb_scan_both(c, pwm, lens, thresh, 1, 5, pos, score, comp));
    printf("scan");
    for (int n = 0; n < N; ++n) printf(" %d:%a:%d", pos[n], score[n], comp[n]);
    printf("\n");
    CHECK(c, cdlgb_destroy(c));
    free(S);
    free(Db);
    return 0;
}

int main(int argc, char** argv) {
    if (argc > 1 && strcmp(argv[1], "gpu") == 0) return run_gpu();
    return run_cpu();
}
