/*
 * cdlgb.h -- C ABI of libcdlgb, the GB300 (sm_103a) implementation of the
 * CDLmotif.jl convolutional-dictionary-learning hot path: the Fourier-domain ADMM
 * (sparse-coding X-step, consensus dictionary D-step, best-iterate tracking) and
 * the PWM scan / count stage that follows it.
 *
 * Conventions
 *   - Plain pointers and sizes only.  Host arrays are caller-owned and use the
 *     reference's Julia column-major layouts, so a Julia `ccall` can pass its
 *     arrays as they are: "(a, b, c) col-major" means element (i, j, k) (0-based)
 *     sits at i + a*(j + b*k).
 *   - Device memory is owned by the library (one context = one dataset's ADMM
 *     state, resident in HBM until cdlgb_destroy).
 *   - Every call returns a cdlgb_status; 0 = OK, negative = error, with the
 *     message available from cdlgb_last_error(ctx).  A failure with no handle to
 *     hold its message (cdlgb_create, cdlgb_ar_create, cdlgb_server_create,
 *     cdlgb_objective_noalloc) leaves it for the calling thread: the *_last_error
 *     call given a null handle returns it.  The library prints nothing, no call
 *     aborts the process and no kernel traps.
 *   - A context is used by one host thread at a time and owns its own CUDA stream.
 *
 * Reference interfaces replaced (paths within kchu25/CDLmotif.jl):
 *   cdl ctor / init_cdl ............ src/SETUP/CDL_setup.jl:165-283
 *   code_update! ................... src/CDL/train.jl:1-44
 *   dict_update! ................... src/CDL/train.jl:46-89
 *   update_best! ................... src/CDL/train.jl:91-98
 *   objective ...................... src/SETUP/CDL_setup.jl:286
 *   cdl_optimize inner loop ........ src/WRAPPER/wrap.jl:6-11
 *   std(X_best[X_best .> 0]) ....... src/WRAPPER/wrap.jl:12
 *   scan_w_gpu! / greedy_search! ... src/SEARCH/scan.jl:176-239
 *   overlapping_scan! / scan_n ..... src/SEARCH/scan.jl:10-21, 89-121
 *   posdicts2pfms (counts) ......... src/SEARCH/helpers.jl:59-96
 *   save_pfms_as_transfac .......... src/SAVE/save_learned_results.jl:184-217
 */
#ifndef CDLGB_H
#define CDLGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cdlgb_ctx cdlgb_ctx;
typedef struct cdlgb_ar cdlgb_ar;      /* activation record (code -> counts stage) */

typedef enum {
    CDLGB_OK = 0,
    CDLGB_EINVAL = -1,          /* bad argument or size */
    CDLGB_ENOMEM_BUDGET = -2,   /* dataset does not fit the HBM budget (admission) */
    CDLGB_ECUDA = -3,           /* a CUDA / cuFFT call failed */
    CDLGB_ETIMEOUT = -4,        /* a bounded device wait gave up */
    CDLGB_ESTATE = -5,          /* call out of order (e.g. no data loaded) */
    CDLGB_ENOTSUP = -6          /* size or option not supported by this build */
} cdlgb_status;

/* Hyper-parameters: the fields of CDL_setup (src/SETUP/WRAPPER_setup.jl:1-13). */
typedef struct {
    int32_t M;                  /* number of filters (default 10) */
    int32_t filter_size;        /* bases per filter; filter length = 4*filter_size (default 4) */
    float rho;                  /* CSC penalty (default 100) */
    float sigma;                /* CDL penalty (default 100) */
    float lambda;               /* sparsity weight (default 0.01) */
    int32_t csc_iter_num;       /* X-steps per outer iteration (default 15) */
    int32_t cdl_iter_num;       /* D-steps per outer iteration (default 1) */
    int32_t iter_num;           /* outer iterations (default 10) */
    float std_threshold_multiplier; /* code threshold = multiplier * std (default 1) */
    float sherman_const_csc;    /* code_update! keyword (default 2) */
    float sherman_const_cdl;    /* dict_update! keyword (default 2) */
    int32_t device;             /* CUDA device ordinal (default 0) */
    int32_t init_mode;          /* D0 == NULL: 0 = random normal, unit norm per filter;
                                   1 = the reference's simplex-per-base draw */
    int32_t fft_mode;           /* 0 = auto (fused in-kernel FFT path where the size is
                                   supported, else cuFFT transforms), 1 = cuFFT, 2 = fused */
    uint64_t hbm_budget_bytes;  /* 0 = free device memory minus a 1 GiB margin */
    float stop_tol;             /* stopping test of cdlgb_run_outer (no counterpart in the
                                   reference, whose loop count is fixed, wrap.jl:6-11):
                                   0 = off (default: iter_num iterations, as the
                                   reference); > 0 = stop after the first outer iteration
                                   whose largest relative residual (CDLGB_FIELD_RESIDUALS
                                   entry 18) is <= stop_tol */
    int32_t track_residuals;    /* 1 = keep the residual record (CDLGB_FIELD_RESIDUALS) up to
                                   date after every code update and D-step; implied by
                                   stop_tol > 0; 0 (default) = not computed (the record
                                   stays zero), as the reference computes none */
} cdlgb_params;

/* Fields readable with cdlgb_get (sizes in elements; all float32 unless noted). */
typedef enum {
    CDLGB_FIELD_X = 0,          /* (Lg, M, N) col-major */
    CDLGB_FIELD_X_BEST = 1,     /* (Lg, M, N) */
    CDLGB_FIELD_D = 2,          /* consensus copies d, (Lg, M, N) */
    CDLGB_FIELD_D_BEST = 3,     /* (Lg, M) */
    CDLGB_FIELD_G1 = 4,         /* (Lg, M) */
    CDLGB_FIELD_G3 = 5,         /* (Lg, M) */
    CDLGB_FIELD_DX = 6,         /* (Lg, N) */
    CDLGB_FIELD_Y1 = 7,         /* (Lg, N) */
    CDLGB_FIELD_Y2_DUAL = 8,    /* y2, (Lg, M, N) */
    CDLGB_FIELD_Y3_DUAL = 9,    /* y3, (Lg, M, N) */
    CDLGB_FIELD_G1_DUAL = 10,   /* g1, (Lg, M, N) */
    CDLGB_FIELD_G3_DUAL = 11,   /* g3, (Lg, M, N) */
    CDLGB_FIELD_TD = 12,        /* (Lg, N) */
    CDLGB_FIELD_G2 = 13,        /* (Lg, N) */
    CDLGB_FIELD_G2_DUAL = 14,   /* g2, (Lg, N) */
    CDLGB_FIELD_Y1_DUAL = 15,   /* y1, (Lg, N) */
    CDLGB_FIELD_OBJ_BEST = 16,  /* one float64 */
    CDLGB_FIELD_DATA = 17,      /* the loaded one-hot data, (4L, N) float32 */
    CDLGB_FIELD_BACKGROUND = 18, /* the shuffled background (cdlgb_make_background), (4L, N) float32 */
    CDLGB_FIELD_RESIDUALS = 19, /* the residual record, 19 float64 (below) */
    CDLGB_FIELD_OUTER_DONE = 20 /* one int32: outer iterations run by the last cdlgb_run_outer */
} cdlgb_field;

/* The residual record (CDLGB_FIELD_RESIDUALS), float64 sums accumulated on the GPU.
 * The reference computes no residual; these follow its dual updates.  After every code
 * update, the primal residuals of its final iterate -- the vectors the next dual
 * updates of code_update! (src/CDL/train.jl:12-14) would add:
 *   [0] sum (X - shrink(X + y2))^2   [1] sum (X - projectionX(X + y3))^2
 *   [2] sum (DX - Y1)^2              [3] sum X^2            [4] sum DX^2
 * after every D-step, the increments its dual updates (train.jl:70-72) added and the
 * change of the consensus dictionary (the D-step's dual residual over sigma):
 *   [5] sum (d - G1_old)^2   [6] sum (d - G3_old)^2   [7] sum (Td - G2)^2
 *   [8] sum d^2              [9] sum Td^2
 *   [10] N sum (G1 - G1_old)^2   [11] N sum (G3 - G3_old)^2   [12] N (sum G1^2 + sum G3^2)
 * and the relative residuals of the stopping test:
 *   [13] sqrt(([0] + [1]) / [3])   [14] sqrt([2] / [4])   [15] sqrt(([5] + [6]) / (2 [8]))
 *   [16] sqrt([7] / [9])           [17] sqrt(([10] + [11]) / [12])   [18] max of [13..17]
 * Sums over d use the spectral state through Parseval's relation where the D-step keeps
 * it.  All zero after cdlgb_init_state, and kept up to date only when
 * params.track_residuals = 1 or params.stop_tol > 0. */

/* Fill *p with the CDL_setup defaults. */
int cdlgb_params_default(cdlgb_params* p);

/* Create a context on p->device.  Replaces nothing by itself: the reference has no
 * handle; its state is the `cdl` struct built by init_cdl. */
int cdlgb_create(const cdlgb_params* p, cdlgb_ctx** out);
int cdlgb_destroy(cdlgb_ctx* ctx);
/* The context's last error message; with ctx = NULL, the calling thread's last failure
 * that had no handle (a failed cdlgb_create, ...), or "null context". */
const char* cdlgb_last_error(const cdlgb_ctx* ctx);

/* Device memory a dataset of N sequences x L bases needs, for admission control.  Where
 * the D-step keeps d, g1, g3 as half-spectra (the default for M <= 128), their
 * time-domain copies (3 x 4 Lg M N bytes) are allocated only when first read through
 * cdlgb_get and are not counted here. */
int cdlgb_footprint(const cdlgb_params* p, int32_t L, int32_t N, uint64_t* bytes);

/* Upload the one-hot data matrix (4L, N) col-major (dna2dummy layout,
 * src/LOAD/to_dummy.jl:29-38; the reference's data_matrix_gpu).  Allocates the ADMM
 * state; fails with CDLGB_ENOMEM_BUDGET if it does not fit. */
int cdlgb_load_data(cdlgb_ctx* ctx, const float* onehot, int32_t L4, int32_t N);

/* read_fasta + data_2_dummy (src/LOAD/read.jl:2-28, src/LOAD/to_dummy.jl:27-38) into
 * the context: the FASTA text is split into '>'-records, each record's header line is
 * dropped and its remaining lines joined; records containing 'N' or 'n' are dropped;
 * the first max_entries (the reference's max_num_read_fasta is 10000) are upper-cased
 * and one-hot encoded on the device from one byte per base.  Records whose length
 * differs from the first one's are zero columns (the reference leaves them
 * uninitialised) and are counted in *n_wrong_len.  A character other than ACGTacgt ->
 * CDLGB_EINVAL (the reference raises a KeyError).  Afterwards the context is loaded as
 * by cdlgb_load_data with 4L = 4 *L_out and N = *N_out.  Output pointers may be NULL. */
int cdlgb_load_fasta(cdlgb_ctx* ctx, const char* text, size_t nbytes, int32_t max_entries,
                     int32_t* N_out, int32_t* L_out, int32_t* n_wrong_len);

/* Dimensions of the loaded problem: L4 = 4L, gamma = 4*filter_size, Lg = L4 + 2*gamma. */
int cdlgb_dims(const cdlgb_ctx* ctx, int32_t* L4, int32_t* N, int32_t* M,
               int32_t* gamma, int32_t* Lg);

/* init_cdl (src/SETUP/CDL_setup.jl:165-283).  X0: (Lg, M, N) col-major or NULL
 * (standard normal from `seed`); D0: (Lg, M) or NULL (per init_mode, from `seed`).
 * X0 is masked to rows (l-1) % 4 == 0 and D0 to the filter support, as the
 * constructor does.  Computes DX, the auxiliaries and obj_best. */
int cdlgb_init_state(cdlgb_ctx* ctx, const float* X0, const float* D0, uint64_t seed);

/* code_update!(c, num_iter) -- src/CDL/train.jl:1-44. */
int cdlgb_code_update(cdlgb_ctx* ctx, int32_t num_iter);

/* dict_update!(c, num_iter) -- src/CDL/train.jl:46-89. */
int cdlgb_dict_update(cdlgb_ctx* ctx, int32_t num_iter);

/* objective(c, S) -- src/SETUP/CDL_setup.jl:286, accumulated in float64 on the GPU. */
int cdlgb_objective(cdlgb_ctx* ctx, double* obj);

/* update_best!(c, S) -- src/CDL/train.jl:91-98.  *improved (may be NULL) = 1 when
 * X_best / D_best were replaced. */
int cdlgb_update_best(cdlgb_ctx* ctx, double* obj, int32_t* improved);

/* iter_num passes of cdl_optimize's loop body (src/WRAPPER/wrap.jl:6-11):
 * code_update!(csc_iter_num); update_best!; dict_update!(cdl_iter_num).
 * objs (may be NULL) receives the objective values, one per pass run.  With
 * params.stop_tol > 0 the loop ends early after the first pass whose largest relative
 * residual is <= stop_tol; CDLGB_FIELD_OUTER_DONE then tells how many passes ran. */
int cdlgb_run_outer(cdlgb_ctx* ctx, int32_t iter_num, double* objs);

/* std(X_best[X_best .> 0]) * multiplier -- src/WRAPPER/wrap.jl:12 (float64 on the GPU). */
int cdlgb_code_threshold(cdlgb_ctx* ctx, double* thresh);

/* Copy a state field to host memory; bytes must equal the field's size. */
int cdlgb_get(cdlgb_ctx* ctx, int32_t field, void* host_dst, size_t bytes);

/* scan_w_gpu! + greedy_search! (src/SEARCH/scan.jl:176-239) on the loaded data.
 * pwms: (K, 4, maxlen) col-major, zero-padded past lens[k]; thresh: K.
 * pos_out: (K, N) col-major, int32, 1-based argmax position of the thresholded
 * forward-strand score, 0 = not found (a best hit at position 1 also reads 0,
 * as in the reference).  Scores are summed in float32 in the reference's order. */
int cdlgb_scan_fwd(cdlgb_ctx* ctx, const float* pwms, const int32_t* lens,
                   const float* thresh, int32_t K, int32_t maxlen, int32_t* pos_out);

/* overlapping_scan! (src/SEARCH/scan.jl:89-121, scan_n :10-21): both strands, the
 * complement being `reverse(pwm)`.  pwms as above.  Outputs (K, N) col-major:
 * pos_out 1-based (0 = no score above thresh[k]), score_out, use_comp_out (1 when
 * the reverse complement won).  Any output pointer may be NULL. */
int cdlgb_scan_both(cdlgb_ctx* ctx, const float* pwms, const int32_t* lens,
                    const float* thresh, int32_t K, int32_t maxlen, int32_t* pos_out,
                    float* score_out, uint8_t* use_comp_out);

/* Autotuner (no counterpart in the reference): times every fused X-step variant that
 * fits this context's Lg and M -- the multi-iteration kernel with each choice of
 * filters per CTA (hence cluster size), then the one-X-step kernel -- with CUDA events
 * on a prefix of the loaded sequences, restoring that prefix's state after each run,
 * and keeps the fastest for the following code updates.  Per candidate i <
 * *n_candidates: ms_per_xstep[i], kind[i] (1 multi-iteration, 2 one X-step),
 * cluster[i] (CTAs per cluster), filters[i] (filters per CTA); *chosen = the winner.
 * Needs an initialised state and the fused path (CDLGB_ENOTSUP otherwise). */
int cdlgb_autotune(cdlgb_ctx* ctx, int32_t max_candidates, double* ms_per_xstep, int32_t* kind,
                   int32_t* cluster, int32_t* filters, int32_t* n_candidates, int32_t* chosen);

/* get_thresh (src/SEARCH/helpers.jl:99) = Float32(pvalue2score(pwm, pval)) for each of
 * the K PWMs (src/SEARCH/PWM_Touzet.jl:199-217: granularity 0.1, flat background),
 * batched on the device.  The rounded PWM entries are exact multiples of the Float64
 * 0.1 and the background probabilities powers of two, so the score distribution is
 * computed exactly as integer counts; the result equals the reference's Double64 one.
 * pwms as for the scans, (K, 4, maxlen) col-major; lens[k] in 1..31; pval in [0, 1].
 * thresh_out: K float32.  CDLGB_ENOTSUP when a PWM's rounded score range exceeds 6144
 * steps of 0.1. */
int cdlgb_pvalue_thresholds(cdlgb_ctx* ctx, const float* pwms, const int32_t* lens,
                            int32_t K, int32_t maxlen, double pval, float* thresh_out);

/* non_overlap_scan!'s selection (src/SEARCH/scan.jl:123-174; with use_comp NULL also
 * non_overlapping_scan_bg!, :48-87), in place on host arrays in the layout of
 * cdlgb_scan_both's outputs, (K, N) col-major: per sequence the entries are taken in
 * decreasing score (first maximum on ties; missing and taken entries count as score 0)
 * until the largest is 0, and an entry is kept when its span [pos, pos + lens[k] - 1]
 * meets no kept span; entries not kept get pos 0, score 0, use_comp 0.  (Replaces the
 * host loop; the background scans of overlapping_scan_bg!, :23-46, are
 * cdlgb_scan_both on a context loaded with the background data.) */
int cdlgb_select_nonoverlapping(cdlgb_ctx* ctx, int32_t* pos, float* score,
                                uint8_t* use_comp, const int32_t* lens, int32_t K);

/* The count matrices behind posdicts2pfms (src/SEARCH/helpers.jl:59-96): for each
 * motif k, the sum of the one-hot windows of length lens[k] at pos[k,n] (1-based,
 * 0 = none), reverse-complemented where use_comp[k,n] != 0 (use_comp may be NULL).
 * counts_out: (4, maxlen, K) col-major int32; nseq_out: K int32 (may be NULL). */
int cdlgb_count_pfms(cdlgb_ctx* ctx, const int32_t* pos, const uint8_t* use_comp,
                     const int32_t* lens, int32_t K, int32_t maxlen,
                     int32_t* counts_out, int32_t* nseq_out);

/* posdicts2pfms's normalisation (src/SEARCH/helpers.jl:66,87-88) in float32:
 * ps = pseudocounts_r*n when smoothing, else (less_pseudocount ? 0.1 : pseudo_count);
 * pfm = (count + ps) / (n + 4 ps).  pfm_out: (4, maxlen, K) col-major. Host only. */
int cdlgb_counts_to_pfms(const int32_t* counts, const int32_t* nseq, const int32_t* lens,
                         int32_t K, int32_t maxlen, float pseudocounts_r,
                         float pseudo_count, int32_t smoothing, int32_t less_pseudocount,
                         float* pfm_out);

/* extension! of extend! (src/SEARCH/extend.jl:31-81 without use_comp, 122-173 with it)
 * for K motifs at once: starting from each motif's positions, add a column on the left
 * and one on the right while the column's information content (its one-hot counts over
 * the motif's sequences plus `pseudocount`, against bg[4]) stays above
 * ic_extension_thresh; a sequence whose new column would leave 1..L is dropped when
 * that column is accepted.  pos: (K, N) col-major, 1-based, 0 = no entry, updated in
 * place (dropped entries become 0, the rest move to the new start); use_comp (K, N) or
 * NULL (the variant without complements); lens: K, updated in place (+ columns added).
 * dec_out / inc_out (K, may be NULL): columns added on the left / right.  Errors:
 * CDLGB_EINVAL where the reference would not return (a motif whose empty column keeps
 * scoring above the threshold) or would raise (a reverse-complemented column that is not
 * one-hot). */
int cdlgb_extend_positions(cdlgb_ctx* ctx, int32_t* pos, const uint8_t* use_comp, int32_t* lens,
                           int32_t K, const float* bg, float pseudocount, float perc_no_less_than,
                           float ic_extension_thresh, int32_t* dec_out, int32_t* inc_out);

/* scores_reevaluation (src/SEARCH/helpers.jl:151-172): score_out[k, n] = the Float32 sum
 * of pwm_k .* the forward one-hot window at pos[k, n] (the reference ignores use_comp
 * here), summed base-major, nucleotide inner; 0 where pos is 0.  pwms (K, 4, maxlen)
 * col-major as for the scans; pos and score_out (K, N) col-major. */
int cdlgb_rescore_positions(cdlgb_ctx* ctx, const float* pwms, const int32_t* pos,
                            const int32_t* lens, int32_t K, int32_t maxlen, float* score_out);

/* trim_this_pfm_by_masking! (src/SEARCH/trim.jl:1-36) for K pfms (4, maxlen, K) col-major
 * of lengths lens: the per-column information content against bg[4] (Float32, as
 * get_ic_col_multiple), then for each of the nmask masks the window starts from the
 * front and window ends from the back whose median IC is below mask_thresh[m] are
 * marked until the first window that is not; front_out[k] / back_out[k] = the leading /
 * trailing marked columns (the trimmed pfm is columns front+1 .. lens-back).  Host only. */
int cdlgb_trim_pfms(const float* pfms, const int32_t* lens, int32_t K, int32_t maxlen,
                    const float* bg, const int32_t* mask_len, const float* mask_thresh,
                    int32_t nmask, int32_t* front_out, int32_t* back_out);

/* The background data of the e-value filter.  The reference shuffles its FASTA file
 * with MEME's `fasta-shuffle-letters -kmer 3` (src/SETUP/LOAD_setup.jl:5-14), an external
 * program.  This replaces it on the device: every loaded sequence is shuffled keeping its
 * length, its first and last (k-1)-mers and the count of every k-mer (Euler-path shuffle,
 * Altschul & Erickson, with Wilson's random arborescence; splitmix64 numbers keyed by
 * (seed, sequence), so the result is reproducible).  A column with no base is a fifth
 * symbol.  k in 1..4 (the reference uses 3).  The result stays on the device next to
 * the data; read it with cdlgb_get(CDLGB_FIELD_BACKGROUND). */
int cdlgb_make_background(cdlgb_ctx* ctx, int32_t k, uint64_t seed);

/* Which one-hot matrix the scans (cdlgb_scan_fwd / _both), cdlgb_count_pfms,
 * cdlgb_extend_positions and cdlgb_rescore_positions read: 0 = the loaded data (the
 * default; reset by every load), 1 = the background.  The ADMM always reads the data.
 * The reference scans its background through the same scan functions
 * (src/SEARCH/e_value_filter.jl:2-13). */
int cdlgb_select_data(cdlgb_ctx* ctx, int32_t which);

/* filter_using_evalue!'s e-values (src/SEARCH/e_value_filter.jl:15-23): for motif k with
 * a = hits[k] sequences hit in the data and b = hits_bg[k] in the background (both out
 * of N), evalues_out[k] = K * pvalue(FisherExactTest(a, N, b, N)), the two-sided
 * "central" p-value min(1, 2 min(P(X <= a), P(X >= a))) of X ~ Hypergeometric(a + N
 * successes, b + N failures, a + b draws) (HypothesisTests 0.10.10 over Distributions
 * 0.25.54), in double precision.  Host only. */
int cdlgb_fisher_evalues(const int32_t* hits, const int32_t* hits_bg, int32_t K, int32_t N,
                         double* evalues_out);

/* One transfac file body as save_pfms_as_transfac writes it
 * (src/SAVE/save_learned_results.jl:186-196): pfm (4, w) col-major, values printed
 * as pfm*1000 in Julia's shortest Float32 form.  reverse_complement != 0 writes the
 * `_c` variant (reverse(pfm)).  Returns the byte count needed (excluding the NUL);
 * writes at most cap bytes including a NUL.  Host only. */
int64_t cdlgb_transfac_format(const float* pfm, int32_t w, int32_t reverse_complement,
                              char* out, size_t cap);

/* ---- Code -> activations -> filter-pair topology -> pair count matrices. ----
 * The activation record (activation_record, src/SETUP/SEARCH_setup.jl:6-57) holds, on
 * the device, the codes of T trainings (X_best rows gamma+1:4:gamma+4L) and their
 * thresholds; filter k = (training, m) for every filter with an activation. */
int cdlgb_ar_create(int32_t N, int32_t L, int32_t M, int32_t T, int32_t device, cdlgb_ar** out);
int cdlgb_ar_destroy(cdlgb_ar* ar);
/* ar = NULL: the calling thread's last failure without a handle (cdlgb_ar_create, ...). */
const char* cdlgb_ar_last_error(const cdlgb_ar* ar);

/* record_training_result! (src/SEARCH/store.jl:1-40): codes of ctx's X_best, activations
 * codes > thresh (thresh > 0, e.g. from cdlgb_code_threshold); appends the filters with
 * any activation (uinds) as filters of training train_num (1-based) with length
 * filter_size bases.  *added (may be NULL) = the number appended. */
int cdlgb_ar_record(cdlgb_ar* ar, cdlgb_ctx* ctx, double thresh, int32_t train_num,
                    int32_t filter_size, int32_t* added);

/* The record's filters: K, and per filter (arrays of >= cap entries, may be NULL) the
 * 1-based filter index within its training, the training number and the length. */
int cdlgb_ar_info(const cdlgb_ar* ar, int32_t* K, int32_t* uinds, int32_t* training_num,
                  int32_t* filter_lengths, int32_t cap);

/* get_spatial_info! / topology_at_nth_pt! (src/SEARCH/store.jl:64-144), cover_starts = 1:
 * integer counts over all sequences of ordered pairs of activations of filters from
 * different trainings.  over (K, K, maxlen), non_over (K, K, L - minlen - 1),
 * next_to (K, K), col-major int32, indexed [fr, fc, distance]. */
int cdlgb_ar_topology(cdlgb_ar* ar, int32_t* over, int32_t* non_over, int32_t* next_to);

/* get_pair_pfms! (src/SEARCH/extractions.jl:18-114) for the given pairs (P, 3) row-major
 * (fr, fc, overlap) 1-based (the reference selects overlap counts > count_threshold in
 * findall order): code-weighted one-hot MSAs summed over sequences, + 0.1 in the span,
 * normalised by the first column.  ctx holds the data.  pfms (P, 4, 2*filter_size-1)
 * col-major float32, span_lens (P). */
int cdlgb_ar_pair_pfms(cdlgb_ar* ar, cdlgb_ctx* ctx, const int32_t* pairs, int32_t P,
                       int32_t filter_size, float* pfms, int32_t* span_lens);

/* ---- Instrumentation and stream control.  No counterpart in the reference, which
 * times phases with `@time` only (src/WRAPPER/wrap.jl:30,52,54,67,80,100,137). ---- */

/* Run the context's work on an existing CUDA stream (cudaStream_t passed as void*),
 * e.g. CUDA.jl's task stream; NULL returns to a stream owned by the context. */
int cdlgb_set_stream(cdlgb_ctx* ctx, void* cuda_stream);

/* Enable per-phase CUDA-event timers (X-step, D-step, objective, fused kernels, data
 * upload + state initialisation, code threshold, scan). */
int cdlgb_profile(cdlgb_ctx* ctx, int32_t enable);

/* Read the accumulated phase times: ms[8], counts[8] (order: X-step, D-step,
 * objective, fused X kernel, set-up (the data upload's copy and kernels, and
 * cdlgb_init_state), code threshold, scan, reserved),
 * the number of this library's kernel launches and of cuFFT executions. */
int cdlgb_profile_read(cdlgb_ctx* ctx, double* ms, int64_t* counts, int64_t* launches,
                       int64_t* fft_calls, int32_t reset);

/* ---- Allocation-free objective.  No counterpart in the reference. ----
 * objective (src/SETUP/CDL_setup.jl:286's formula, 0.5*||W*DX - S||^2 + lambda*sum|X|)
 * of caller-owned DEVICE buffers X (Lg, M, N) col-major, DX (Lg, N), S (4L, N), with
 * Lg = L4 + 2*gamma, accumulated in float64; the value is written to *obj (host).
 * It calls no cudaMalloc / cudaFree: for callers whose device memory belongs to their
 * own allocator (e.g. a CUDA.jl memory pool holding the free memory, or a serving loop
 * with a fixed budget).  Its scratch is a static 1 MiB device array: at most 65536
 * sequences (larger N returns CDLGB_EINVAL before any GPU work); every call shares it,
 * so calls that overlap on the GPU race; the first call on a device looks up the
 * array's address and should come before any stream capture.  CUDA loads modules
 * lazily by default, so the array is only backed by device memory at that lookup:
 * make the first call (or a cdlgb_create on that device, which does the lookup as a
 * warm-up) before a memory pool takes the free memory, or set
 * CUDA_MODULE_LOADING=EAGER.  sum |X| is widened to float64 per element.
 * stream: cudaStream_t or NULL (legacy default stream). */
int cdlgb_objective_noalloc(const float* X, const float* DX, const float* S, int32_t L4,
                            int32_t N, int32_t M, int32_t gamma, float lambda, double* obj,
                            void* stream);

/* ---- Training server: continuous batching of many datasets on one GPU. ----
 * Replaces the reference's sequential loop over datasets, find_motifs_fasta_folder
 * (src/CDLmotif.jl:84-93), each trained by cdl_optimize (src/WRAPPER/wrap.jl:1-32).
 * Requests are submitted from any host thread at any time and admitted in arrival order
 * as soon as a slot is free and their device footprint (cdlgb_footprint) fits in what
 * the requests in flight leave of the HBM budget; each runs one training (init from
 * `seed`, iter_num outer iterations with the params' stopping test, the code threshold)
 * on its own context and stream, so kernels of different datasets overlap on the
 * device, and its ADMM state stays resident until the training ends.  Results do not
 * depend on what else is in flight.  All server calls are thread-safe. */
typedef struct cdlgb_server cdlgb_server;

typedef struct {
    int32_t slots;              /* trainings in flight at most (1..64) */
    int32_t device;             /* CUDA device ordinal */
    int32_t iter_num;           /* outer iterations per request; 0 = params.iter_num */
    int32_t keep_codes;         /* 1 = keep X_best of every finished request for fetch */
    int32_t pad_friendly;       /* 1 = pad each dataset's sequences with empty (all-zero)
                                   columns to the next length the register-FFT kernels
                                   cover (within 8 % more transform columns; else the next
                                   length whose transform factors into primes <= 31) */
    uint64_t hbm_budget_bytes;  /* 0 = 85 % of the device's free memory at creation */
    uint64_t seed;              /* initialisation seed of every request */
} cdlgb_server_config;

enum { CDLGB_REQ_PENDING = 0, CDLGB_REQ_RUNNING = 1, CDLGB_REQ_DONE = 2, CDLGB_REQ_FAILED = 3 };

typedef struct {
    int32_t state;              /* CDLGB_REQ_* */
    int32_t status;             /* the training's cdlgb_status when FAILED */
    int32_t N, L4, M, Lg;       /* dataset and transform sizes (M, Lg once done) */
    int32_t outer_done;         /* outer iterations run */
    uint64_t footprint_bytes;   /* device memory admitted for it */
    double obj_best;            /* best objective (float64) */
    double code_thresh;         /* std(X_best[X_best .> 0]) * multiplier (wrap.jl:12) */
    double t_submit, t_admit, t_done, t_now;   /* seconds on the server's clock; -1 = not yet */
    char error[256];            /* message when FAILED */
} cdlgb_request_info;

int cdlgb_server_create(const cdlgb_params* p, const cdlgb_server_config* cfg, cdlgb_server** out);
/* Copy a (4L, N) col-major one-hot dataset into the queue; *request_id identifies it.
 * CDLGB_ENOMEM_BUDGET when its footprint exceeds the whole budget (it can never run). */
int cdlgb_server_submit(cdlgb_server* s, const float* onehot, int32_t L4, int32_t N,
                        int64_t* request_id);
/* The same from FASTA text, parsed by cdlgb_load_fasta's rules (one byte per base is
 * kept until the request runs): the drop-in for one file of find_motifs_fasta_folder. */
int cdlgb_server_submit_fasta(cdlgb_server* s, const char* text, size_t nbytes,
                              int32_t max_entries, int64_t* request_id);
/* State of a request; wait_ms > 0 waits up to that long for it to finish, < 0 waits
 * until it does, 0 returns at once.  The result fields (status, M, Lg, outer_done,
 * obj_best, code_thresh, t_done, error) are filled once the request is done or
 * failed, and zero (t_done -1) before. */
int cdlgb_server_poll(cdlgb_server* s, int64_t request_id, int32_t wait_ms, cdlgb_request_info* info);
/* Copy a finished request's results: D_best (Lg, M) float32 (D_bytes = 4 Lg M), up to
 * objs_cap objectives, X_best (Lg, M, N) float32 when keep_codes; NULL skips one. */
int cdlgb_server_fetch(cdlgb_server* s, int64_t request_id, float* D_best, size_t D_bytes,
                       double* objs, int32_t objs_cap, float* X_best, size_t X_bytes);
/* Forget a finished request (its results are freed). */
int cdlgb_server_release(cdlgb_server* s, int64_t request_id);
/* Queue depth, trainings in flight, admitted bytes and the budget. */
int cdlgb_server_stats(cdlgb_server* s, int32_t* pending, int32_t* running, uint64_t* in_use,
                       uint64_t* budget);
/* The message of the server's last failed call, copied into a buffer of the calling
 * thread (valid until that thread's next call of this function); s = NULL: the calling
 * thread's last failure without a handle (cdlgb_server_create, ...). */
const char* cdlgb_server_last_error(const cdlgb_server* s);
/* Wait for the trainings in flight, drop the requests not yet admitted, free everything. */
int cdlgb_server_destroy(cdlgb_server* s);

#ifdef __cplusplus
}
#endif
#endif /* CDLGB_H */
