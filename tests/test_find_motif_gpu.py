"""End to end through the library, the way find_motif composes the hot path
(src/WRAPPER/wrap.jl:42-117, src/CDLmotif.jl:62-67): FASTA text -> cdlgb_load_fasta ->
two trainings (cdl_optimize, wrap.jl:1-32) -> record_training_result! ->
get_spatial_info! -> get_pair_pfms! -> PWMs and Touzet thresholds -> two refinement
rounds (overlapping_scan!, non_overlap_scan!, extend! with the PFM re-evaluation,
masked_trim!, wrap.jl:80-98) -> save_pfms_as_transfac's text
(src/SAVE/save_learned_results.jl:184-217).

Beside it the oracle's pipeline, stage by stage, from the same inputs: the data from
the oracle's FASTA reader; the trainings from the same initial states (FP64 oracle,
held to the float32 parity tolerance); every later stage from the GPU's outputs of the
stage before, where it must be bit-exact (the integer topology counts, pairs, spans,
positions, count matrices, PFMs, thresholds and the transfac bytes), except the pair
PFMs, float32 sums of code-weighted windows (1e-5)."""
import numpy as np
import pytest

from oracle import cdl_oracle as O
from oracle import search_oracle as SO

from conftest import rel

pytestmark = pytest.mark.gpu

TOL_X = 1e-4


def test_find_motif_pipeline_against_oracle(pkg, built_lib):
    synth = pkg.synth
    N, L, M, fs = 120, 48, 6, 3
    bases, _, _ = synth.plant_dataset(23, N, L, [7, 9], [0.7, 0.6])
    text = synth.to_fasta(bases).encode()
    setup = pkg.CDLSetup(M=M, filter_size=fs, lambda_=0.1, rho=1.0, sigma=100.0)
    Lg = 4 * L + 8 * fs
    gamma, L4 = 4 * fs, 4 * L

    # FASTA ingest (read_fasta + data_2_dummy)
    S_ref, _ = SO.read_fasta_onehot(text)
    ctxs, threshs, Xbs = [], [], []
    try:
        for t in range(2):
            c = pkg.CDL(setup)
            ctxs.append(c)
            info = c.load_fasta(text)
            assert (info["N"], info["L"], info["wrong_length"]) == (N, L, 0)
            np.testing.assert_array_equal(c.data(), S_ref)
            # one training of cdl_optimize from fixed initial states (3 outer iterations)
            X0 = synth.init_X0(50 + t, N, M, Lg)
            D0 = synth.init_D0_unit_norm(50 + t, M, Lg, 4 * fs)
            c.init_state(X0, D0)
            objs = pkg.run_outer(c, 3)
            ref = O.init_cdl(S_ref, M, fs, 1.0, 100.0, 0.1, X0=X0, D0=D0)
            np.testing.assert_allclose(objs, O.run_outer(ref, 3), rtol=1e-5)
            Xb = c.X_best
            assert rel(Xb, ref.X_best) < TOL_X
            th = pkg.code_threshold(c)
            assert th == pytest.approx(O.code_threshold(Xb), rel=1e-12)
            threshs.append(th)
            Xbs.append(Xb)

        with pkg.ActivationRecord(N, L, M, T=2) as ar:
            # record_training_result! and the filter-pair topology (integers)
            for t in range(2):
                pkg.record_training_result(ctxs[t], threshs[t], ar, t + 1, fs)
            u, tn, fl = ar.info()
            codes = np.stack([SO.record_codes(Xbs[t], gamma, L4) for t in range(2)])
            start_pos = np.stack([codes[tn[k] - 1][:, u[k] - 1, :] > np.float32(threshs[tn[k] - 1])
                                  for k in range(len(u))], axis=1)
            over, non_over, next_to = pkg.get_spatial_info(ar)
            ro, rn, rx = SO.activation_topology(start_pos, tn, fl, L)
            np.testing.assert_array_equal(over, ro)
            np.testing.assert_array_equal(non_over, rn)
            np.testing.assert_array_equal(next_to, rx)
            # get_pair_pfms! on the most frequent overlaps
            thr = int(np.percentile(over[over > 0], 80))
            pairs, spans, pfms = pkg.get_pair_pfms(ar, ctxs[0], over, thr, fs)
            rpairs, rspans, rpfms = SO.pair_msas(over, start_pos, fl, tn, u, codes, S_ref, thr, fs)
            assert [tuple(int(v) for v in p) for p in pairs] == rpairs and len(rpairs) > 0
            np.testing.assert_array_equal(spans, rspans)
            for a, b in zip(pfms, rpfms):
                np.testing.assert_allclose(a, b, rtol=1e-5, atol=1e-6)

        c = ctxs[0]
        pwms = [pkg.pfm2pwm(p) for p in pfms]
        thresh = pkg.get_thresh(c, pwms)
        np.testing.assert_array_equal(thresh, np.array([SO.pvalue2score(p, 2.7e-4) for p in pwms], np.float32))
        rounds = 0
        for _ in range(2):
            if not pwms:
                break
            lens = np.array([p.shape[1] for p in pwms], np.int32)
            # overlapping_scan! (both strands)
            pos, sc, uc = pkg.overlapping_scan(c, pwms, thresh)
            rp, rs, rc = SO.overlapping_scan(S_ref, pwms, lens, thresh)
            np.testing.assert_array_equal(pos, rp.T)
            np.testing.assert_array_equal(sc, rs.T)
            np.testing.assert_array_equal(uc, rc.T)
            # non_overlap_scan!
            pos, sc, uc = pkg.non_overlap_scan(c, pos, sc, lens, uc)
            rp2, rs2, rc2 = SO.non_overlap_select(rp.T, rs.T, rc.T, lens)
            np.testing.assert_array_equal(pos, rp2)
            np.testing.assert_array_equal(uc, rc2)
            # extend!: extension, then the PFMs re-evaluated from the new positions
            ext = pkg.extend(c, pos, lens, fs, use_comp=uc)
            npos, nl, _, _ = SO.extend_positions(S_ref, rp2, rc2, lens)
            keep = (npos > 0).any(axis=0) & (nl > fs + 2)
            np.testing.assert_array_equal(ext["keep"], keep)
            kept = np.flatnonzero(keep)
            np.testing.assert_array_equal(ext["positions"], npos[:, kept])
            np.testing.assert_array_equal(ext["lens"], nl[keep])
            if not len(kept):
                break
            counts, nseq = SO.count_matrices(S_ref, npos[:, kept].T, rc2[:, kept].T, nl[keep])
            rpf = SO.counts_to_pfms(counts, nseq, nl[keep])
            for a, b in zip(ext["pfms"], rpf):
                np.testing.assert_array_equal(a, b)
            # masked_trim! and the PWMs / thresholds of the next round
            tr = pkg.masked_trim(ext["pfms"], fs, ext["positions"], ext["use_comp"], c=c)
            fb = [SO.trim_pfm_by_masking(p) for p in rpf]
            np.testing.assert_array_equal(tr["front"], [f for f, _ in fb])
            np.testing.assert_array_equal(tr["back"], [b for _, b in fb])
            if not len(tr["pfms"]):
                break
            pwms, thresh = tr["pwms"], tr["thresh"]
            np.testing.assert_array_equal(thresh, np.array([SO.pvalue2score(p, 2.7e-4) for p in pwms],
                                                           np.float32))
            final_pfms = tr["pfms"]
            rounds += 1
        assert rounds >= 1
        # save_pfms_as_transfac's text, byte for byte
        for p in final_pfms:
            assert pkg.transfac_text(p) == SO.transfac_text(p)
            assert pkg.transfac_text(p, True) == SO.transfac_text(SO.pwm_complement(p))
    finally:
        for c in ctxs:
            c.close()
