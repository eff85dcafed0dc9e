"""GPU parity of the motif refinement: extension! (k_extend) and scores_reevaluation
(k_rescore) through the C ABI against the oracle, bit for bit (positions, lengths and
integer counts are exact; the IC decisions use the same Float32 operations)."""
import numpy as np
import pytest

from oracle import search_oracle as SO

from test_refine_cpu import kat_data

pytestmark = pytest.mark.gpu


def _ctx(pkg, S):
    c = pkg.CDL(pkg.CDLSetup(M=2, filter_size=2))
    c.load_data(S)
    return c


def test_extension_known_answers(pkg, built_lib):
    pos = np.array([1, 5, 5, 5, 5, 5], np.int32)[:, None]
    with _ctx(pkg, kat_data()) as c:
        new, ln, dec, inc = pkg.extension(c, pos, [3])
        assert (int(dec[0]), int(inc[0]), int(ln[0])) == (1, 0, 4)
        np.testing.assert_array_equal(new[:, 0], [0, 4, 4, 4, 4, 4])
        with pytest.raises(pkg.CDLGBError):
            pkg.extension(c, pos, [3], bg=(0.7, 0.1, 0.1, 0.1))   # the reference never returns
    with _ctx(pkg, kat_data(col3="CCCCC")) as c:
        new, ln, dec, inc = pkg.extension(c, pos, [3])
        assert (int(dec[0]), int(inc[0]), int(ln[0])) == (4, 0, 7)
        np.testing.assert_array_equal(new[:, 0], [0, 1, 1, 1, 1, 1])
    S = kat_data(comp_seq0=True)
    pos5 = np.full((6, 1), 5, np.int32)
    comp = np.array([1, 0, 0, 0, 0, 0], np.uint8)[:, None]
    with _ctx(pkg, S) as c:
        new, ln, dec, inc = pkg.extension(c, pos5, [3], comp)
        assert (int(dec[0]), int(inc[0]), int(ln[0])) == (1, 0, 4)
        np.testing.assert_array_equal(new[:, 0], [5, 4, 4, 4, 4, 4])
    S2 = S.copy()
    S2[0, 4 * 7:4 * 8] = 0.0
    with _ctx(pkg, S2) as c:
        with pytest.raises(pkg.CDLGBError):
            pkg.extension(c, pos5, [3], comp)                     # dummy_comp's KeyError


def _planted(pkg, seed, N, L):
    from cdlmotif_gb300 import synth
    bases, motifs, _ = synth.plant_dataset(seed, N, L, [12, 16, 9], [0.5, 0.35, 0.3])
    S = synth.onehot(bases)
    # scan with the middle of each motif so that the extension has columns to find
    pwms = []
    for m in motifs:
        core = m[:, 2:-2]
        pfm = ((core + 0.05) / 1.2).astype(np.float32)
        pwms.append(np.log2(pfm / np.float32(0.25)).astype(np.float32))
    thresh = np.array([0.55 * float(np.sum(np.max(p, axis=0))) for p in pwms], np.float32)
    return S, pwms, thresh


@pytest.mark.parametrize("seed,N,L", [(1, 400, 100), (2, 2000, 60), (3, 57, 31)])
@pytest.mark.parametrize("ic_thresh", [0.075, 0.6])
def test_extension_matches_oracle(pkg, built_lib, seed, N, L, ic_thresh):
    S, pwms, thresh = _planted(pkg, seed, N, L)
    with _ctx(pkg, S) as c:
        pos, score, comp = pkg.overlapping_scan(c, pwms, thresh)
        lens = np.array([p.shape[1] for p in pwms], np.int32)
        assert (pos > 0).sum() > 0
        for uc in (comp, None):
            new, ln, dec, inc = pkg.extension(c, pos, lens, uc, ic_extension_thresh=ic_thresh)
            rp, rl, rd, ri = SO.extend_positions(S, pos, uc, lens, ic_extension_thresh=ic_thresh)
            np.testing.assert_array_equal(new, rp)
            np.testing.assert_array_equal(ln, rl)
            np.testing.assert_array_equal(dec, rd)
            np.testing.assert_array_equal(inc, ri)
        # extend! as a whole: filter, then posdicts2pfms on the new positions
        out = pkg.extend(c, pos, lens, filter_size=4, use_comp=comp, ic_extension_thresh=ic_thresh)
        rp, rl, _, _ = SO.extend_positions(S, pos, comp, lens, ic_extension_thresh=ic_thresh)
        keep = ((rp > 0).sum(axis=0) > 0) & (rl > 4 + 2)
        np.testing.assert_array_equal(out["keep"], keep)
        if keep.any():
            cnt, ns = SO.count_matrices(S, rp[:, keep].T, comp[:, keep].T, rl[keep])
            ref = SO.counts_to_pfms(cnt, ns, rl[keep])
            for a, b in zip(out["pfms"], ref):
                np.testing.assert_array_equal(a, b)


def test_extension_moves_planted_motif_to_full_width(pkg, built_lib):
    """On a strongly planted motif scanned with its core only, the extension recovers
    columns on both sides."""
    S, pwms, thresh = _planted(pkg, 11, 3000, 80)
    with _ctx(pkg, S) as c:
        pos, score, comp = pkg.overlapping_scan(c, pwms, thresh)
        lens = np.array([p.shape[1] for p in pwms], np.int32)
        new, ln, dec, inc = pkg.extension(c, pos, lens, comp)
        assert int((ln - lens).max()) >= 2


@pytest.mark.parametrize("seed,N,L", [(4, 300, 100), (5, 33, 40)])
def test_rescore_matches_oracle(pkg, built_lib, seed, N, L):
    S, pwms, thresh = _planted(pkg, seed, N, L)
    with _ctx(pkg, S) as c:
        pos, score, comp = pkg.overlapping_scan(c, pwms, thresh)
        got = pkg.scores_reevaluation(c, pwms, pos)
        ref = SO.scores_reevaluation(S, pwms, pos, [p.shape[1] for p in pwms])
        np.testing.assert_array_equal(got, ref)
        # forward entries score as the scan scored them (same window, same order)
        fwd = (pos > 0) & (comp == 0)
        np.testing.assert_allclose(got[fwd], score[fwd], rtol=1e-5, atol=1e-5)
