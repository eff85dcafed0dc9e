"""GPU parity of the PWM scans and count matrices: bit-exact against the oracle
(same PWMs and thresholds -> identical positions, float32 scores, strands, integer
counts and PFMs)."""
import os

import numpy as np
import pytest

from oracle import search_oracle as SO

from conftest import random_onehot

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _ctx(pkg, S):
    c = pkg.CDL(pkg.CDLSetup(M=2, filter_size=2))
    c.load_data(S)
    return c


def _random_pwms(rng, K, lo, hi):
    lens = rng.integers(lo, hi, K).astype(np.int32)
    pwms = []
    for w in lens:
        pfm = rng.dirichlet(0.4 * np.ones(4), size=int(w)).T
        pfm = (pfm + 0.02) / 1.08
        pwms.append(np.log2(pfm / 0.25).astype(np.float32))
    thresh = np.array([0.3 * np.sum(np.max(p, axis=0)) for p in pwms], np.float32)
    return pwms, lens, thresh


def _pad(pwms, lens):
    K, maxlen = len(lens), int(max(lens))
    pw = np.zeros((K, 4, maxlen), np.float32)
    for k in range(K):
        pw[k, :, : lens[k]] = pwms[k][:, : lens[k]]
    return pw


def test_golden_scan(pkg, built_lib):
    g = np.load(os.path.join(GOLD, "scan_small.npz"))
    lens = g["lens"]
    pwms = [g["pwms"][k, :, : lens[k]] for k in range(len(lens))]
    with _ctx(pkg, g["S"]) as c:
        pos_fwd = pkg.scan_w_gpu(c, pwms, g["thresh"])
        np.testing.assert_array_equal(pos_fwd.T, g["pos_fwd"])
        pos, score, comp = pkg.overlapping_scan(c, pwms, g["thresh"])
        np.testing.assert_array_equal(pos.T, g["pos"])
        np.testing.assert_array_equal(score.T, g["score"])
        np.testing.assert_array_equal(comp.T, g["comp"])
        counts, nseq = pkg.count_matrices(c, pos, lens, comp)
        np.testing.assert_array_equal(counts, g["counts"])
        np.testing.assert_array_equal(nseq, g["nseq"])
        pfms = pkg.posdicts2pfms(c, pos, lens, comp)
        for k in range(len(lens)):
            np.testing.assert_array_equal(pfms[k], g["pfms"][k, :, : lens[k]])


@pytest.mark.parametrize("dense", [False, True])
@pytest.mark.parametrize("N,L,K", [(300, 200, 8), (64, 100, 20), (7, 31, 3)])
def test_scans_bit_exact_random(pkg, built_lib, N, L, K, dense, monkeypatch):
    """Both the sparse sums (the default on one-hot data with finite PWMs: only the
    terms whose entry is 1, in the reference's order) and the dense ones."""
    if dense:
        monkeypatch.setenv("CDLGB_SCAN_DENSE", "1")
    rng = np.random.default_rng(N + L + K)
    S, _ = random_onehot(rng, N, L)
    pwms, lens, thresh = _random_pwms(rng, K, 4, 21)
    with _ctx(pkg, S) as c:
        pos_fwd = pkg.scan_w_gpu(c, pwms, thresh)
        ref_fwd = SO.scan_w_gpu_positions(_pad(pwms, lens), S, lens, thresh)
        np.testing.assert_array_equal(pos_fwd.T, ref_fwd)
        pos, score, comp = pkg.overlapping_scan(c, pwms, thresh)
        rp, rs, rc = SO.overlapping_scan(S, pwms, lens, thresh)
        np.testing.assert_array_equal(pos.T, rp)
        np.testing.assert_array_equal(score.T, rs)
        np.testing.assert_array_equal(comp.T, rc)
        counts, nseq = pkg.count_matrices(c, pos, lens, comp)
        rcnt, rn = SO.count_matrices(S, rp, rc, lens)
        np.testing.assert_array_equal(counts, rcnt)
        np.testing.assert_array_equal(nseq, rn)


@pytest.mark.parametrize("N,L,K,lo,hi", [(3, 1100, 3, 4, 21), (4, 40, 300, 20, 32)])
def test_two_strand_scan_unstaged_sizes(pkg, built_lib, N, L, K, lo, hi):
    """The sizes the staged two-strand kernel does not take (more than 1024 positions,
    more than 64 KB of staged PWMs) run the unstaged kernel: bit-exact too."""
    rng = np.random.default_rng(N * L + K)
    S, _ = random_onehot(rng, N, L)
    pwms, lens, thresh = _random_pwms(rng, K, lo, hi)
    with _ctx(pkg, S) as c:
        pos, score, comp = pkg.overlapping_scan(c, pwms, thresh)
        rp, rs, rc = SO.overlapping_scan(S, pwms, lens, thresh)
        np.testing.assert_array_equal(pos.T, rp)
        np.testing.assert_array_equal(score.T, rs)
        np.testing.assert_array_equal(comp.T, rc)


def test_scan_edge_cases(pkg, built_lib):
    rng = np.random.default_rng(3)
    N, L = 12, 9
    S, _ = random_onehot(rng, N, L)
    pwms = [np.log2(rng.dirichlet(np.ones(4), size=w).T / 0.25 + 1e-3).astype(np.float32)
            for w in (12, 9, 1, 4)]                      # longer than L, == L, width 1
    lens = np.array([12, 9, 1, 4], np.int32)
    for thresh in (np.array([0, 0, 0, 0], np.float32), np.array([-50, -50, -50, -50], np.float32),
                   np.array([1e9] * 4, np.float32)):
        with _ctx(pkg, S) as c:
            pos_fwd = pkg.scan_w_gpu(c, pwms, thresh)
            np.testing.assert_array_equal(pos_fwd.T, SO.scan_w_gpu_positions(_pad(pwms, lens), S, lens, thresh))
            pos, score, comp = pkg.overlapping_scan(c, pwms, thresh)
            rp, rs, rc = SO.overlapping_scan(S, pwms, lens, thresh)
            np.testing.assert_array_equal(pos.T, rp)
            np.testing.assert_array_equal(score.T, rs)
            np.testing.assert_array_equal(comp.T, rc)


def test_scan_ties_first_position(pkg, built_lib):
    """Repeated motif occurrences: equal scores resolve to the first position, and a
    best hit at position 1 reads 0 in scan_w_gpu (scan.jl:197)."""
    L = 20
    seq = "ACGTACGTACGTACGTACGT"
    S = np.zeros((2, 4 * L), np.float32)
    for i, ch in enumerate(seq):
        S[0, 4 * i + "ACGT".index(ch)] = 1
    for i, ch in enumerate("TT" + seq[:-2]):
        S[1, 4 * i + "ACGT".index(ch)] = 1
    pwm = np.full((4, 4), -1.0, np.float32)
    for i, ch in enumerate("ACGT"):
        pwm["ACGT".index(ch), i] = 1.0
    th = np.array([0.5], np.float32)
    with _ctx(pkg, S) as c:
        pos = pkg.scan_w_gpu(c, [pwm], th)
        assert pos[0, 0] == 0 and pos[1, 0] == 3
        p2, s2, c2 = pkg.overlapping_scan(c, [pwm], th)
        rp, rs, rc = SO.overlapping_scan(S, [pwm], [4], th)
        np.testing.assert_array_equal(p2.T, rp)
        assert p2[0, 0] == 1


def test_count_rejects_out_of_range_window(pkg, built_lib):
    rng = np.random.default_rng(4)
    S, _ = random_onehot(rng, 3, 10)
    with _ctx(pkg, S) as c:
        pos = np.array([[8], [1], [0]], np.int32)     # window of 4 at base 8 leaves L=10
        with pytest.raises(pkg.CDLGBError) as e:
            pkg.count_matrices(c, pos, [4])
        assert e.value.status == -1


@pytest.mark.parametrize("K", [6, 40])
def test_non_overlap_scan_matches_oracle(pkg, built_lib, K):
    """non_overlap_scan! on the GPU against the oracle's restatement of the host loop,
    on the output of overlapping_scan (with and without use_comp): identical arrays."""
    rng = np.random.default_rng(17 + K)
    S, _ = random_onehot(rng, 300, 60)
    pwms, lens, thresh = _random_pwms(rng, K, 4, 12)
    with _ctx(pkg, S) as c:
        pos, score, comp = pkg.overlapping_scan(c, pwms, thresh)
        assert (pos > 0).sum() > 0
        p2, s2, c2 = pkg.non_overlap_scan(c, pos, score, lens, comp)
        rp, rs, rc = SO.non_overlap_select(pos, score, comp, lens)
        np.testing.assert_array_equal(p2, rp)
        np.testing.assert_array_equal(s2, rs)
        np.testing.assert_array_equal(c2, rc)
        assert (p2 > 0).sum() < (pos > 0).sum()          # overlaps were removed
        p3, s3, _ = pkg.non_overlap_scan(c, pos, score, lens)
        np.testing.assert_array_equal(p3, rp)
        np.testing.assert_array_equal(s3, rs)


@pytest.mark.parametrize("pval", [2.7e-4, 1e-3, 0.05])
def test_pvalue_thresholds_match_oracle(pkg, built_lib, pval):
    """get_thresh / pvalue2score (PWM_Touzet.jl:199-217) batched on the GPU with exact
    integer counts, against the exact-rational restatement: identical float32."""
    rng = np.random.default_rng(int(pval * 1e6) % 1000)
    pwms, lens, _ = _random_pwms(rng, 12, 3, 12)
    with _ctx(pkg, random_onehot(rng, 4, 30)[0]) as c:
        th = pkg.get_thresh(c, pwms, pval)
    ref = np.array([SO.pvalue2score(p, pval) for p in pwms], np.float32)
    np.testing.assert_array_equal(th, ref)


@pytest.mark.parametrize("bad", [-np.inf, np.inf, np.nan])
def test_scan_nonfinite_pwm_entries(pkg, built_lib, bad):
    """A PWM with a non-finite entry (log2 of a zero PFM entry is -Inf) takes the dense
    sums, where Inf * 0 is NaN as in the reference: results equal the oracle's."""
    rng = np.random.default_rng(12)
    N, L = 40, 60
    S, _ = random_onehot(rng, N, L)
    pwms, lens, thresh = _random_pwms(rng, 5, 4, 12)
    pwms[2] = pwms[2].copy()
    pwms[2][1, 0] = bad
    with _ctx(pkg, S) as c:
        pos_fwd = pkg.scan_w_gpu(c, pwms, thresh)
        np.testing.assert_array_equal(pos_fwd.T, SO.scan_w_gpu_positions(_pad(pwms, lens), S, lens, thresh))
        pos, score, comp = pkg.overlapping_scan(c, pwms, thresh)
        rp, rs, rc = SO.overlapping_scan(S, pwms, lens, thresh)
        np.testing.assert_array_equal(pos.T, rp)
        np.testing.assert_array_equal(score.T, rs)
        np.testing.assert_array_equal(comp.T, rc)


def test_scan_zero_columns(pkg, built_lib):
    """Sequences with empty columns (a record of the wrong length, or padding) score
    only their real bases: sparse and dense sums agree with the oracle."""
    rng = np.random.default_rng(13)
    N, L = 30, 80
    S, _ = random_onehot(rng, N, L)
    S[3] = 0.0
    S[5, 4 * 60:] = 0.0
    pwms, lens, thresh = _random_pwms(rng, 6, 4, 20)
    with _ctx(pkg, S) as c:
        pos_fwd = pkg.scan_w_gpu(c, pwms, thresh)
        np.testing.assert_array_equal(pos_fwd.T, SO.scan_w_gpu_positions(_pad(pwms, lens), S, lens, thresh))
        pos, score, comp = pkg.overlapping_scan(c, pwms, thresh)
        rp, rs, rc = SO.overlapping_scan(S, pwms, lens, thresh)
        np.testing.assert_array_equal(pos.T, rp)
        np.testing.assert_array_equal(score.T, rs)
        np.testing.assert_array_equal(comp.T, rc)


@pytest.mark.parametrize("lo,hi", [(1, 17), (9, 17), (12, 33), (30, 40)])
def test_sparse_scan_width_classes(pkg, built_lib, lo, hi):
    """Every sparse two-strand kernel -- packed 16-bit masks (PWMs of at most 16
    columns), 32-bit and 64-bit masks -- against the oracle, bit for bit."""
    rng = np.random.default_rng(lo * 100 + hi)
    N, L = 50, 150
    S, _ = random_onehot(rng, N, L)
    pwms, lens, thresh = _random_pwms(rng, 9, lo, hi)
    with _ctx(pkg, S) as c:
        pos, score, comp = pkg.overlapping_scan(c, pwms, thresh)
        rp, rs, rc = SO.overlapping_scan(S, pwms, lens, thresh)
        np.testing.assert_array_equal(pos.T, rp)
        np.testing.assert_array_equal(score.T, rs)
        np.testing.assert_array_equal(comp.T, rc)
