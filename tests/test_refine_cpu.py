"""CPU tests of the motif-refinement oracle (extension! of extend!, the masking trim of
masked_trim!, scores_reevaluation) against hand-derived answers, and of the library's
host-side trim against the oracle."""
import numpy as np
import pytest

from oracle import search_oracle as SO

BASE = {"A": 0, "C": 1, "G": 2, "T": 3}


def onehot_rows(seqs):
    """list of equal-length ACGT strings -> (N, 4L) float32 one-hot."""
    L = len(seqs[0])
    out = np.zeros((len(seqs), L, 4), np.float32)
    for n, s in enumerate(seqs):
        for i, ch in enumerate(s):
            out[n, i, BASE[ch]] = 1.0
    return out.reshape(len(seqs), 4 * L)


def put(s, pos1, ch):
    """string s with base ch at 1-based position pos1."""
    return s[: pos1 - 1] + ch + s[pos1:]


# Six sequences of length 12.  Sequence 0 holds the motif (length 3) at position 1,
# sequences 1..5 at position 5; column 4 of sequences 1..5 is A, column 3 and column 8
# read A C G T A.
def kat_data(col3="ACGTA", comp_seq0=False):
    seqs = []
    s0 = "CCCCCCCCCCCC"
    if comp_seq0:
        # reverse-complemented entry at position 5: its left column is 8 (complemented),
        # its right column is 4 (complemented), its second left column is 9
        s0 = put(put(put(s0, 8, "T"), 4, "G"), 9, "A")
    else:
        s0 = put(s0, 4, "C")
    seqs.append(s0)
    for i in range(5):
        s = "GGGGGGGGGGGG"
        s = put(s, 4, "A")
        s = put(s, 3, col3[i])
        s = put(s, 8, "ACGTA"[i])
        seqs.append(s)
    return onehot_rows(seqs)


def test_ic_column_values():
    # (counts + 5) / (n + 20): (6,0,0,0) -> 0.1027 > 0.075; (5,0,0,0) -> 0.0781 > 0.075;
    # (2,1,1,1) -> 0.0034; (3,3,0,0) -> 0.0388
    def ic(c):
        c = np.asarray(c, np.float32)
        col = ((c + np.float32(5)) / np.float32(c.sum() + np.float32(20))).astype(np.float32)
        return float(SO.ic_col_single(col, (0.25,) * 4))
    assert ic([6, 0, 0, 0]) == pytest.approx(0.10274, abs=2e-5)
    assert ic([5, 0, 0, 0]) == pytest.approx(0.07807, abs=2e-5)
    assert ic([2, 1, 1, 1]) == pytest.approx(0.00339, abs=2e-5)
    assert ic([3, 3, 0, 0]) == pytest.approx(0.03876, abs=2e-5)
    assert ic([0, 0, 0, 0]) == 0.0


def test_extension_known_answer_with_exclusion():
    """Loop pass 1: left column 4 counts A x5 (sequence 0 has no column 0 and is dropped
    when the column is accepted): IC 0.078 > 0.075, dec = 1.  Right column 8 over the
    five remaining: (2,1,1,1), stop.  Pass 2: left column 3 (2,1,1,1), stop."""
    S = kat_data()
    pos = np.array([1, 5, 5, 5, 5, 5], np.int32)
    new, ln, dec, inc = SO.extension(S, pos, 3, None)
    assert (dec, inc, ln) == (1, 0, 4)
    np.testing.assert_array_equal(new, [0, 4, 4, 4, 4, 4])


def test_extension_usage_bound_never_fires():
    """Reference quirk: num_included is decremented only in explore_sides!'s copy, so
    after sequence 0 is dropped (5 of 6 left, usage bound floor(0.95 * 6) = 5) the loop
    still runs: column 3 = C x5 is accepted in pass 2 (dec = 2); column 2 (all G) is
    then scored (0,0,5,0): IC 0.078, accepted too; column 1 (all G) likewise, and the
    next left column is out of range for every sequence: the empty column scores 0."""
    S = kat_data(col3="CCCCC")
    pos = np.array([1, 5, 5, 5, 5, 5], np.int32)
    new, ln, dec, inc = SO.extension(S, pos, 3, None)
    assert (dec, inc, ln) == (4, 0, 7)
    np.testing.assert_array_equal(new, [0, 1, 1, 1, 1, 1])


def test_extension_known_answer_reverse_complement():
    """Sequence 0 is a reverse-complemented entry at position 5: its left column is 8
    (T, complemented A), so pass 1 left counts A x6 (IC 0.103), dec = 1; its right
    column is 4 (G -> C): (2,2,1,1), stop; pass 2 left: its column 9 (A -> T) with
    A C G T A: (2,1,1,2), stop.  New starts: p - dec forward, p - inc (= 5) complemented."""
    S = kat_data(comp_seq0=True)
    pos = np.array([5, 5, 5, 5, 5, 5], np.int32)
    comp = np.array([1, 0, 0, 0, 0, 0], np.uint8)
    new, ln, dec, inc = SO.extension(S, pos, 3, comp)
    assert (dec, inc, ln) == (1, 0, 4)
    np.testing.assert_array_equal(new, [5, 4, 4, 4, 4, 4])


def test_extension_no_entries_and_not_onehot():
    S = kat_data()
    new, ln, dec, inc = SO.extension(S, np.zeros(6, np.int32), 3, None)
    assert (dec, inc, ln) == (0, 0, 3)
    S2 = S.copy()
    S2[0, 4 * 7:4 * 8] = 0.0           # sequence 0's column 8 is no base
    with pytest.raises(KeyError):
        SO.extension(S2, np.array([5, 5, 5, 5, 5, 5], np.int32), 3,
                     np.array([1, 0, 0, 0, 0, 0], np.uint8))


def test_extension_endless_is_reported():
    """With a background far from flat the pseudocount-only column of an empty side
    scores above the threshold for ever (the reference does not return)."""
    S = kat_data()
    with pytest.raises(RuntimeError):
        SO.extension(S, np.array([1, 5, 5, 5, 5, 5], np.int32), 3, None,
                     bg=(0.7, 0.1, 0.1, 0.1))


def _ic_pfm(cols):
    return np.array(cols, np.float32).T


def test_trim_known_answers():
    u = [0.25, 0.25, 0.25, 0.25]
    h = [0.97, 0.01, 0.01, 0.01]
    # ic = [0, 0, h x6, 0, 0]: masks 8 and 4 stop at once, mask 2 marks columns 1 and
    # 10, mask 1 marks 2 and 9 -> trim 2 at each end
    assert SO.trim_pfm_by_masking(_ic_pfm([u, u] + [h] * 6 + [u, u])) == (2, 2)
    # ic = [0, .294, .294, h, h, h]: mask 4 marks column 1 (median .294), mask 2
    # column 2; column 3 (.294 >= .2) stays although window 2 covered it
    m = [0.55, 0.15, 0.15, 0.15]
    assert float(SO.ic_cols(_ic_pfm([m]))[0]) == pytest.approx(0.2940, abs=2e-4)
    assert SO.trim_pfm_by_masking(_ic_pfm([u, m, m, h, h, h])) == (2, 0)
    # nothing to trim; and a pfm shorter than every mask but 1
    assert SO.trim_pfm_by_masking(_ic_pfm([h] * 5)) == (0, 0)
    assert SO.trim_pfm_by_masking(_ic_pfm([u])) == (1, 1)


def test_scores_reevaluation_forward_window():
    S = kat_data()
    pw = np.arange(12, dtype=np.float32).reshape(3, 4).T * np.float32(0.5)   # (4, 3)
    pos = np.array([[1], [5], [5], [0], [5], [5]], np.int32)
    sc = SO.scores_reevaluation(S, [pw], pos, [3])
    # sequence 0 reads C C C at 1..3: rows C of columns 1..3 = 0.5, 2.5, 4.5
    assert sc[0, 0] == np.float32(7.5)
    # sequences 1.. read G G G at 5..7: 1 + 3 + 5
    assert sc[1, 0] == np.float32(9.0)
    assert sc[3, 0] == 0.0


def test_trim_c_matches_oracle(pkg, built_lib):
    rng = np.random.default_rng(7)
    pfms = []
    for _ in range(40):
        w = int(rng.integers(1, 25))
        alpha = rng.choice([0.2, 1.0, 20.0], size=w)
        cols = np.stack([rng.dirichlet(a * np.ones(4)) for a in alpha], axis=1)
        pfms.append(((cols + 0.01) / 1.04).astype(np.float32))
    front, back = pkg.trim_pfms(pfms)
    for k, p in enumerate(pfms):
        assert (int(front[k]), int(back[k])) == SO.trim_pfm_by_masking(p), k


def test_masked_trim_positions_and_filter(pkg, built_lib):
    u = [0.25] * 4
    h = [0.97, 0.01, 0.01, 0.01]
    pfms = [_ic_pfm([u, u] + [h] * 12 + [u]), _ic_pfm([h] * 3)]
    pos = np.array([[3, 2], [0, 4], [7, 0]], np.int32)
    comp = np.array([[1, 0], [0, 0], [0, 0]], np.uint8)
    out = pkg.masked_trim(pfms, filter_size=4, positions=pos, use_comp=comp, after_merged=True)
    assert list(out["front"]) == [2, 0] and list(out["back"]) == [1, 0]
    assert list(out["keep"]) == [True, False]
    # after_merged: the reverse-complemented entry moves by the back trim
    np.testing.assert_array_equal(out["positions"][:, 0], [4, 0, 9])
    assert out["pfms"][0].shape == (4, 12)
