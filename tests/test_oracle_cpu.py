"""CPU tests: the oracle against known answers and the committed golden fixtures.

The reference's own test suite is empty (test/runtests.jl:4-6) and it cannot run
here, so the oracle is pinned by known-answer tests of the mathematics it restates
and by one test per reference quirk."""
import os

import numpy as np
import pytest

from oracle import cdl_oracle as O
from oracle import search_oracle as SO

from conftest import random_onehot, rel

GOLD = os.path.join(os.path.dirname(__file__), "golden")


# ------------------------------------------------------------------ known answers
def test_sherman_csc_solves_normal_equations():
    """sherman_CSC_* (csc_kernels.jl:8-49) == dense solve of (conj(a) a^T + 2 I) x = RHS."""
    rng = np.random.default_rng(0)
    M, Lg, N = 5, 7, 3
    a = rng.standard_normal((M, Lg)) + 1j * rng.standard_normal((M, Lg))
    R = rng.standard_normal((N, M, Lg)) + 1j * rng.standard_normal((N, M, Lg))
    x = O.sherman_csc(a, R, 2.0)
    for n in range(N):
        for l in range(Lg):
            A = np.outer(np.conj(a[:, l]), a[:, l]) + 2.0 * np.eye(M)
            np.testing.assert_allclose(x[n, :, l], np.linalg.solve(A, R[n, :, l]), rtol=1e-12, atol=1e-12)


def test_sherman_cdl_has_no_half_factor():
    """Quirk: sherman_CDL_combine (cdl_kernels.jl:24-33) omits the division by the
    constant, so the D-step result is 2x the solution of (conj(b) b^T + 2 I) x = RHS."""
    rng = np.random.default_rng(1)
    N, M, Lg = 2, 4, 6
    b = rng.standard_normal((N, M, Lg)) + 1j * rng.standard_normal((N, M, Lg))
    R = rng.standard_normal((N, M, Lg)) + 1j * rng.standard_normal((N, M, Lg))
    x = O.sherman_cdl(b, R, 2.0)
    for n in range(N):
        for l in range(Lg):
            A = np.outer(np.conj(b[n, :, l]), b[n, :, l]) + 2.0 * np.eye(M)
            np.testing.assert_allclose(x[n, :, l], 2.0 * np.linalg.solve(A, R[n, :, l]), rtol=1e-12,
                                       atol=1e-12)


def test_fft_product_is_circular_convolution():
    """DX = real(ifft(sum_m D-hat X-hat)) (CDL_setup.jl:197-203) == sum_m D[m] (*) X[n,m]."""
    rng = np.random.default_rng(2)
    S, _ = random_onehot(rng, 3, 5)
    c = O.init_cdl(S, 2, 1, 1.0, 100.0, 0.1, rng=rng)
    Lg = c.Lg
    direct = np.zeros((c.N, Lg))
    for n in range(c.N):
        for m in range(c.M):
            for t in range(Lg):
                for s in range(Lg):
                    direct[n, (t + s) % Lg] += c.G1[m, t] * c.X[n, m, s]
    np.testing.assert_allclose(c.DX, direct, rtol=1e-12, atol=1e-12)


def test_init_shapes_and_constraints():
    rng = np.random.default_rng(3)
    S, _ = random_onehot(rng, 4, 6)
    c = O.init_cdl(S, 3, 2, 1.0, 100.0, 0.1, rng=rng)
    assert c.Lg == 4 * 6 + 2 * 8 and c.gamma == 8
    assert np.all(c.X[..., np.arange(c.Lg) % 4 != 0] == 0)       # enforce_dummy_code_constraint!
    assert np.all(c.G1[:, c.gamma:] == 0)                          # P_D support
    grp = c.G1[:, : c.gamma].reshape(3, -1, 4).sum(-1)
    np.testing.assert_allclose(grp, 1.0, rtol=1e-12)               # rand_probvec per base
    np.testing.assert_allclose(c.WtS[:, c.gamma:c.gamma + c.L], S)
    assert c.obj_best == pytest.approx(O.objective(c))


# ------------------------------------------------------------------ quirks
def test_quirk_prox_group_off_by_one():
    """Q2: prox_simplex_zeros! (cdl_kernels.jl:59) uses rows i+1..i+4 with i = 4 floor(l/4),
    so 1-based row 4 is corrected with rows 5..8."""
    Lg, M = 16, 1
    P = np.zeros((M, Lg)); P[:, :8] = 1
    v = np.arange(1, Lg + 1, dtype=np.float64)[None]
    G = O.prox_simplex_zeros(v, P)
    assert G[0, 0] == pytest.approx(1 - 0.25 * (1 + 2 + 3 + 4 - 1))     # l=1: rows 1..4
    assert G[0, 3] == pytest.approx(4 - 0.25 * (5 + 6 + 7 + 8 - 1))     # l=4: rows 5..8
    assert G[0, 7] == pytest.approx(8 - 0.25 * (9 + 10 + 11 + 12 - 1))  # l=8: rows 9..12
    assert np.all(G[0, 8:] == 0)


def test_quirk_shrink_uses_lambda():
    """Q4: shrink! thresholds at lambda, not lambda/rho (csc_kernels.jl:61)."""
    t = np.array([-0.3, -0.05, 0.0, 0.05, 0.3])
    np.testing.assert_allclose(O.shrink(t, 0.1), [-0.2, 0, 0, 0, 0.2])


def test_quirk_scan_position_one_is_not_found():
    """Q3: scan_w_gpu! maps an argmax of 1 to 0 (scan.jl:197)."""
    L = 6
    S = np.zeros((2, 4 * L), np.float32)
    seqs = ["ACGTTT", "TTACGT"]
    for n, s in enumerate(seqs):
        for i, ch in enumerate(s):
            S[n, 4 * i + "ACGT".index(ch)] = 1
    pwm = np.full((4, 4), -2.0, np.float32)
    for i, ch in enumerate("ACGT"):
        pwm[("ACGT").index(ch), i] = 2.0
    pw = pwm[None]
    pos = SO.scan_w_gpu_positions(pw, S, np.array([4]), np.array([1.0], np.float32))
    assert pos[0, 0] == 0          # best hit at base 1 -> "not found"
    assert pos[0, 1] == 3          # best hit at base 3


# ------------------------------------------------------------------ scan oracle
def _stepped_state(seed=3):
    """A small state one full outer iteration in (d differs from G1 per sequence, the
    duals are non-zero), for the ordering tests."""
    rng = np.random.default_rng(seed)
    N, L, M, fs = 4, 10, 3, 2
    S, _ = random_onehot(rng, N, L)
    Lg = 4 * L + 8 * fs
    X0 = rng.standard_normal((N, M, Lg)).astype(np.float32)
    D0 = rng.standard_normal((M, Lg)).astype(np.float32)
    c = O.init_cdl(S, M, fs, 1.0, 100.0, 0.1, X0=X0, D0=D0)
    O.run_outer(c, 1)
    return c


def test_quirk_xstep_reads_consensus_G1_not_d():
    """Quirk Q5 (src/CDL/train.jl:18-27): code_update! builds the Sherman-Morrison system
    from G1-hat, the consensus dictionary, never from the per-sequence copies d: the
    X-step's result does not move when d and d-hat change, and does when G1-hat does."""
    import copy
    base = _stepped_state()
    a, b, g = copy.deepcopy(base), copy.deepcopy(base), copy.deepcopy(base)
    b.d = (b.d * 3.0 + 1.0).astype(b.d.dtype)
    b.dh = np.fft.fft(b.d.astype(np.complex128), axis=-1).astype(b.dh.dtype)
    g.G1h = (g.G1h * 1.5).astype(g.G1h.dtype)
    for st in (a, b, g):
        O.code_update(st, 1)
    np.testing.assert_array_equal(a.X, b.X)
    np.testing.assert_array_equal(a.DX, b.DX)
    assert not np.array_equal(a.X, g.X)


def test_quirk_dual_update_ordering():
    """Quirk Q6 (src/CDL/train.jl:7-14, 35, 40): y1 += DX - Y1 and y3 += X - Y3 use the
    Y1 and Y3 of the previous X-step (update_Y1! and projectionX! run after the
    solve), y2 += X - Y2 uses the Y2 that shrink! has just formed from the X and y2
    entering this X-step."""
    import copy
    c = _stepped_state()
    X0, DX0, Y1o, Y3o = c.X.copy(), c.DX.copy(), c.Y1.copy(), c.Y3.copy()
    y1o, y2o, y3o = c.y1.copy(), c.y2.copy(), c.y3.copy()
    Y2n = O.shrink(X0 + y2o, c.lam).astype(c.dtype)                # :7, fresh
    O.code_update(c, 1)
    np.testing.assert_array_equal(c.y1, y1o + DX0 - Y1o)           # :12, previous Y1
    np.testing.assert_array_equal(c.y2, y2o + X0 - Y2n)            # :13, fresh Y2
    np.testing.assert_array_equal(c.y3, y3o + X0 - Y3o)            # :14, previous Y3
    assert not np.array_equal(c.Y1, Y1o) and not np.array_equal(c.Y3, Y3o)


def test_quirk_td_uses_d_hat_before_the_dictionary_solve():
    """Quirk Q6, D-step (src/CDL/train.jl:56-60): Td = real(ifft(sum_m Y3-hat d-hat))
    is formed from d-hat before sherman_CDL_combine replaces it in the same D-step."""
    c = _stepped_state()
    Y3h, dh_old = c.Y3h.copy(), c.dh.copy()
    Td_old = np.real(np.fft.ifft(np.sum(Y3h * dh_old, axis=1), axis=-1)).astype(c.dtype)
    O.dict_update(c, 1)
    np.testing.assert_allclose(c.Td, Td_old, rtol=1e-6, atol=1e-6)
    Td_new = np.real(np.fft.ifft(np.sum(Y3h * c.dh, axis=1), axis=-1)).astype(c.dtype)
    assert not np.allclose(c.Td, Td_new, rtol=1e-3, atol=1e-3)


def test_scan_oracle_integer_brute_force():
    """With integer PWM entries and one-hot data the FP32 scores are exact integers;
    compare the oracle's scans with a direct count."""
    rng = np.random.default_rng(5)
    N, L, K = 30, 25, 4
    S, bases = random_onehot(rng, N, L)
    lens = rng.integers(2, 8, K)
    pwms = [rng.integers(-3, 4, (4, w)).astype(np.float32) for w in lens]
    thresh = np.array([1.0] * K, np.float32)
    pos, score, comp = SO.overlapping_scan(S, pwms, lens, thresh)
    for k in range(K):
        w = lens[k]
        pw = pwms[k]
        pc = pw[::-1, ::-1]
        for n in range(N):
            f = [sum(pw[bases[n, i + j], j] for j in range(w)) for i in range(L - w + 1)]
            r = [sum(pc[bases[n, i + j], j] for j in range(w)) for i in range(L - w + 1)]
            bf, br = max(f), max(r)
            best, use_c = (bf, False) if bf >= br else (br, True)
            if best > 1.0:
                assert pos[k, n] == (1 + (f.index(bf) if not use_c else r.index(br)))
                assert score[k, n] == best and comp[k, n] == use_c
            else:
                assert pos[k, n] == 0


def test_non_overlap_select_known_answers():
    """non_overlap_scan! (scan.jl:123-174): highest score first (ties: lower motif index),
    a span meeting a kept span is dropped, entries with no hit stay empty."""
    lens = [4, 4, 3, 5]
    # (N, K): sequence 0: motif 0 at 1 (score 5), motif 1 at 3 (4, overlaps 0), motif 2 at
    # 10 (3), motif 3 absent;  sequence 1: a tie between motifs 1 and 2 at overlapping
    # spans -> motif 1 kept;  sequence 2: negative scores beside an absent motif (score 0
    # wins argmax at once) -> nothing kept;  sequence 3: only negative scores -> the
    # largest is taken, then the zeroed entry ends the loop
    pos = np.array([[1, 3, 10, 0], [0, 5, 6, 20], [2, 9, 0, 0], [2, 9, 15, 30]], np.int32)
    score = np.array([[5, 4, 3, 0], [0, 2, 2, 1], [-1, -2, 0, 0], [-1, -2, -3, -0.5]], np.float32)
    comp = np.array([[1, 1, 0, 0], [0, 1, 1, 1], [1, 0, 0, 0], [1, 1, 1, 1]], np.uint8)
    p2, s2, c2 = SO.non_overlap_select(pos, score, comp, lens)
    np.testing.assert_array_equal(p2, [[1, 0, 10, 0], [0, 5, 0, 20], [0, 0, 0, 0], [0, 0, 0, 30]])
    np.testing.assert_array_equal(s2, [[5, 0, 3, 0], [0, 2, 0, 1], [0, 0, 0, 0], [0, 0, 0, -0.5]])
    np.testing.assert_array_equal(c2, [[1, 0, 0, 0], [0, 1, 0, 1], [0, 0, 0, 0], [0, 0, 0, 1]])


FASTA_TEXT = (b">s1 first\nACGT\nAC\n>s2\nacgtac\n>s3 with an N\nACGNAC\n"
              b">s4 short\nACG\n>s5\nTTTTGG\n")


def test_read_fasta_onehot_rules():
    """reading/read_fasta (read.jl:2-28) + data_2_dummy (to_dummy.jl:27-38): header lines
    dropped, lines joined, records with N dropped, upper-cased, max_entries after the
    filter, records of another length left as zero rows."""
    S, reads = SO.read_fasta_onehot(FASTA_TEXT)
    assert reads == ["ACGTAC", "ACGTAC", "ACG", "TTTTGG"]
    assert S.shape == (4, 24)
    np.testing.assert_array_equal(S[0], S[1])
    assert S[2].sum() == 0 and S[3].sum() == 6
    np.testing.assert_array_equal(S[0].reshape(6, 4).argmax(1), [0, 1, 2, 3, 0, 1])
    S3, reads3 = SO.read_fasta_onehot(FASTA_TEXT, max_entries=2)
    assert reads3 == ["ACGTAC", "ACGTAC"] and S3.shape == (2, 24)


def test_pvalue2score_known_answers():
    """find_largest_alpha (PWM_Touzet.jl:130-142) returns the first key (ascending) whose
    tail probability is below pval; with one column (2, 0, 0, 0) the rounded keys are 0
    (probability 3/4) and floor(2 / 0.1) 0.1 = 1.9 (the Float64 0.1 is above 1/10)."""
    pwm = np.array([[2.0], [0.0], [0.0], [0.0]], np.float32)
    assert SO.pvalue2score(pwm, 0.25) == np.float32(1.9)
    assert SO.pvalue2score(pwm, 0.3) == np.float32(1.9)
    pwm2 = np.array([[1.0, 1.0], [0.0, 0.0], [0.0, 0.0], [0.0, 0.0]], np.float32)
    # keys 0 (9/16), 0.9 (6/16: one column hit... floor(1/0.1)=9), 1.8 (1/16)
    assert SO.pvalue2score(pwm2, 1.0 / 16) == np.float32(1.8)
    assert SO.pvalue2score(pwm2, 0.5) == np.float32(0.9)


def test_count_matrices_revcomp():
    S = np.zeros((1, 4 * 5), np.float32)
    for i, ch in enumerate("AACGT"):
        S[0, 4 * i + "ACGT".index(ch)] = 1
    counts, nseq = SO.count_matrices(S, np.array([[2]]), np.array([[1]]), [3])
    # window ACG reverse-complemented = CGT
    exp = np.zeros((3, 4), int)
    for i, ch in enumerate("CGT"):
        exp[i, "ACGT".index(ch)] = 1
    np.testing.assert_array_equal(counts[0], exp)
    assert nseq[0] == 1


# ------------------------------------------------------------------ transfac format
def test_transfac_hand_derived():
    """save_pfms_as_transfac (save_learned_results.jl:186-196): 2-digit row labels,
    values pfm*1000 in Julia Float32 shortest form, tab separated, XX trailer."""
    pfm = np.array([[0.25, 0.5], [0.25, 0.25], [0.25, 0.125], [0.25, 0.125]], np.float32)
    exp = ("ID\t\nXX\t\nBF\t\nXX\t\nP0\tA\tC\tG\tT\n"
           "01\t250.0\t250.0\t250.0\t250.0\n"
           "02\t500.0\t250.0\t125.0\t125.0\n"
           "XX\t\n")
    assert SO.transfac_text(pfm) == exp
    p2 = np.array([[0.1], [0.2], [0.3], [0.4]], np.float32)
    assert SO.transfac_text(p2).splitlines()[5] == "01\t100.0\t200.0\t300.0\t400.0"
    p3 = np.full((4, 10), np.float32(1 / 3), np.float32)
    assert SO.transfac_text(p3).splitlines()[14].startswith("10\t333.33334\t")


def test_julia_float_strings():
    f = SO.julia_float32_string
    assert f(np.float32(250)) == "250.0"
    assert f(np.float32(0.1)) == "0.1"
    assert f(np.float32(1e-5)) == "1.0e-5"
    assert f(np.float32(1e6)) == "1.0e6"
    assert f(np.float32(123456)) == "123456.0"
    assert f(np.float32(1 / 3)) == "0.33333334"


# ------------------------------------------------------------------ golden fixtures
@pytest.mark.parametrize("name", ["admm_tiny", "admm_small", "admm_refdefaults"])
def test_oracle_reproduces_golden(name):
    g = np.load(os.path.join(GOLD, name + ".npz"))
    M, fs, lam, rho, sigma, outer, csc, cdl = g["params"]
    c = O.init_cdl(g["S"], int(M), int(fs), rho, sigma, lam, X0=g["X0"], D0=g["D0"])
    assert c.obj_best == pytest.approx(float(g["obj0"]), rel=1e-12)
    objs = O.run_outer(c, int(outer), int(csc), int(cdl))
    np.testing.assert_allclose(objs, g["objs"], rtol=1e-10)
    assert rel(c.X, g["X"]) < 1e-6 and rel(c.d, g["d"]) < 1e-6
    assert rel(c.G1, g["G1"]) < 1e-6


def test_scan_oracle_reproduces_golden():
    g = np.load(os.path.join(GOLD, "scan_small.npz"))
    pos_fwd = SO.scan_w_gpu_positions(g["pwms"], g["S"], g["lens"], g["thresh"])
    np.testing.assert_array_equal(pos_fwd, g["pos_fwd"])
    pwms = [g["pwms"][k, :, : g["lens"][k]] for k in range(len(g["lens"]))]
    pos, score, comp = SO.overlapping_scan(g["S"], pwms, g["lens"], g["thresh"])
    np.testing.assert_array_equal(pos, g["pos"])
    np.testing.assert_array_equal(score, g["score"])
    np.testing.assert_array_equal(comp, g["comp"])


def test_select_pairs_is_julia_findall_order(pkg, built_lib):
    """findall on Julia (K, K, maxlen) walks fr fastest, then fc, then the overlap."""
    rng = np.random.default_rng(9)
    over = rng.integers(0, 10, (3, 4, 4)).astype(np.int32)
    got = [tuple(int(v) for v in p) for p in pkg.select_pairs(over, 6)]
    exp = [(fr + 1, fc + 1, o + 1) for o in range(3) for fc in range(4) for fr in range(4)
           if over[o, fc, fr] > 6]
    assert got == exp
