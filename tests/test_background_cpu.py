"""CPU tests of the background (k-let shuffle) oracle and of the Fisher e-values:
the shuffle keeps every k-mer count and both end (k-1)-mers, its random stream is
splitmix64, and the library's host e-values match exact rational arithmetic."""
import numpy as np
import pytest

from oracle import search_oracle as SO


def test_splitmix64_published_value():
    # splitmix64 with state 0: the first output is mix(0 + golden gamma)
    assert SO._mix64(0x9E3779B97F4A7C15) == 0xE220A8397B1DCDAF


def test_below_is_in_range_and_deterministic():
    r1, r2 = SO.SplitMix(5, 3), SO.SplitMix(5, 3)
    a = [r1.below(7) for _ in range(200)]
    assert a == [r2.below(7) for _ in range(200)]
    assert min(a) >= 0 and max(a) <= 6 and len(set(a)) == 7
    assert [SO.SplitMix(5, 4).below(7) for _ in range(20)] != a[:20]


@pytest.mark.parametrize("k", [1, 2, 3, 4])
def test_klet_shuffle_keeps_kmers_and_ends(k):
    rng = np.random.default_rng(k)
    for n in range(30):
        L = int(rng.integers(1, 60))
        sym = rng.integers(0, 5 if n % 3 == 0 else 4, L)
        out = SO.klet_shuffle_seq(sym, k, SO.SplitMix(11, n))
        assert len(out) == L
        assert SO.kmer_counts(out, k) == SO.kmer_counts(sym, k)
        if k > 1 and L >= k:
            assert list(out[: k - 1]) == list(sym[: k - 1])
            assert list(out[L - k + 1:]) == list(sym[L - k + 1:])


def test_klet_shuffle_moves_long_sequences():
    rng = np.random.default_rng(0)
    sym = rng.integers(0, 4, 300)
    out = SO.klet_shuffle_seq(sym, 3, SO.SplitMix(1, 0))
    assert list(out) != list(sym)


def test_onehot_symbols_and_background_layout():
    data = np.zeros((2, 12), np.float32)
    data[0, [0, 5, 10]] = 1.0            # A C G
    data[1, 3] = 1.0                     # T, then a column with no base twice
    np.testing.assert_array_equal(SO.onehot_symbols(data), [[0, 1, 2], [3, 4, 4]])
    bg = SO.make_background(data, k=1, seed=3)
    assert bg.shape == data.shape
    assert sorted(SO.onehot_symbols(bg)[0]) == [0, 1, 2]
    assert sorted(SO.onehot_symbols(bg)[1]) == [3, 4, 4]


def test_fisher_hand_derived():
    # [3 3; 0 3]: X ~ Hyp(6 successes, 3 failures, 3 draws), P(X >= 3) = 20/84
    assert SO.fisher_evalue_exact(3, 0, 3, 1) == pytest.approx(40 / 84, rel=1e-15)
    # no hits anywhere: X = 0 surely, p = 1, e-value = K
    assert SO.fisher_evalue_exact(0, 0, 5, 7) == 7.0


def test_fisher_c_matches_exact(pkg, built_lib):
    rng = np.random.default_rng(3)
    for N in (1, 7, 100, 2000):
        K = 9
        a = rng.integers(0, N + 1, K)
        b = rng.integers(0, N + 1, K)
        a[0], b[0] = N, 0
        a[1], b[1] = 0, 0
        ev = pkg.fisher_evalues(a, b, N)
        for i in range(K):
            ref = SO.fisher_evalue_exact(int(a[i]), int(b[i]), N, K)
            assert ev[i] == pytest.approx(ref, rel=1e-9, abs=1e-300), (N, a[i], b[i])
