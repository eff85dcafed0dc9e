"""GPU parity of the background shuffle (k_klet_shuffle) and the e-value filter:
the device shuffle equals the oracle's draw for draw; at the full 20000 x 200 size
every sequence keeps its k-mer counts and end (k-1)-mers; filter_using_evalue
agrees with the oracle's scans and exact Fisher e-values."""
import numpy as np
import pytest

from oracle import search_oracle as SO

pytestmark = pytest.mark.gpu


def _ctx(pkg, S):
    c = pkg.CDL(pkg.CDLSetup(M=2, filter_size=2))
    c.load_data(S)
    return c


def _data(seed, N, L, holes=True):
    from cdlmotif_gb300 import synth
    rng = np.random.default_rng(seed)
    S = synth.onehot(rng.integers(0, 4, (N, L)).astype(np.uint8))
    if holes:                                   # a few columns with no base
        for n in range(0, N, 7):
            S[n, 4 * int(rng.integers(0, L)):][:4] = 0.0
    return S


@pytest.mark.parametrize("k", [1, 2, 3, 4])
@pytest.mark.parametrize("N,L", [(40, 100), (9, 5), (3, 2)])
def test_background_matches_oracle(pkg, built_lib, k, N, L):
    S = _data(k * 100 + L, N, L)
    with _ctx(pkg, S) as c:
        c.make_background(k=k, seed=1234)
        got = c.background()
    np.testing.assert_array_equal(got, SO.make_background(S, k=k, seed=1234))


def _kmer_codes(sym, k):
    N, L = sym.shape
    codes = np.zeros((N, L - k + 1), np.int64)
    for j in range(k):
        codes = codes * 5 + sym[:, j:L - k + 1 + j]
    return codes


def test_background_properties_full_size(pkg, built_lib):
    N, L, k = 20000, 200, 3
    S = _data(5, N, L)
    with _ctx(pkg, S) as c:
        c.make_background(k=k, seed=99)
        bg = c.background()
        again = c.background()
        c.make_background(k=k, seed=99)
        np.testing.assert_array_equal(c.background(), again)   # reproducible
    s0, s1 = SO.onehot_symbols(S), SO.onehot_symbols(bg)
    np.testing.assert_array_equal(s0[:, :k - 1], s1[:, :k - 1])
    np.testing.assert_array_equal(s0[:, L - k + 1:], s1[:, L - k + 1:])
    c0, c1 = _kmer_codes(s0, k), _kmer_codes(s1, k)
    V = 5 ** k
    rows = np.repeat(np.arange(N), c0.shape[1])
    h0 = np.bincount(rows * V + c0.ravel(), minlength=N * V)
    h1 = np.bincount(rows * V + c1.ravel(), minlength=N * V)
    np.testing.assert_array_equal(h0, h1)
    assert (s0 != s1).any(axis=1).mean() > 0.99


@pytest.mark.parametrize("cpu,non_overlap", [(False, False), (True, False), (True, True)])
def test_filter_using_evalue_matches_oracle(pkg, built_lib, cpu, non_overlap):
    from cdlmotif_gb300 import synth
    bases, motifs, _ = synth.plant_dataset(21, 600, 80, [12, 8, 10, 7], [0.5, 0.02, 0.3, 0.0])
    S = synth.onehot(bases)
    pwms = [np.log2(((m + 0.05) / 1.2) / 0.25).astype(np.float32) for m in motifs]
    lens = np.array([p.shape[1] for p in pwms], np.int32)
    thresh = np.array([0.6 * float(np.sum(np.max(p, axis=0))) for p in pwms], np.float32)
    with _ctx(pkg, S) as c:
        pos, _, _ = pkg.overlapping_scan(c, pwms, thresh)
        c.make_background(k=3, seed=7)
        out = pkg.filter_using_evalue(c, pwms, thresh, pos, cpu=cpu, non_overlap=non_overlap)
        # the scans read the data again after the filter
        np.testing.assert_array_equal(pkg.overlapping_scan(c, pwms, thresh)[0], pos)
    bg = SO.make_background(S, k=3, seed=7)
    pad = np.zeros((len(pwms), 4, int(lens.max())), np.float32)
    for i, p in enumerate(pwms):
        pad[i, :, : lens[i]] = p
    if not cpu:
        bpos = SO.scan_w_gpu_positions(pad, bg, lens, thresh)          # (K, N)
        hb = (bpos > 0).sum(axis=1)
    else:
        rp, rs, _ = SO.overlapping_scan(bg, pwms, lens, thresh)       # (K, N)
        if non_overlap:
            rp, rs, _ = SO.non_overlap_select(rp.T, rs.T, None, lens)
            hb = (rp > 0).sum(axis=0)
        else:
            hb = (rp > 0).sum(axis=1)
    ha = (pos > 0).sum(axis=0)
    np.testing.assert_array_equal(out["hits_bg"], hb)
    np.testing.assert_array_equal(out["hits"], ha)
    K = len(pwms)
    ref = np.array([SO.fisher_evalue_exact(int(ha[i]), int(hb[i]), 600, K) for i in range(K)])
    np.testing.assert_allclose(out["evalues"], ref, rtol=1e-9, atol=0)
    thr = np.float32(1e-3 if cpu else 0.5)
    np.testing.assert_array_equal(out["keep"], (ref < thr) & (lens > 5))
