"""GPU parity of the code -> activation -> topology -> pair-PFM stage
(record_training_result!, topology_at_nth_pt!, get_pair_pfms!) against the oracle:
filter selection and integer overlap / gap / adjacency counts bit-exact, pair PFMs
(float32 sums of code-weighted one-hot windows) within 1e-5 relative."""
import numpy as np
import pytest

from oracle import search_oracle as SO

pytestmark = pytest.mark.gpu


def _two_trainings(pkg, N=80, L=40, M=6, fs=3):
    synth = pkg.synth
    bases, _, _ = synth.plant_dataset(11, N, L, [6, 8], [0.6, 0.6])
    S = synth.onehot(bases)
    setup = pkg.CDLSetup(M=M, filter_size=fs, lambda_=0.1, rho=1.0, sigma=100.0, iter_num=3)
    ctxs, threshs, Xbs = [], [], []
    for t in range(2):
        c, th, _ = pkg.cdl_train(setup, S, seed=100 + t)
        ctxs.append(c)
        threshs.append(th)
        Xbs.append(c.X_best)
    return S, ctxs, threshs, Xbs


def test_record_topology_pairs_match_oracle(pkg, built_lib):
    N, L, M, fs = 80, 40, 6, 3
    S, ctxs, threshs, Xbs = _two_trainings(pkg, N, L, M, fs)
    gamma, L4 = 4 * fs, 4 * L
    try:
        with pkg.ActivationRecord(N, L, M, T=2) as ar:
            added = [pkg.record_training_result(ctxs[t], threshs[t], ar, t + 1, fs) for t in range(2)]
            u, tn, fl = ar.info()
            assert len(u) == sum(added)
            codes = np.stack([SO.record_codes(Xbs[t], gamma, L4) for t in range(2)])   # (T, N, M, C)
            for t in range(2):
                exp = [m + 1 for m in range(M) if (codes[t][:, m, :] > np.float32(threshs[t])).any()]
                assert list(u[tn == t + 1]) == exp
            start_pos = np.stack([codes[tn[k] - 1][:, u[k] - 1, :] > np.float32(threshs[tn[k] - 1])
                                  for k in range(len(u))], axis=1)                     # (N, K, C)
            over, non_over, next_to = pkg.get_spatial_info(ar)
            ro, rn, rx = SO.activation_topology(start_pos, tn, fl, L)
            np.testing.assert_array_equal(over, ro)
            np.testing.assert_array_equal(non_over, rn)
            np.testing.assert_array_equal(next_to, rx)
            assert over.sum() > 0
            thr = int(np.percentile(over[over > 0], 60))
            pairs, spans, pfms = pkg.get_pair_pfms(ar, ctxs[0], over, thr, fs)
            rpairs, rspans, rpfms = SO.pair_msas(over, start_pos, fl, tn, u, codes, S, thr, fs)
            assert [tuple(int(v) for v in p) for p in pairs] == rpairs
            assert len(rpairs) > 0
            np.testing.assert_array_equal(spans, rspans)
            for a, b in zip(pfms, rpfms):
                np.testing.assert_allclose(a, b, rtol=1e-5, atol=1e-6)
                np.testing.assert_allclose(a.sum(axis=0)[0], 1.0, rtol=1e-5)
    finally:
        for c in ctxs:
            c.close()


def test_record_rejects_bad_threshold(pkg, built_lib):
    rng = np.random.default_rng(2)
    N, L, M, fs = 8, 12, 3, 2
    bases = rng.integers(0, 4, (N, L)).astype(np.uint8)
    S = pkg.synth.onehot(bases)
    setup = pkg.CDLSetup(M=M, filter_size=fs)
    with pkg.init_cdl(setup, S, seed=1) as c, pkg.ActivationRecord(N, L, M, T=2) as ar:
        with pytest.raises(pkg.CDLGBError):
            pkg.record_training_result(c, 0.0, ar, 1, fs)      # store.jl:8 asserts thresh > 0
        with pytest.raises(pkg.CDLGBError):
            pkg.record_training_result(c, 0.5, ar, 3, fs)      # training 3 of 2
