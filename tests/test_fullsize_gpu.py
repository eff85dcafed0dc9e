"""Size-independent properties at the full N = 20000, L = 200, K = 64, W = 16 size
(Lg = 928), where the oracle cannot run:

* the X-step couples no sequences, so a code update of all 20000 sequences and the
  same code update of a few of them alone give the same bits for those sequences
  (every field the X-step writes);
* the D-step's consensus is an average over sequences: duplicating every sequence
  (2N sequences, each twice) leaves the dictionary where N gives it, up to the
  reassociation of the sums."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N, L, M, FS = 20000, 200, 64, 16


def _setup(pkg):
    return pkg.CDLSetup(M=M, filter_size=FS, lambda_=0.1, rho=1.0, sigma=100.0)


@pytest.fixture(scope="module")
def data(pkg):
    bases, _, _ = pkg.synth.plant_dataset(2024, N, L, [8, 11, 14, 17, 20], [0.1, 0.175, 0.25, 0.325, 0.4])
    return pkg.synth.onehot(bases)


def test_code_update_is_per_sequence_at_full_size(pkg, built_lib, data):
    pick = np.array([0, 1, 7777, 12345, N - 1])
    fields = ("X", "y2", "y3", "DX", "Y1", "y1")
    with pkg.init_cdl(_setup(pkg), data, seed=5) as c:
        X0 = c.get("X")[pick].copy()
        D0 = c.get("d")[0].copy()
        pkg.code_update(c, 15)
        big = {f: c.get(f)[pick] for f in fields}
    with pkg.init_cdl(_setup(pkg), data[pick], X0=X0, D0=D0) as c:
        pkg.code_update(c, 15)
        for f in fields:
            np.testing.assert_array_equal(c.get(f), big[f], err_msg=f)


def test_dictionary_of_duplicated_sequences(pkg, built_lib, data):
    sub = data[:2500]
    two = np.concatenate([sub, sub])
    with pkg.init_cdl(_setup(pkg), sub, seed=9) as c:
        X0 = c.get("X")          # the drawn codes depend on the sequence index: reuse them
    res = []
    for S, X in ((sub, X0), (two, np.concatenate([X0, X0]))):
        with pkg.init_cdl(_setup(pkg), S, X0=X, seed=9) as c:
            pkg.run_outer(c, 2)
            res.append((c.get("G1"), c.get("D_best")))
    for a, b in zip(res[0], res[1]):
        assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(a)
