"""The FP64 reference used by the precision study, run on the CPU against the oracle."""
import numpy as np
import pytest

from oracle import cdl_oracle as O

from conftest import random_onehot, rel


def test_fp64_reference_matches_oracle(pkg):
    pytest.importorskip("torch")
    from cdlmotif_gb300.fp64ref import FP64Reference
    rng = np.random.default_rng(31)
    N, L, M, fs = 7, 14, 3, 2
    S, _ = random_onehot(rng, N, L)
    Lg = 4 * L + 8 * fs
    X0 = rng.standard_normal((N, M, Lg))
    D0 = rng.standard_normal((M, Lg))
    ref = O.init_cdl(S, M, fs, 1.0, 100.0, 0.1, X0=X0, D0=D0)
    f = FP64Reference(S, X0, D0, M, fs, 1.0, 100.0, 0.1, device="cpu", chunk=3)
    assert f.obj_best == pytest.approx(ref.obj_best, rel=1e-12)
    objs = f.run_outer(3)
    objs_ref = O.run_outer(ref, 3)
    np.testing.assert_allclose(objs, objs_ref, rtol=1e-10)
    assert rel(f.X.numpy(), ref.X) < 1e-10
    assert rel(f.d.numpy(), ref.d) < 1e-10
    assert rel(f.G1.numpy(), ref.G1) < 1e-10
    assert rel(f.D_best.numpy(), ref.D_best) < 1e-10
