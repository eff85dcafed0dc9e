"""The torch restatements used by the precision study and the long-run GPU parity test,
run on the CPU in float64 against the NumPy oracle: states, objectives and the residual
record."""
import numpy as np
import pytest

from oracle import cdl_oracle as O

from conftest import random_onehot, rel


@pytest.mark.parametrize("form", ["half_spectrum", "literal"])
def test_torch_restatement_matches_oracle(form):
    torch = pytest.importorskip("torch")
    from oracle import torch_admm as T
    rng = np.random.default_rng(31)
    N, L, M, fs = 7, 14, 3, 2
    S, _ = random_onehot(rng, N, L)
    Lg = 4 * L + 8 * fs
    X0 = rng.standard_normal((N, M, Lg))
    D0 = rng.standard_normal((M, Lg))
    ref = O.init_cdl(S, M, fs, 1.0, 100.0, 0.1, X0=X0, D0=D0)
    cls = T.HalfSpectrumADMM if form == "half_spectrum" else T.LiteralADMM
    f = cls(S, X0, D0, M, fs, 1.0, 100.0, 0.1, device="cpu", chunk=3, dtype=torch.float64)
    assert f.obj_best == pytest.approx(ref.obj_best, rel=1e-12)
    objs = f.run_outer(3)
    objs_ref = O.run_outer(ref, 3)
    np.testing.assert_allclose(objs, objs_ref, rtol=1e-10)
    assert rel(f.X.numpy(), ref.X) < 1e-10
    assert rel(f.d.numpy(), ref.d) < 1e-10
    assert rel(f.G1.numpy(), ref.G1) < 1e-10
    assert rel(f.D_best.numpy(), ref.D_best) < 1e-10
    np.testing.assert_allclose(f.resid, ref.resid, rtol=1e-8)
    rr, rr_ref = T.relative_residuals(f.resid), O.relative_residuals(ref.resid)
    for k in rr:
        assert rr[k] == pytest.approx(rr_ref[k], rel=1e-8)


def test_residuals_are_the_dual_increments():
    """The D-step's residuals are the squared increments of g1, g3, g2 (train.jl:70-72),
    and the code update's are the increments the next dual updates (train.jl:12-14) add."""
    rng = np.random.default_rng(5)
    N, L, M, fs = 5, 12, 3, 2
    S, _ = random_onehot(rng, N, L)
    Lg = 4 * L + 8 * fs
    c = O.init_cdl(S, M, fs, 1.0, 100.0, 0.1, X0=rng.standard_normal((N, M, Lg)),
                   D0=rng.standard_normal((M, Lg)))
    O.code_update(c, 4)
    y1, y2, y3 = c.y1.copy(), c.y2.copy(), c.y3.copy()
    r = c.resid.copy()
    O.code_update(c, 1)
    # the next X-step's dual updates add exactly the residual vectors
    # (y3 there uses the stored Y3 = projectionX(X + y3), so the increment is X - Y3)
    assert np.sum((c.y2 - y2) ** 2) == pytest.approx(r[0], rel=1e-9)
    assert np.sum((c.y3 - y3) ** 2) == pytest.approx(r[1], rel=1e-9)
    assert np.sum((c.y1 - y1) ** 2) == pytest.approx(r[2], rel=1e-9)
    g1, g2, g3 = c.g1.copy(), c.g2.copy(), c.g3.copy()
    G1, G3 = c.G1.copy(), c.G3.copy()
    O.dict_update(c, 1)
    assert np.sum((c.g1 - g1) ** 2) == pytest.approx(c.resid[5], rel=1e-9)
    assert np.sum((c.g3 - g3) ** 2) == pytest.approx(c.resid[6], rel=1e-9)
    assert np.sum((c.g2 - g2) ** 2) == pytest.approx(c.resid[7], rel=1e-9)
    assert N * np.sum((c.G1 - G1) ** 2) == pytest.approx(c.resid[10], rel=1e-9)
    assert N * np.sum((c.G3 - G3) ** 2) == pytest.approx(c.resid[11], rel=1e-9)
