"""The reference-structured CUDA baseline (baseline/refstruct.cu, the comparator that
stands in for the reference's CUDA.jl path) reproduces the oracle: it is timed as the
reference GPU path, so it has to compute the same ADMM.  Tolerances as for the
product path (X, d relative L2 <= 1e-4 after 2 outer iterations, objective 1e-5)."""
import os
import sys

import numpy as np
import pytest

from oracle import cdl_oracle as O

from conftest import rel

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def refstruct():
    sys.path.insert(0, os.path.join(ROOT, "baseline"))
    import refstruct as R
    R.build()
    return R


@pytest.mark.parametrize("shape", [(6, 40, 5, 4), (5, 100, 16, 12)])
def test_refstruct_matches_oracle(pkg, refstruct, shape):
    N, L, M, fs = shape
    synth = pkg.synth
    bases, _, _ = synth.plant_dataset(21, N, L, [6, 10], [0.5, 0.5])
    S = synth.onehot(bases)
    Lg = 4 * L + 8 * fs
    X0 = synth.init_X0(6, N, M, Lg)
    D0 = synth.init_D0_unit_norm(6, M, Lg, 4 * fs)
    ref = O.init_cdl(S, M, fs, 1.0, 100.0, 0.1, X0=X0, D0=D0)
    objs_ref = O.run_outer(ref, 2)
    with refstruct.RefStruct(S, X0, D0, M, fs) as rs:
        objs = rs.run_outer(2)
        np.testing.assert_allclose(objs, objs_ref, rtol=1e-5)
        assert rel(rs.get("X"), ref.X) < 1e-4
        assert rel(rs.get("d"), ref.d) < 1e-4
        assert rel(rs.get("G1"), ref.G1) < 1e-4
        assert rel(rs.get("D_best"), ref.D_best) < 1e-4
