"""The residual record and the stopping test (FP64 sums on the GPU) against the oracle's
restatement, through the C ABI, on every X-step and D-step path."""
import numpy as np
import pytest

from oracle import cdl_oracle as O

pytestmark = pytest.mark.gpu

# the residual vectors are differences of FP32 quantities that agree with FP64 to ~1e-5
# relative, so their norms are compared on the scale of the iterate they belong to:
# |sqrt(r_gpu) - sqrt(r_ref)| <= 1e-3 sqrt(r_ref) + 1e-4 sqrt(norm)
TOL_REL, TOL_NORM = 1e-3, 1e-4
PAIRS = [(0, 3), (1, 3), (2, 4), (5, 8), (6, 8), (7, 9), (10, 12), (11, 12)]
NORMS = [3, 4, 8, 9, 12]


def _case(pkg, N, L, M, fs, seed=3):
    synth = pkg.synth
    bases, _, _ = synth.plant_dataset(seed, N, L, [8, 12], [0.4, 0.4])
    S = synth.onehot(bases)
    Lg = 4 * L + 8 * fs
    return S, synth.init_X0(seed, N, M, Lg), synth.init_D0_unit_norm(seed, M, Lg, 4 * fs)


def _check_record(got, ref):
    # |DX|^2 covers the zero-padded rows, where every float32 path drifts (1e-3 there)
    for k in NORMS:
        assert got[k] == pytest.approx(ref[k], rel=1e-3), k
    for k, kn in PAIRS:
        a, b, nrm = np.sqrt(got[k]), np.sqrt(ref[k]), np.sqrt(ref[kn])
        assert abs(a - b) <= TOL_REL * b + TOL_NORM * nrm, (k, a, b, nrm)
    rr = O.relative_residuals(ref)
    for i, name in enumerate(("primal_x", "primal_dx", "primal_d", "primal_td", "dual_d")):
        assert got[13 + i] == pytest.approx(rr[name], rel=2e-3, abs=1e-5), name
    assert got[18] == max(got[13:18])


@pytest.mark.parametrize("path", ["multi_iter", "one_xstep", "cufft", "time_domain_dstep"])
@pytest.mark.parametrize("shape", [(6, 200, 64, 16), (12, 100, 16, 12)])
def test_residual_record_against_oracle(pkg, built_lib, path, shape, monkeypatch):
    N, L, M, fs = shape
    if path == "one_xstep":
        monkeypatch.setenv("CDLGB_XITER", "0")
    if path == "time_domain_dstep":
        monkeypatch.setenv("CDLGB_DSPEC", "0")
    S, X0, D0 = _case(pkg, N, L, M, fs)
    ref = O.init_cdl(S, M, fs, 1.0, 100.0, 0.1, X0=X0, D0=D0)
    setup = pkg.CDLSetup(M=M, filter_size=fs, lambda_=0.1, rho=1.0, sigma=100.0,
                         track_residuals=True)
    with pkg.init_cdl(setup, S, X0=X0, D0=D0, fft_mode=1 if path == "cufft" else 0) as c:
        assert np.all(c.residuals() == 0.0)
        for it in range(2):
            pkg.code_update(c, 15)
            O.code_update(ref, 15)
            got = c.residuals()
            for k in range(5):
                assert np.sqrt(got[k]) == pytest.approx(np.sqrt(ref.resid[k]), rel=TOL_REL,
                                                        abs=TOL_NORM * np.sqrt(ref.resid[3 if k < 2 else 4]))
            pkg.update_best(c)
            O.update_best(ref)
            pkg.dict_update(c, 1)
            O.dict_update(ref, 1)
            _check_record(c.residuals(), ref.resid)


def test_stopping_test(pkg, built_lib):
    """stop_tol = 0 runs the fixed count (the reference's loop); stop_tol > 0 ends after
    the first outer iteration whose largest relative residual is <= stop_tol."""
    N, L, M, fs = 12, 100, 16, 12
    S, X0, D0 = _case(pkg, N, L, M, fs, seed=8)
    setup = pkg.CDLSetup(M=M, filter_size=fs, lambda_=0.1, rho=1.0, sigma=100.0,
                         track_residuals=True)
    rel_max, objs = [], []
    with pkg.init_cdl(setup, S, X0=X0, D0=D0) as c:
        for _ in range(8):
            objs.append(pkg.run_outer(c, 1)[0])
            rel_max.append(c.residuals()[18])
        assert c.outer_done == 1
    with pkg.init_cdl(setup, S, X0=X0, D0=D0) as c:
        o = pkg.run_outer(c, 8)
        assert c.outer_done == 8 and len(o) == 8
        np.testing.assert_array_equal(o, objs)
    # without residual tracking (the default) the record stays zero and the iterates
    # are the same bits: the residual sums change no result
    setup.track_residuals = False
    with pkg.init_cdl(setup, S, X0=X0, D0=D0) as c:
        np.testing.assert_array_equal(pkg.run_outer(c, 8), objs)
        assert np.all(c.residuals() == 0.0)
    setup.track_residuals = True
    for k in (2, 5):
        tol = float(np.float32(rel_max[k]) * np.float32(1.0000001))
        want = next(i for i, v in enumerate(rel_max) if v <= tol) + 1
        setup.stop_tol = tol
        with pkg.init_cdl(setup, S, X0=X0, D0=D0) as c:
            o = pkg.run_outer(c, 8)
            assert c.outer_done == want and len(o) == want
            np.testing.assert_array_equal(o, objs[:want])
    setup.stop_tol = 1e30
    with pkg.init_cdl(setup, S, X0=X0, D0=D0) as c:
        assert len(pkg.run_outer(c, 8)) == 1
