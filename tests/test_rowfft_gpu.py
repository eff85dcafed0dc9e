"""The register-FFT row transforms (k_rows_r2c / k_rows_c2r) that take the place of
cuFFT's batched R2C / C2R on every length with streaming transforms: G1-hat at each
code update (src/CDL/train.jl:3), the initial DX (src/SETUP/CDL_setup.jl:238-241), and
the D-step's rfft(G2 - g2), rfft(G3), Td and the three sums over sequences
(src/CDL/train.jl:52-72).  Odd row counts (N odd) pair the last row with zeros.

Checked against the FP64 oracle at the suite's tolerances (DX after init 1e-5, fields
after an outer iteration 1e-4, objectives 1e-5), against the same run on cuFFT
(CDLGB_ROWFFT=0), and that the default path makes no cuFFT call at all."""
import numpy as np
import pytest

from oracle import cdl_oracle as O

from conftest import rel

pytestmark = pytest.mark.gpu

TOL_X = 1e-4
TOL_OBJ = 1e-5

# (N, L, M, W): Lg = 4L + 8W = 928 = 32 x 29, 496 = 16 x 31, 544 = 32 x 17, 992 = 32 x 31,
# 528 = 16 x 33, 432 = 16 x 27, 800 = 32 x 25, 832 = 32 x 26, 416 = 16 x 26; odd M (7, 9):
# each sequence's last filter row is paired with zeros
SHAPES = [(5, 200, 8, 16), (7, 100, 16, 12), (4, 104, 16, 16), (3, 216, 16, 16), (5, 100, 16, 16),
          (5, 100, 8, 4), (3, 168, 16, 16), (5, 200, 16, 4), (4, 96, 8, 4), (5, 100, 7, 16),
          (3, 200, 9, 16)]


@pytest.mark.parametrize("shape", SHAPES)
def test_row_transforms_against_oracle_and_cufft(pkg, built_lib, monkeypatch, shape):
    N, L, M, fs = shape
    synth = pkg.synth
    bases, _, _ = synth.plant_dataset(29, N, L, [8], [0.4])
    S = synth.onehot(bases)
    Lg = 4 * L + 8 * fs
    X0 = synth.init_X0(9, N, M, Lg)
    D0 = synth.init_D0_unit_norm(9, M, Lg, 4 * fs)
    ref = O.init_cdl(S, M, fs, 1.0, 100.0, 0.1, X0=X0, D0=D0)
    DX_init = ref.DX.copy()
    objs_ref = O.run_outer(ref, 1)
    setup = pkg.CDLSetup(M=M, filter_size=fs, lambda_=0.1, rho=1.0, sigma=100.0)
    fields = ("X", "DX", "d", "g1", "g3", "G1", "G3", "Td", "G2", "g2")
    out = {}
    for v in ("1", "0"):
        monkeypatch.setenv("CDLGB_ROWFFT", v)
        with pkg.init_cdl(setup, S, X0=X0, D0=D0, fft_mode=2) as c:
            r = {"DX_init": c.get("DX")}
            r["objs"] = pkg.run_outer(c, 1)
            r.update({f: c.get(f) for f in fields})
            r["fft_calls"] = c.profile_read()["fft_calls"]
            out[v] = r
    row, cu = out["1"], out["0"]
    assert row["fft_calls"] == 0          # no cuFFT plan or call on this path
    assert cu["fft_calls"] > 0
    # the initial DX is transforms only (no iteration to amplify rounding): the register
    # FFT is as accurate as cuFFT there
    e_row, e_cu = rel(row["DX_init"], DX_init), rel(cu["DX_init"], DX_init)
    assert e_row < 1e-5 and e_row <= max(2.0 * e_cu, 1e-6), (e_row, e_cu)
    assert rel(row["DX_init"], cu["DX_init"]) < 1e-5
    np.testing.assert_allclose(row["objs"], objs_ref, rtol=TOL_OBJ)
    np.testing.assert_allclose(row["objs"], cu["objs"], rtol=TOL_OBJ)
    for f in fields:
        assert rel(row[f], getattr(ref, f)) < TOL_X, f
        assert rel(row[f], cu[f]) < 2 * TOL_X, f
