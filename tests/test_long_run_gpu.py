"""Long runs on the N=1000/L=100/K=16/W=12 workload (Lg = 496): the float32 CUDA path's
distance from an all-FP64 reference against the distance of the reference's own
statement order evaluated in float32 (oracle/torch_admm.py, full complex FFTs), after
10 outer iterations (150 X-steps, 10 D-steps) -- through the C ABI.

Why an envelope and not the 1e-4 tolerance: with lambda 0.1 and rho 1 this ADMM
amplifies rounding differences by roughly 1.3x per outer iteration, so every float32
evaluation, the reference's own included, drifts from FP64 past 1e-4 within a few outer
iterations (measured: X 3e-4 at 10, 5e-3 at 20, O(1) by 50).  The test holds the CUDA
path to 2.5x the reference order's own float32 drift, and the objective to the same."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ENVELOPE = 2.5
FIELDS = ("X", "X_best", "d", "D_best", "G1")


def test_ten_outer_iterations_within_float32_envelope(pkg, built_lib):
    torch = pytest.importorskip("torch")
    from oracle.torch_admm import FP64Reference, LiteralADMM
    synth = pkg.synth
    N, L, M, fs = 1000, 100, 16, 12
    bases, _, _ = synth.plant_dataset(11, N, L, [10, 10], [0.3, 0.3])
    S = synth.onehot(bases)
    Lg = 4 * L + 8 * fs
    X0 = synth.init_X0(1, N, M, Lg)
    D0 = synth.init_D0_unit_norm(1, M, Lg, 4 * fs)
    dev = "cuda:0"
    ref = FP64Reference(S, X0, D0, M, fs, 1.0, 100.0, 0.1, device=dev)
    lit = LiteralADMM(S, X0, D0, M, fs, 1.0, 100.0, 0.1, device=dev, dtype=torch.float32)

    def rel(a, b):
        a = torch.as_tensor(a).to(dev, torch.float64)
        return float((a - b).norm() / b.norm())

    setup = pkg.CDLSetup(M=M, filter_size=fs, lambda_=0.1, rho=1.0, sigma=100.0)
    with pkg.init_cdl(setup, S, X0=X0, D0=D0) as c:
        for it in range(1, 11):
            o = float(pkg.run_outer(c, 1)[0])
            o64 = ref.run_outer(1)[0]
            ol = lit.run_outer(1)[0]
            if it not in (5, 10):
                continue
            gap, gap_l = abs(o - o64) / abs(o64), abs(ol - o64) / abs(o64)
            assert gap <= ENVELOPE * gap_l + 1e-6, (it, gap, gap_l)
            for f in FIELDS:
                e = rel(getattr(c, f), getattr(ref, f))
                el = rel(getattr(lit, f), getattr(ref, f))
                assert e <= ENVELOPE * el + 1e-5, (it, f, e, el)
