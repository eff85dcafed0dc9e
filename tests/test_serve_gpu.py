"""Serving: datasets admitted while others run give the same result as alone."""
import numpy as np
import pytest



def _datasets(pkg):
    synth = pkg.synth
    out = []
    for i, (N, L) in enumerate([(60, 40), (150, 30), (40, 60), (90, 44)]):
        bases, _, _ = synth.plant_dataset(40 + i, N, L, [6], [0.5])
        out.append(synth.onehot(bases))
    return out


@pytest.mark.gpu
def test_results_same_alone_and_in_the_mix(pkg, built_lib):
    from cdlmotif_gb300 import serve
    setup = pkg.CDLSetup(M=6, filter_size=3, lambda_=0.1, rho=1.0, sigma=100.0)
    data = _datasets(pkg)
    alone = [serve.run_training(setup, d, iter_num=2, seed=7, device=0) for d in data]
    res = serve.serve_stream(setup, [(0.0, d) for d in data], slots=4, iter_num=2, seed=7,
                             hbm_budget=8 << 30)
    assert res["completed"] == len(data) and not res["rejected"]
    for i, a in enumerate(alone):
        b = res["results"][i]
        np.testing.assert_array_equal(a["D_best"], b["D_best"])
        np.testing.assert_array_equal(a["objs"], b["objs"])
        assert a["code_thresh"] == b["code_thresh"]


@pytest.mark.gpu
def test_admission_by_footprint(pkg, built_lib):
    from cdlmotif_gb300 import serve
    setup = pkg.CDLSetup(M=4, filter_size=2)
    data = _datasets(pkg)[:2]
    fp = serve.footprint_bytes(setup, 40, 60)
    res = serve.serve_stream(setup, [(0.0, d) for d in data], slots=2, iter_num=1, seed=1,
                             hbm_budget=fp // 2)
    assert res["completed"] == 0 and len(res["rejected"]) == 2


@pytest.mark.parametrize("L", [50, 101, 333, 999])
def test_friendly_length(pkg, L):
    from cdlmotif_gb300 import serve
    Lp = serve.friendly_length(L, 16)
    n = 4 * Lp + 128
    assert Lp >= L and n % 16 == 0
    for p in (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31):
        while n % p == 0:
            n //= p
    assert n == 1
