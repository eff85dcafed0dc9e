"""Serving through the library's training server (cdlgb_server_*): datasets admitted
while others run give the same result as alone; admission by footprint; the request
calls from several host threads."""
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


@pytest.mark.gpu
def test_server_calls_from_threads(pkg, built_lib):
    """submit from four host threads at once, poll until done, fetch D_best, objectives
    and the codes (X_best), release; the results equal the single-context training."""
    import threading
    from cdlmotif_gb300 import serve
    setup = pkg.CDLSetup(M=6, filter_size=3, lambda_=0.1, rho=1.0, sigma=100.0)
    data = _datasets(pkg)
    ids = [None] * len(data)
    with serve.Server(setup, slots=3, iter_num=2, seed=5, hbm_budget=8 << 30, keep_codes=True) as srv:
        def sub(i):
            ids[i] = srv.submit(data[i])
        th = [threading.Thread(target=sub, args=(i,)) for i in range(len(data))]
        for t in th:
            t.start()
        for t in th:
            t.join()
        assert len(set(ids)) == len(data)
        for rid in ids:
            # the result fields are published with the final state only
            info = srv.poll(rid, wait_ms=0)
            if info["state"] in ("pending", "running"):
                assert info["status"] == 0 and info["error"] is None and info["t_done"] == -1.0
                assert info["M"] == 0 and info["outer_done"] == 0 and info["obj_best"] == 0.0
        for i, rid in enumerate(ids):
            info = srv.poll(rid, wait_ms=-1)
            assert info["state"] == "done", info
            assert info["N"] == data[i].shape[0] and info["outer_done"] == 2
            assert 0 <= info["t_submit"] <= info["t_admit"] <= info["t_done"]
            res = srv.fetch(rid, codes=True)
            c = pkg.init_cdl(setup, data[i], seed=5)
            with c:
                objs = pkg.run_outer(c, 2)
                np.testing.assert_array_equal(res["objs"], objs)
                np.testing.assert_array_equal(res["D_best"], c.D_best)
                np.testing.assert_array_equal(res["X_best"], c.X_best)
                assert res["code_thresh"] == pkg.code_threshold(c)
            srv.release(rid)
        st = srv.stats()
        assert st["pending"] == 0 and st["running"] == 0 and st["in_use"] == 0
        with pytest.raises(pkg.CDLGBError):
            srv.poll(ids[0])            # released


@pytest.mark.gpu
def test_server_refuses_what_never_fits(pkg, built_lib):
    from cdlmotif_gb300 import serve
    setup = pkg.CDLSetup(M=4, filter_size=2)
    d = _datasets(pkg)[0]
    fp = serve.footprint_bytes(setup, d.shape[1] // 4, d.shape[0])
    with serve.Server(setup, slots=1, iter_num=1, hbm_budget=fp - 1) as srv:
        with pytest.raises(pkg.CDLGBError) as e:
            srv.submit(d)
        assert e.value.status == -2
    with serve.Server(setup, slots=1, iter_num=1, hbm_budget=fp) as srv:
        rid = srv.submit(d)
        assert srv.poll(rid, wait_ms=-1)["state"] == "done"


@pytest.mark.gpu
def test_device_memory_comes_back(pkg, built_lib):
    """Contexts allocate stream-ordered from the library's device pool: after a
    training's context is destroyed (and the device synchronised) its memory is back,
    so repeated trainings do not grow the process's footprint; a server keeps what its
    finished datasets free for reuse while it lives and gives it back when it ends."""
    torch = pytest.importorskip("torch")
    from cdlmotif_gb300 import serve
    setup = pkg.CDLSetup(M=32, filter_size=16, lambda_=0.1, rho=1.0, sigma=100.0)
    bases, _, _ = pkg.synth.plant_dataset(5, 2000, 200, [10], [0.3])
    S = pkg.synth.onehot(bases)
    need = serve.footprint_bytes(setup, 200, 2000)
    slack = 128 << 20
    serve.run_training(setup, S, iter_num=1, seed=1, device=0)    # modules, tables, pinned slab
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        serve.run_training(setup, S, iter_num=1, seed=1, device=0)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] >= free0 - slack
    with serve.Server(setup, slots=2, iter_num=1, seed=1) as s:
        ids = [s.submit(S) for _ in range(3)]
        for rid in ids:
            assert s.poll(rid, wait_ms=-1)["state"] == "done"
        torch.cuda.synchronize()
        held = torch.cuda.mem_get_info()[0]
        assert held <= free0 - need // 2          # the pool keeps the freed blocks
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] >= free0 - slack
