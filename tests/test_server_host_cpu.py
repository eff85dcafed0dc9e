"""The training server's host logic (csrc/server.cpp) on a machine without a GPU: every
training fails at cdlgb_create, so each request runs through admission, a worker, the
failure path and release without device work.  Covers the request life cycle and its
timestamps, polls concurrent with submissions from several threads, admission refusal
by footprint, the friendly-length padding, and argument errors.  Skipped where a GPU is present (the
trainings would then succeed; tests/test_serve_gpu.py covers that side)."""
import threading

import numpy as np
import pytest


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


pytestmark = pytest.mark.skipif(_has_gpu(), reason="trainings succeed on a GPU")

ECUDA, EINVAL, ENOMEM_BUDGET, ESTATE = -3, -1, -2, -5
BUDGET = 8 << 30


def _data(pkg, seed, N=6, L=40):
    bases, _, _ = pkg.synth.plant_dataset(seed, N, L, [6], [0.5])
    return pkg.synth.onehot(bases)


def _setup(pkg):
    return pkg.CDLSetup(M=4, filter_size=2)


def test_failed_trainings_are_reported_and_released(pkg, built_lib):
    from cdlmotif_gb300 import serve
    with serve.Server(_setup(pkg), slots=2, hbm_budget=BUDGET, iter_num=1) as srv:
        ids = [srv.submit(_data(pkg, s)) for s in range(5)]
        assert len(set(ids)) == 5
        for rid in ids:
            info = srv.poll(rid, wait_ms=-1)
            assert info["state"] == "failed" and info["status"] == ECUDA
            assert info["error"].startswith("cdlgb_create: device 0:")   # the worker's reason
            assert 0 <= info["t_submit"] <= info["t_admit"] <= info["t_done"] <= info["t_now"]
            assert info["N"] == 6 and info["L4"] == 160 and info["footprint_bytes"] > 0
            with pytest.raises(pkg.CDLGBError) as e:
                srv.fetch(rid)
            assert e.value.status == ESTATE
            srv.release(rid)
            with pytest.raises(pkg.CDLGBError) as e:
                srv.poll(rid)
            assert e.value.status == EINVAL
        assert srv.stats() == {"pending": 0, "running": 0, "in_use": 0, "budget": BUDGET}


def test_results_published_with_the_final_state(pkg, built_lib):
    """Four threads submit while a fifth polls every known request without waiting, and
    nothing fails or crashes; a request seen pending or running carries no result fields
    yet (status 0, no message, t_done -1) -- here the failures are immediate, so such
    states are seldom seen (tests/test_serve_gpu.py sees them during real trainings);
    every request ends failed with its status and message."""
    from cdlmotif_gb300 import serve
    data = [_data(pkg, s) for s in range(4)]
    with serve.Server(_setup(pkg), slots=3, hbm_budget=BUDGET, iter_num=1) as srv:
        ids, lock, done = [], threading.Lock(), threading.Event()
        errors = []

        def submitter(k):
            try:
                for j in range(6):
                    rid = srv.submit(data[(k + j) % 4])
                    with lock:
                        ids.append(rid)
            except Exception as e:          # reported below
                errors.append(e)

        seen_unfinished = []

        def poller():
            try:
                while not done.is_set():
                    with lock:
                        cur = list(ids)
                    for rid in cur:
                        info = srv.poll(rid, wait_ms=0)
                        if info["state"] in ("pending", "running"):
                            seen_unfinished.append(info)
            except Exception as e:
                errors.append(e)

        pt = threading.Thread(target=poller)
        pt.start()
        th = [threading.Thread(target=submitter, args=(k,)) for k in range(4)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        for rid in ids:
            assert srv.poll(rid, wait_ms=-1)["state"] == "failed"
        done.set()
        pt.join()
        assert not errors, errors
        assert len(set(ids)) == 24
        for info in seen_unfinished:
            assert info["status"] == 0 and info["error"] is None and info["t_done"] == -1.0
            assert info["M"] == 0 and info["outer_done"] == 0
        for rid in ids:
            info = srv.poll(rid)
            assert info["status"] == ECUDA and info["error"]
            srv.release(rid)
        assert srv.stats()["in_use"] == 0


def test_admission_refuses_what_never_fits(pkg, built_lib):
    from cdlmotif_gb300 import serve
    S = _data(pkg, 1)
    fp = serve.footprint_bytes(_setup(pkg), S.shape[1] // 4, S.shape[0])
    with serve.Server(_setup(pkg), slots=1, hbm_budget=fp - 1, iter_num=1) as srv:
        with pytest.raises(pkg.CDLGBError) as e:
            srv.submit(S)
        assert e.value.status == ENOMEM_BUDGET and "budget" in str(e.value)
        assert srv.stats()["pending"] == 0
    with serve.Server(_setup(pkg), slots=1, hbm_budget=fp, iter_num=1) as srv:
        assert srv.poll(srv.submit(S), wait_ms=-1)["footprint_bytes"] == fp


@pytest.mark.parametrize("L", [43, 101, 150])
def test_friendly_padding_of_submissions(pkg, built_lib, L):
    """With pad_friendly the server pads each sequence to the length the Python mirror
    (serve.friendly_length) names, for one-hot and FASTA submissions alike."""
    from cdlmotif_gb300 import serve
    setup = pkg.CDLSetup(M=4, filter_size=16)
    bases, _, _ = pkg.synth.plant_dataset(3, 4, L, [6], [0.5])
    Lp = serve.friendly_length(L, 16)
    with serve.Server(setup, slots=1, hbm_budget=BUDGET, iter_num=1, pad_friendly=True) as srv:
        a = srv.poll(srv.submit(pkg.synth.onehot(bases)), wait_ms=-1)
        b = srv.poll(srv.submit_fasta(pkg.synth.to_fasta(bases)), wait_ms=-1)
    assert a["L4"] == b["L4"] == 4 * Lp and a["N"] == b["N"] == 4


def test_bad_arguments(pkg, built_lib):
    from cdlmotif_gb300 import serve
    with pytest.raises(pkg.CDLGBError) as e:
        serve.Server(_setup(pkg), slots=0, hbm_budget=BUDGET)
    assert e.value.status == EINVAL
    with serve.Server(_setup(pkg), slots=1, hbm_budget=BUDGET, iter_num=1) as srv:
        with pytest.raises(pkg.CDLGBError) as e:
            srv.submit(np.zeros((3, 6), np.float32))        # 4L not a multiple of 4
        assert e.value.status == EINVAL
        with pytest.raises(pkg.CDLGBError) as e:
            srv.poll(12345)
        assert e.value.status == EINVAL
        with pytest.raises(pkg.CDLGBError) as e:
            srv.release(12345)
        assert e.value.status == EINVAL


def test_destroy_with_requests_queued(pkg, built_lib):
    """Closing the server while requests wait drops them and returns."""
    from cdlmotif_gb300 import serve
    srv = serve.Server(_setup(pkg), slots=1, hbm_budget=BUDGET, iter_num=1)
    for s in range(8):
        srv.submit(_data(pkg, s))
    srv.close()


_FASTA = {
    "multi-line records, lower case": b">a\nACGTAC\nGTAC\n>b desc\nacgtacgtac\n>c\nTTTTGGGGCC\n",
    "records with N dropped": b">a\nACGTN\n>b\nACGTA\n>c\nacgtn\n>d\nCCCCA\n",
    "empty chunks and no final newline": b">>a\nACGT\n>\n>b\nTTGA",
    "ragged lengths": b">a\nACGTACGT\n>b\nACG\n>c\nGGGGCCCC\n",
    "max entries after the N filter": b">a\nAAAN\n>b\nACGT\n>c\nCCCC\n>d\nGGGG\n>e\nTTTT\n",
}


@pytest.mark.parametrize("name", sorted(_FASTA))
def test_fasta_submissions_match_the_oracle_reader(pkg, built_lib, name):
    """The server parses FASTA submissions on the host by read_fasta's rules
    (src/LOAD/read.jl:2-28): its dataset sizes equal the oracle reader's."""
    from cdlmotif_gb300 import serve
    from oracle import search_oracle as SO
    text = _FASTA[name]
    cap = 3 if name.startswith("max") else 10000
    S_ref, reads = SO.read_fasta_onehot(text, cap)
    with serve.Server(_setup(pkg), slots=1, hbm_budget=BUDGET, iter_num=1) as srv:
        info = srv.poll(srv.submit_fasta(text, cap), wait_ms=-1)
    assert (info["N"], info["L4"]) == S_ref.shape, (name, reads)


@pytest.mark.parametrize("text", [b">a\r\nACGT\r\n>b\r\nACGT\r\n",   # CR kept, as split("\n") keeps it
                                  b">a\nACGU\n",                    # not a base
                                  b">a\nNNNN\n>b\nACGN\n",          # every record dropped
                                  b"", b">a\n\n>b\nACGT\n"])       # nothing, or an empty first record
def test_fasta_submissions_rejected(pkg, built_lib, text):
    """Inputs the reference's reader fails on (a character dummy[] has no entry for) or
    that leave no usable first record are refused at submission, before any device work."""
    from cdlmotif_gb300 import serve
    with serve.Server(_setup(pkg), slots=1, hbm_budget=BUDGET, iter_num=1) as srv:
        with pytest.raises(pkg.CDLGBError) as e:
            srv.submit_fasta(text)
        assert e.value.status == EINVAL and str(e.value)
        assert srv.stats()["pending"] == 0


def test_serve_stream_collects_refusals_and_failures(pkg, built_lib):
    """The request replay behind `bench.py --serve` (serve.serve_stream): arrivals spaced
    in time, one-hot and FASTA requests, one dataset refused at submission for its
    footprint and the rest failing here; every request is accounted for and the
    latency figures are empty rather than made up."""
    import math
    from cdlmotif_gb300 import serve
    setup = _setup(pkg)
    small = [_data(pkg, s) for s in range(3)]
    big = _data(pkg, 9, N=400, L=120)
    fp_small, fp_big = serve.footprint_bytes(setup, 40, 6), serve.footprint_bytes(setup, 120, 400)
    budget = (fp_small + fp_big) // 2          # the small ones fit, the big one never does
    assert fp_small <= budget < fp_big
    bases, _, _ = pkg.synth.plant_dataset(4, 5, 40, [6], [0.5])
    reqs = [(0.0, small[0]), (0.02, big), (0.04, small[1]),
            (0.06, pkg.synth.to_fasta(bases)), (0.08, small[2])]
    res = serve.serve_stream(setup, reqs, slots=2, iter_num=1, hbm_budget=budget)
    assert res["requests"] == 5 and res["completed"] == 0 and res["results"] == {}
    msgs = res["rejected"]
    assert len(msgs) == 5
    assert sum("budget" in m for m in msgs) == 1
    assert sum(m.startswith("cdlgb_create") for m in msgs) == 4
    assert math.isnan(res["p50_s"]) and math.isnan(res["p99_s"])
    assert res["datasets_per_hr"] is None and res["mean_queue_s"] is None
