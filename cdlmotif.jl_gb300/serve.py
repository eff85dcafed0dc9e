"""Continuous-batching training server: a thin wrapper of the C ABI's cdlgb_server_*.

The reference processes FASTA files one after another (find_motifs_fasta_folder,
src/CDLmotif.jl:84-93), each through cdl_optimize (src/WRAPPER/wrap.jl:1-32).  The
library's server (csrc/server.cpp) admits requests (one dataset each) while others are
on the GPU: a request takes a slot when one is free and its device footprint
(cdlgb_footprint: ADMM state + scratch for its N and L) fits the HBM budget left by
the requests in flight, in arrival order.  Every admitted request runs on its own
context (own CUDA stream, state resident until it finishes) on one of the server's
worker threads, so the kernels of different datasets overlap on the device.

Because every kernel is deterministic and a context shares no device memory with
another, a dataset's result does not depend on what else is in flight.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import RequestInfo, ServerConfig, ptr
from . import CDL, CDLSetup, CDLGBError, init_cdl, code_update, dict_update, update_best, code_threshold

STATES = {0: "pending", 1: "running", 2: "done", 3: "failed"}


def footprint_bytes(setup: CDLSetup, L: int, N: int, fft_mode: int = 0) -> int:
    p = setup.params(fft_mode=fft_mode)
    b = C.c_uint64()
    st = _lib.lib().cdlgb_footprint(C.byref(p), int(L), int(N), C.byref(b))
    if st != 0:
        raise CDLGBError(st, "cdlgb_footprint")
    return int(b.value)


# transform lengths of the multi-iteration X-step kernel's variants (csrc/xiter.cu)
REGISTER_LG = (288, 320, 336, 352, 368, 384, 400, 416, 432, 448, 464, 480, 496, 528, 544, 576, 608,
               640, 672, 704, 736, 768, 800, 832, 864, 896, 928, 960, 992)


def friendly_length(L: int, filter_size: int) -> int:
    """A padded length L' >= L for serving: the smallest whose transform length
    4L' + 8W is one of the multi-iteration kernel's (REGISTER_LG) if that costs at most
    8 % more transform columns, else the smallest whose transform length factors into
    primes <= 31 with a power of two of at least 16 (the generic in-kernel FFTs)."""
    def ok(n):
        if n % 16:
            return False
        for p in (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31):
            while n % p == 0:
                n //= p
        return n == 1
    lg = 4 * L + 8 * filter_size
    for n in REGISTER_LG:
        if lg <= n <= 1.08 * lg and (n - 8 * filter_size) % 4 == 0:
            return (n - 8 * filter_size) // 4
    Lp = L
    while not ok(4 * Lp + 8 * filter_size):
        Lp += 1
    return Lp


def pad_onehot(S: np.ndarray, L: int, Lp: int) -> np.ndarray:
    """Pad sequences of L bases to Lp with uniform 'N-like' columns of zeros."""
    N = S.shape[0]
    out = np.zeros((N, 4 * Lp), np.float32)
    out[:, : 4 * L] = S
    return out


class Server:
    """The library's training server (cdlgb_server_create): `slots` trainings in flight
    at most, admitted by footprint within `hbm_budget` bytes (0 = 85 % of free device
    memory), each `iter_num` outer iterations from `seed`."""

    def __init__(self, setup: CDLSetup, slots: int = 8, hbm_budget: int = 0, device: int = 0,
                 iter_num: int | None = None, seed: int = 0, keep_codes: bool = False,
                 pad_friendly: bool = False):
        L = _lib.lib()
        self.setup = setup
        self._p = setup.params(device=device)
        cfg = ServerConfig(slots=int(slots), device=int(device),
                           iter_num=int(setup.iter_num if iter_num is None else iter_num),
                           keep_codes=int(bool(keep_codes)), pad_friendly=int(bool(pad_friendly)),
                           hbm_budget_bytes=int(hbm_budget),
                           seed=int(seed) & (2**64 - 1))
        h = C.c_void_p()
        st = L.cdlgb_server_create(C.byref(self._p), C.byref(cfg), C.byref(h))
        if st != 0:
            raise CDLGBError(st, L.cdlgb_server_last_error(None).decode())
        self._h = h
        self.iter_num = cfg.iter_num

    def _check(self, st):
        if st != 0:
            msg = _lib.lib().cdlgb_server_last_error(self._h)
            raise CDLGBError(st, msg.decode() if msg else "")

    def submit(self, data: np.ndarray) -> int:
        """Queue one dataset, (N, 4L) one-hot; returns its request id.  Raises
        CDLGBError(ENOMEM_BUDGET) when it can never fit."""
        S = np.ascontiguousarray(data, np.float32)
        rid = C.c_int64()
        self._check(_lib.lib().cdlgb_server_submit(self._h, ptr(S, C.c_float), S.shape[1],
                                                   S.shape[0], C.byref(rid)))
        return rid.value

    def submit_fasta(self, fasta, max_entries: int = 10000) -> int:
        """Queue one dataset given as FASTA text (str or bytes), parsed by the rules of
        read_fasta / data_2_dummy (src/LOAD/read.jl:2-28, src/LOAD/to_dummy.jl:27-38)."""
        text = fasta.encode() if isinstance(fasta, str) else bytes(fasta)
        rid = C.c_int64()
        self._check(_lib.lib().cdlgb_server_submit_fasta(self._h, text, len(text), int(max_entries),
                                                         C.byref(rid)))
        return rid.value

    def poll(self, rid: int, wait_ms: int = 0) -> dict:
        info = RequestInfo()
        self._check(_lib.lib().cdlgb_server_poll(self._h, int(rid), int(wait_ms), C.byref(info)))
        out = {k: getattr(info, k) for k, _ in RequestInfo._fields_ if k != "error"}
        out["state"] = STATES[info.state]
        out["error"] = info.error.decode() or None
        return out

    def fetch(self, rid: int, codes: bool = False) -> dict:
        info = self.poll(rid)
        M, Lg, N = info["M"], info["Lg"], info["N"]
        D = np.empty((M, Lg), np.float32)
        objs = np.zeros(max(info["outer_done"], 1), np.float64)
        X = np.empty((N, M, Lg), np.float32) if codes else None
        self._check(_lib.lib().cdlgb_server_fetch(
            self._h, int(rid), ptr(D, C.c_float), D.nbytes, ptr(objs, C.c_double), objs.size,
            ptr(X, C.c_float) if codes else None, X.nbytes if codes else 0))
        res = {"D_best": D, "objs": objs[:info["outer_done"]], "code_thresh": info["code_thresh"],
               "obj_best": info["obj_best"], "N": N, "L4": info["L4"]}
        if codes:
            res["X_best"] = X
        return res

    def release(self, rid: int):
        self._check(_lib.lib().cdlgb_server_release(self._h, int(rid)))

    def stats(self) -> dict:
        p, r = C.c_int32(), C.c_int32()
        u, b = C.c_uint64(), C.c_uint64()
        self._check(_lib.lib().cdlgb_server_stats(self._h, C.byref(p), C.byref(r), C.byref(u), C.byref(b)))
        return {"pending": p.value, "running": r.value, "in_use": u.value, "budget": b.value}

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().cdlgb_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_training(setup: CDLSetup, data: np.ndarray, iter_num: int, seed: int, device: int,
                 profile: bool = False) -> dict:
    """One cdl_optimize training (src/WRAPPER/wrap.jl:5-12) of one dataset on its own
    context: init, iter_num outer iterations, code threshold; returns D_best, objectives
    and the threshold (with `profile`, also the device time of all of it from the
    library's CUDA-event phase timers, device_ms: the data upload's copy and kernels,
    the initialisation, X-steps, D-steps, objectives and the code threshold)."""
    c = CDL(setup, device=device)
    try:
        if profile:
            c.profile(True)
        c.load_data(data)
        c.init_state(None, None, seed)
        objs = []
        for _ in range(iter_num):
            code_update(c, setup.csc_iter_num)
            o, _ = update_best(c)
            dict_update(c, setup.cdl_iter_num)
            objs.append(o)
        out = {"D_best": c.D_best, "objs": np.array(objs), "code_thresh": code_threshold(c),
               "N": c.N, "L4": c.L}
        if profile:
            pr = c.profile_read()
            out["device_ms"] = sum(pr[k][0] for k in ("setup", "xstep", "dstep", "objective", "threshold"))
        return out
    finally:
        c.close()


def percentile(v, q):
    return float(np.percentile(np.asarray(v, np.float64), q)) if len(v) else float("nan")


def serve_stream(setup: CDLSetup, requests: list[tuple[float, np.ndarray]], slots: int = 8,
                 iter_num: int = 3, seed: int = 0, device: int = 0, hbm_budget: int = 0,
                 keep_results: bool = True, pad_friendly: bool = False) -> dict:
    """Replays (arrival offset s, one-hot data (N, 4L) or FASTA text) requests against the
    library's server,
    sleeping until each arrival; returns latency percentiles and throughput (latency =
    finish - arrival on the server's clock)."""
    with Server(setup, slots=slots, iter_num=iter_num, seed=seed, device=device,
                hbm_budget=hbm_budget, pad_friendly=pad_friendly) as srv:
        t0 = time.perf_counter()
        ids, rejected = {}, []
        for i, (t_arr, data) in enumerate(requests):
            delay = t_arr - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
            try:
                ids[i] = srv.submit_fasta(data) if isinstance(data, (bytes, str)) else srv.submit(data)
            except CDLGBError as e:
                rejected.append(str(e))
        infos, results = {}, {}
        for i, rid in ids.items():
            infos[i] = srv.poll(rid, wait_ms=-1)
            if infos[i]["state"] == "done" and keep_results:
                results[i] = srv.fetch(rid)
            srv.release(rid)
    ok = [v for v in infos.values() if v["state"] == "done"]
    failed = [v["error"] for v in infos.values() if v["state"] != "done"]
    lat = [v["t_done"] - v["t_submit"] for v in ok]
    t_first = min((v["t_submit"] for v in infos.values()), default=0.0)
    span = max((v["t_done"] for v in ok), default=float("nan")) - t_first
    return {"requests": len(requests), "completed": len(ok), "rejected": rejected + failed,
            "p50_s": percentile(lat, 50), "p99_s": percentile(lat, 99),
            "mean_queue_s": float(np.mean([v["t_admit"] - v["t_submit"] for v in ok])) if ok else None,
            "makespan_s": span, "datasets_per_hr": 3600.0 * len(ok) / span if span > 0 else None,
            "results": results}
