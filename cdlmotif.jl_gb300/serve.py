"""Continuous-batching request loop for many CDL trainings on one GPU.

The reference processes FASTA files one after another (find_motifs_fasta_folder,
src/CDLmotif.jl:84-93), each through cdl_optimize (src/WRAPPER/wrap.jl:1-32).  Here
requests (one dataset each) arrive at any time and are admitted while others are on
the GPU: a request takes a slot when one is free and its device footprint
(cdlgb_footprint: ADMM state + scratch for its N and L) fits the HBM budget left by
the requests in flight; otherwise it waits in arrival order.  Every admitted request
runs on its own context (own CUDA stream, state resident until it finishes), so the
kernels of different datasets overlap on the device; the ctypes calls release the
GIL, so one host thread per slot is enough to keep them fed.

Because every kernel is deterministic and a context shares no device memory with
another, a dataset's result does not depend on what else is in flight.
"""
from __future__ import annotations

import ctypes as C
import queue
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from . import (CDLSetup, CDLGBError, init_cdl, code_update, dict_update, update_best,
               code_threshold)


def footprint_bytes(setup: CDLSetup, L: int, N: int, fft_mode: int = 0) -> int:
    p = setup.params(fft_mode=fft_mode)
    b = C.c_uint64()
    st = _lib.lib().cdlgb_footprint(C.byref(p), int(L), int(N), C.byref(b))
    if st != 0:
        raise CDLGBError(st, "cdlgb_footprint")
    return int(b.value)


# transform lengths of the multi-iteration X-step kernel's variants (csrc/xiter.cu)
REGISTER_LG = (496, 544, 608, 736, 928, 992)


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


@dataclass
class Request:
    rid: int
    data: np.ndarray                   # (N, 4L) one-hot
    arrival: float = 0.0               # seconds on the server clock
    admitted: float = 0.0
    done: float = 0.0
    footprint: int = 0
    result: dict = field(default_factory=dict)
    error: str | None = None


class Server:
    """Admits requests by HBM footprint into at most `slots` concurrent trainings."""

    def __init__(self, setup: CDLSetup, slots: int = 8, hbm_budget: int = 0, device: int = 0,
                 iter_num: int | None = None, seed: int = 0):
        self.setup = setup
        self.slots = slots
        self.device = device
        self.iter_num = setup.iter_num if iter_num is None else iter_num
        self.seed = seed
        if hbm_budget <= 0:
            import torch  # noqa: F401  (only for the free-memory query)
            free, _total = torch.cuda.mem_get_info(device)
            hbm_budget = int(free * 0.85)
        self.budget = hbm_budget
        self.in_use = 0
        self.cv = threading.Condition()
        self.pending: list[Request] = []
        self.running = 0
        self.work: queue.Queue = queue.Queue()
        self.finished: list[Request] = []
        self.t0 = time.perf_counter()
        self.stop = False
        self.threads = [threading.Thread(target=self._worker, daemon=True) for _ in range(slots)]
        for t in self.threads:
            t.start()
        self.admitter = threading.Thread(target=self._admit_loop, daemon=True)
        self.admitter.start()

    def now(self) -> float:
        return time.perf_counter() - self.t0

    def submit(self, req: Request):
        req.arrival = self.now()
        req.footprint = footprint_bytes(self.setup, req.data.shape[1] // 4, req.data.shape[0])
        with self.cv:
            if req.footprint > self.budget:
                req.error = f"needs {req.footprint / 1e9:.1f} GB > budget {self.budget / 1e9:.1f} GB"
                req.done = self.now()
                self.finished.append(req)
            else:
                self.pending.append(req)
            self.cv.notify_all()

    def _admit_loop(self):
        while True:
            with self.cv:
                while not self.stop and not (self.pending and self.running < self.slots and
                                             self.in_use + self.pending[0].footprint <= self.budget):
                    self.cv.wait(0.05)
                if self.stop and not self.pending:
                    return
                if not self.pending:
                    continue
                req = self.pending.pop(0)
                self.in_use += req.footprint
                self.running += 1
                req.admitted = self.now()
            self.work.put(req)

    def _worker(self):
        while True:
            req = self.work.get()
            if req is None:
                return
            try:
                req.result = run_training(self.setup, req.data, self.iter_num, self.seed,
                                          self.device)
            except CDLGBError as e:
                req.error = str(e)
            req.done = self.now()
            with self.cv:
                self.in_use -= req.footprint
                self.running -= 1
                self.finished.append(req)
                self.cv.notify_all()

    def drain(self, n_expected: int, timeout: float = 3600.0) -> list[Request]:
        t_end = time.perf_counter() + timeout
        with self.cv:
            while len(self.finished) < n_expected and time.perf_counter() < t_end:
                self.cv.wait(0.1)
        return list(self.finished)

    def close(self):
        with self.cv:
            self.stop = True
            self.cv.notify_all()
        self.admitter.join()
        for _ in self.threads:
            self.work.put(None)
        for t in self.threads:
            t.join()


def run_training(setup: CDLSetup, data: np.ndarray, iter_num: int, seed: int, device: int) -> dict:
    """One cdl_optimize training (src/WRAPPER/wrap.jl:5-12) of one dataset: init, iter_num
    outer iterations, code threshold; returns D_best, objectives and the threshold."""
    c = init_cdl(setup, data, seed=seed, device=device)
    try:
        objs = []
        for _ in range(iter_num):
            code_update(c, setup.csc_iter_num)
            o, _ = update_best(c)
            dict_update(c, setup.cdl_iter_num)
            objs.append(o)
        return {"D_best": c.D_best, "objs": np.array(objs), "code_thresh": code_threshold(c),
                "N": c.N, "L4": c.L}
    finally:
        c.close()


def percentile(v, q):
    return float(np.percentile(np.asarray(v, np.float64), q)) if len(v) else float("nan")


def serve_stream(setup: CDLSetup, requests: list[tuple[float, np.ndarray]], slots: int = 8,
                 iter_num: int = 3, seed: int = 0, device: int = 0, hbm_budget: int = 0) -> dict:
    """Replays (arrival offset s, one-hot data) requests against a Server, sleeping until
    each arrival; returns latency percentiles and throughput."""
    srv = Server(setup, slots=slots, iter_num=iter_num, seed=seed, device=device,
                 hbm_budget=hbm_budget)
    t0 = srv.now()
    for i, (t_arr, data) in enumerate(requests):
        delay = t_arr - (srv.now() - t0)
        if delay > 0:
            time.sleep(delay)
        srv.submit(Request(rid=i, data=data))
    done = srv.drain(len(requests))
    srv.close()
    ok = [r for r in done if r.error is None]
    lat = [r.done - r.arrival for r in ok]
    span = max(r.done for r in done) - t0 if done else float("nan")
    return {"requests": len(requests), "completed": len(ok),
            "rejected": [r.error for r in done if r.error],
            "p50_s": percentile(lat, 50), "p99_s": percentile(lat, 99),
            "mean_queue_s": float(np.mean([r.admitted - r.arrival for r in ok])) if ok else None,
            "makespan_s": span, "datasets_per_hr": 3600.0 * len(ok) / span if span > 0 else None,
            "results": {r.rid: r.result for r in ok}}
