"""Generate the golden fixtures in this folder from the CPU oracle.

The reference (Julia + CUDA.jl 3.9) cannot run here and its own test suite is
empty, so these fixtures are produced by the FP64 oracle (oracle/cdl_oracle.py,
oracle/search_oracle.py) on seeded inputs; the oracle itself is pinned by the
known-answer tests in tests/test_oracle_cpu.py.  Run from the repository root:

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import cdl_oracle as O          # noqa: E402
from oracle import search_oracle as SO      # noqa: E402


def onehot(rng, N, L):
    b = rng.integers(0, 4, (N, L))
    S = np.zeros((N, L, 4), np.float32)
    S[np.arange(N)[:, None], np.arange(L)[None], b] = 1
    return S.reshape(N, 4 * L)


def admm_case(name, seed, N, L, M, fs, lam, rho, sigma, outer, csc=15, cdl=1):
    rng = np.random.default_rng(seed)
    S = onehot(rng, N, L)
    gamma = 4 * fs
    Lg = 4 * L + 2 * gamma
    X0 = rng.standard_normal((N, M, Lg)).astype(np.float32)
    X0[..., np.arange(Lg) % 4 != 0] = 0
    D0 = np.zeros((M, Lg), np.float32)
    v = rng.standard_normal((M, gamma))
    D0[:, :gamma] = v / np.linalg.norm(v, axis=1, keepdims=True)
    c = O.init_cdl(S, M, fs, rho, sigma, lam, X0=X0, D0=D0)
    obj0 = c.obj_best
    objs = O.run_outer(c, outer, csc, cdl)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), S=S, X0=X0, D0=D0,
                        params=np.array([M, fs, lam, rho, sigma, outer, csc, cdl], np.float64),
                        obj0=obj0, objs=np.array(objs), X=c.X.astype(np.float32),
                        X_best=c.X_best.astype(np.float32), d=c.d.astype(np.float32),
                        G1=c.G1.astype(np.float32), G3=c.G3.astype(np.float32),
                        DX=c.DX.astype(np.float32), D_best=c.D_best.astype(np.float32),
                        obj_best=c.obj_best)


def scan_case(name, seed, N, L, K):
    rng = np.random.default_rng(seed)
    S = onehot(rng, N, L)
    lens = rng.integers(3, 12, K).astype(np.int32)
    pfms = [rng.dirichlet(0.3 * np.ones(4), size=w).T.astype(np.float32) for w in lens]
    pfms = [((p + np.float32(0.05)) / np.float32(1.2)).astype(np.float32) for p in pfms]
    pwms = [np.log2(p / np.float32(0.25)).astype(np.float32) for p in pfms]
    maxlen = int(lens.max())
    pw = np.zeros((K, 4, maxlen), np.float32)
    for k in range(K):
        pw[k, :, : lens[k]] = pwms[k]
    thresh = np.array([np.float32(0.25 * np.sum(np.max(p, axis=0))) for p in pwms], np.float32)
    pos_fwd = SO.scan_w_gpu_positions(pw, S, lens, thresh)
    pos, score, comp = SO.overlapping_scan(S, pwms, lens, thresh)
    counts, nseq = SO.count_matrices(S, pos, comp, lens)
    pfm_out = SO.counts_to_pfms(counts, nseq, lens)
    pfm_pad = np.zeros((K, 4, maxlen), np.float32)
    for k in range(K):
        pfm_pad[k, :, : lens[k]] = pfm_out[k]
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), S=S, pwms=pw, lens=lens,
                        thresh=thresh, pos_fwd=pos_fwd, pos=pos, score=score, comp=comp,
                        counts=counts, nseq=nseq, pfms=pfm_pad,
                        transfac=np.array(SO.transfac_text(pfm_out[0])),
                        transfac_c=np.array(SO.transfac_text(SO.pwm_complement(pfm_out[0]))))


if __name__ == "__main__":
    admm_case("admm_tiny", 1, N=8, L=12, M=3, fs=2, lam=0.1, rho=1.0, sigma=100.0, outer=3)
    admm_case("admm_small", 2, N=24, L=25, M=6, fs=4, lam=0.1, rho=1.0, sigma=100.0, outer=2)
    admm_case("admm_refdefaults", 3, N=16, L=20, M=4, fs=3, lam=0.01, rho=100.0, sigma=100.0,
              outer=2)
    scan_case("scan_small", 4, N=40, L=30, K=6)
    print("written:", sorted(f for f in os.listdir(HERE) if f.endswith(".npz")))
