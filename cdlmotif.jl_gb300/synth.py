"""Seeded synthetic DNA datasets with planted motifs.

The reference's simulation recipe (src/LOAD/sample.jl:139-172,
src/SETUP/SIM_setup.jl:14-35, src/SETUP/TYPE_setup.jl:10,16) is: i.i.d. uniform
ACGT background; motif PWM columns drawn from Dirichlet(0.1 * 1_4); each motif is
planted in a sequence with probability = its occupancy, at a uniform position,
reverse-complemented with probability 0.5.  This module follows that recipe with a
seeded numpy PCG64 generator (the reference is unseeded).  No public dataset is
involved.

The one-hot layout is the reference's ``dna2dummy`` (src/LOAD/to_dummy.jl:2-9):
base i of a sequence occupies rows 4(i-1)+1..4i, in A, C, G, T order.
"""
from __future__ import annotations

import numpy as np

ALPHABET = "ACGT"


def plant_dataset(seed: int, N: int, L: int, motif_widths, occupancies,
                  alpha: float = 0.1, p_revcomp: float = 0.5):
    """Returns (bases uint8 (N, L) in 0..3, motifs list of (4, w) PFMs, truth list of
    (k, n, pos0, revcomp))."""
    rng = np.random.Generator(np.random.PCG64(seed))
    bases = rng.integers(0, 4, size=(N, L), dtype=np.uint8)
    motifs = [rng.dirichlet(alpha * np.ones(4), size=int(w)).T for w in motif_widths]
    truth = []
    for k, (pfm, occ) in enumerate(zip(motifs, occupancies)):
        w = pfm.shape[1]
        if w > L:
            continue
        cum = np.cumsum(pfm, axis=0)
        hit = rng.random(N) < occ
        for n in np.nonzero(hit)[0]:
            u = rng.random(w)
            site = np.minimum((u[None, :] > cum).sum(axis=0), 3).astype(np.uint8)
            rc = rng.random() < p_revcomp
            if rc:
                site = (3 - site)[::-1]
            pos = int(rng.integers(0, L - w + 1))
            bases[n, pos:pos + w] = site
            truth.append((k, int(n), pos, bool(rc)))
    return bases, motifs, truth


def onehot(bases: np.ndarray) -> np.ndarray:
    """(N, L) base codes -> (N, 4L) float32 one-hot == Julia (4L, N) column-major."""
    N, L = bases.shape
    out = np.zeros((N, L, 4), np.float32)
    out[np.arange(N)[:, None], np.arange(L)[None, :], bases] = 1.0
    return out.reshape(N, 4 * L)


def to_fasta(bases: np.ndarray) -> str:
    lut = np.frombuffer(ALPHABET.encode(), np.uint8)
    lines = []
    for n in range(bases.shape[0]):
        lines.append(f">seq{n + 1}")
        lines.append(lut[bases[n]].tobytes().decode())
    return "\n".join(lines) + "\n"


def init_X0(seed: int, N: int, M: int, Lg: int) -> np.ndarray:
    """X0 as the reference draws it (src/SETUP/CDL_setup.jl:191-192): standard normal,
    zero unless (l-1) % 4 == 0.  Shape (N, M, Lg) float32."""
    rng = np.random.Generator(np.random.PCG64(seed ^ 0x5EED))
    X = rng.standard_normal((N, M, Lg), dtype=np.float32)
    X[..., (np.arange(Lg) % 4) != 0] = 0.0
    return X


def init_D0_unit_norm(seed: int, M: int, Lg: int, filter_len: int) -> np.ndarray:
    """Random-normal filters on rows 1..filter_len, each normalised to unit L2 norm.
    Shape (M, Lg) float32."""
    rng = np.random.Generator(np.random.PCG64(seed ^ 0xD1C7))
    D = np.zeros((M, Lg), np.float32)
    v = rng.standard_normal((M, filter_len))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    D[:, :filter_len] = v
    return D


# The workloads of the benchmark configurations, by name.
CONFIGS = {
    # N=1000, L=100, 2 motifs w=10 at 30 %, K=16 filters of 12 bases, lambda 0.1, rho 1.0
    "plain_n1000_l100_k16": dict(N=1000, L=100, M=16, filter_size=12, widths=[10, 10],
                                 occ=[0.3, 0.3], lam=0.1, rho=1.0, sigma=100.0, iters=50),
    # N=20000, L=200, 5 motifs w 8..20 at 10..40 %, K=64 filters of 16 bases
    "plain_n20000_l200_k64": dict(N=20000, L=200, M=64, filter_size=16,
                                  widths=[8, 11, 14, 17, 20], occ=[0.1, 0.175, 0.25, 0.325, 0.4],
                                  lam=0.1, rho=1.0, sigma=100.0, iters=100),
}
