"""CPU oracle for the CDLmotif convolutional-dictionary-learning ADMM.

TEST INFRASTRUCTURE ONLY.  This module is the checker that the CUDA product path
is compared against; only ``tests/``, ``__graft_entry__.smoke()`` and the CPU
baseline legs of ``bench.py`` may import it.  The product (``libcdlgb.so`` and
the host package) never calls into it.

Parity status: **parity unpinned**.  The reference (kchu25/CDLmotif.jl) is pure
Julia + CUDA.jl 3.9; neither Julia nor that CUDA.jl runs here, and the reference's
own test suite is empty (test/runtests.jl:4-6), so there are no reference golden
vectors to pin this restatement against.  It is pinned instead by known-answer
tests (Sherman-Morrison vs a dense solve, FFT products vs direct circular
convolution) and by the fixtures in tests/golden/, which this module generates.

What it restates, step by step and in the reference's order (full complex FFTs of
real arrays promoted to complex, inverse scaled by 1/L_gamma, real part kept):

* ``cdl`` constructor / ``init_cdl``        src/SETUP/CDL_setup.jl:165-283
* ``make_D_projector``                      src/SETUP/CDL_setup.jl:15-27
* ``enforce_dummy_code_constraint!``        src/SETUP/CDL_setup.jl:29-40
* ``rand_probvec``                          src/SETUP/CDL_setup.jl:58-68
* ``code_update!``                          src/CDL/train.jl:1-44
  (``shrink!``, ``projectionX!``, ``update_Y1!``, ``sherman_CSC_*``:
  src/CDL/csc_kernels.jl:8-95)
* ``dict_update!``                          src/CDL/train.jl:46-89
  (``sherman_CDL_RHS!``, ``sherman_CDL_combine``, ``projection2box!``,
  ``prox_simplex_zeros!``, ``update_g2!``: src/CDL/cdl_kernels.jl:2-77)
* ``update_best!``                          src/CDL/train.jl:91-98
* ``objective``                             src/SETUP/CDL_setup.jl:286
* ``cdl_optimize`` inner loop               src/WRAPPER/wrap.jl:1-32

Memory layout: a Julia column-major array of dims (Lg, M, N) is held here as a
C-order numpy array of shape (N, M, Lg) -- the same bytes.  (Lg, N) -> (N, Lg),
(Lg, M) -> (M, Lg), the one-hot data (4L, N) -> (N, 4L).
"""
from __future__ import annotations

import numpy as np


def make_D_projector(Lg: int, M: int, filter_len) -> np.ndarray:
    """src/SETUP/CDL_setup.jl:15-27 -- 1 on rows 1..filter_len[m] of column m."""
    P = np.zeros((M, Lg))
    for m in range(M):
        P[m, : int(filter_len[m])] = 1.0
    return P


def rand_probvec(rng: np.random.Generator, d: int) -> np.ndarray:
    """src/SETUP/CDL_setup.jl:59-66 -- uniform point on the (d-1)-simplex
    (sorted uniforms, differences)."""
    unif = rng.random(d - 1)
    w = np.zeros(d + 1)
    w[1:d] = np.sort(unif)
    w[d] = 1.0
    return np.diff(w)


def reference_D_init(rng, Lg: int, M: int, filter_len) -> np.ndarray:
    """src/SETUP/CDL_setup.jl:182-183 -- per 4-row group a simplex vector, masked by P_D."""
    P = make_D_projector(Lg, M, filter_len)
    D = np.stack([np.concatenate([rand_probvec(rng, 4) for _ in range(Lg // 4)]) for _ in range(M)])
    return P * D


def enforce_dummy_code_constraint(X: np.ndarray) -> np.ndarray:
    """src/SETUP/CDL_setup.jl:29-40 -- zero X[l,m,n] unless (l-1) % 4 == 0 (1-based)."""
    X = X.copy()
    mask = (np.arange(X.shape[-1]) % 4) != 0
    X[..., mask] = 0.0
    return X


def shrink(t: np.ndarray, lam) -> np.ndarray:
    """src/CDL/csc_kernels.jl:53-64 -- sign(t) * max(|t| - lambda, 0) (lambda, not lambda/rho)."""
    return np.sign(t) * np.maximum(np.abs(t) - lam, 0.0)


def projectionX(X: np.ndarray, y3: np.ndarray) -> np.ndarray:
    """src/CDL/csc_kernels.jl:68-82 -- X + y3 on rows (l-1) % 4 == 0, else 0."""
    Y3 = X + y3
    mask = (np.arange(X.shape[-1]) % 4) != 0
    Y3[..., mask] = 0.0
    return Y3


def projection2box(v: np.ndarray, P_D: np.ndarray) -> np.ndarray:
    """src/CDL/cdl_kernels.jl:37-51."""
    G = np.where(v >= 1, np.where(P_D != 0, 1.0, 0.0),
                 np.where(v <= 0, 0.0, np.where(P_D != 0, v, 0.0)))
    return G.astype(v.dtype)


def prox_simplex_zeros(v: np.ndarray, P_D: np.ndarray) -> np.ndarray:
    """src/CDL/cdl_kernels.jl:53-66, including the group-index quirk: for 1-based
    row l the group starts at i = 4*floor(l/4), so rows l = 4, 8, ... use the
    NEXT group of four (rows i+1..i+4)."""
    M, Lg = v.shape
    G = np.zeros_like(v)
    for l0 in range(Lg):
        if not np.any(P_D[:, l0] != 0):  # the group is only read on the support
            continue
        i = 4 * ((l0 + 1) // 4)          # 0-based start of rows i+1..i+4 (1-based)
        grp = v[:, i] + v[:, i + 1] + v[:, i + 2] + v[:, i + 3]
        val = v[:, l0] - 0.25 * (grp - 1.0)
        G[:, l0] = np.where(P_D[:, l0] != 0, val, 0.0)
    return G


class CDLState:
    """Field-for-field restatement of ``struct cdl`` (src/SETUP/CDL_setup.jl:70-163)."""


def _fft(a):
    return np.fft.fft(a, axis=-1)


def _ifft(a):
    return np.fft.ifft(a, axis=-1)


def init_cdl(S: np.ndarray, M: int, filter_size: int, rho: float, sigma: float, lam: float,
             X0: np.ndarray | None = None, D0: np.ndarray | None = None,
             rng: np.random.Generator | None = None, dtype=np.float64) -> CDLState:
    """``cdl{T,S,Q}(M, filter_len, rho, sigma, lambda, dat)`` -- src/SETUP/CDL_setup.jl:165-270,
    called by ``init_cdl`` (:273-283) with filter_len = 4*filter_size for every filter.

    ``S`` is the one-hot data, shape (N, 4L).  ``X0`` (N, M, Lg) and ``D0`` (M, Lg)
    replace the reference's unseeded ``CUDA.randn`` and ``rand_probvec`` draws so that
    both sides of a parity test start from the same point; ``X0`` still goes through
    ``enforce_dummy_code_constraint!`` and ``D0`` through the P_D mask, as in the
    constructor."""
    cdt = np.complex128 if dtype == np.float64 else np.complex64
    S = np.asarray(S, dtype=dtype)
    N, L4 = S.shape
    assert L4 % 4 == 0, "first dimension of dat must be multiple of 4s"
    filter_len = [4 * filter_size] * M
    gamma = max(filter_len)
    Lg = L4 + 2 * gamma
    rng = rng if rng is not None else np.random.default_rng(0)
    c = CDLState()
    c.N, c.M, c.L, c.gamma, c.Lg = N, M, L4, gamma, Lg
    c.filter_len = filter_len
    c.rho, c.sigma, c.lam = dtype(rho), dtype(sigma), dtype(lam)
    c.dtype, c.cdtype = dtype, cdt
    c.P_D = make_D_projector(Lg, M, filter_len).astype(dtype)
    if D0 is None:
        D = reference_D_init(rng, Lg, M, filter_len)
    else:
        D = np.asarray(D0, dtype=np.float64).reshape(M, Lg)
    D = (c.P_D * D).astype(dtype)
    if X0 is None:
        X = rng.standard_normal((N, M, Lg))
    else:
        X = np.asarray(X0, dtype=np.float64).reshape(N, M, Lg)
    X = enforce_dummy_code_constraint(X).astype(dtype)

    Dh = _fft(D.astype(cdt))
    Xh = _fft(X.astype(cdt))
    DoX = np.sum(Dh[None] * Xh, axis=1)
    c.DX = np.real(_ifft(DoX)).astype(dtype)
    c.dh = np.broadcast_to(Dh[None], (N, M, Lg)).astype(cdt)
    c.Td = np.zeros((N, Lg), dtype)
    c.d = np.real(_ifft(c.dh)).astype(dtype)
    c.X, c.Xh = X, Xh.astype(cdt)
    # mask W: (4L, Lg) selector with identity on columns gamma+1..gamma+4L
    c.WtW_diag = np.zeros(Lg, dtype)
    c.WtW_diag[gamma:gamma + L4] = 1.0
    c.WtS = np.zeros((N, Lg), dtype)
    c.WtS[:, gamma:gamma + L4] = S
    c.S = S
    c.Y1 = np.zeros((N, Lg), dtype)
    c.Y2 = X.copy()
    c.Y3 = X.copy()
    c.Y1h = _fft(c.Y1.astype(cdt))
    c.Y2h = _fft(c.Y2.astype(cdt))
    c.Y3h = c.Y2h.copy()
    c.y1 = c.Y1.copy()
    c.y2 = np.zeros((N, M, Lg), dtype)
    c.y3 = c.y2.copy()
    c.y1h = c.Y1h.copy()
    c.y2h = _fft(c.y2.astype(cdt))
    c.y3h = c.y2h.copy()
    c.G1 = D.copy()
    c.G2 = c.DX.copy()
    c.G3 = D.copy()
    c.G1h = _fft(c.G1.astype(cdt))
    c.G2h = _fft(c.G2.astype(cdt))
    c.G3h = c.G1h.copy()
    c.g1 = c.y2.copy()
    c.g2 = c.Y1.copy()
    c.g3 = c.y2.copy()
    c.g1h = c.y2h.copy()
    c.g2h = c.Y1h.copy()
    c.g3h = c.y2h.copy()
    c.D_best = c.G1.copy()
    c.X_best = c.Y3.copy()
    c.obj_best = objective(c)
    c.D0, c.X0 = D, X
    c.resid = np.zeros(13)
    return c


def WDX(c: CDLState) -> np.ndarray:
    """W*DX: rows gamma+1..gamma+4L of DX (the dense 0/1 gemm of src/CDL/train.jl:28)."""
    return c.DX[:, c.gamma:c.gamma + c.L]


def objective(c: CDLState) -> float:
    """src/SETUP/CDL_setup.jl:286 -- 0.5*||W*DX - S||^2 + lambda*sum|X| (accumulated in FP64)."""
    r = (WDX(c) - c.S).astype(np.float64)
    return float(0.5 * np.sum(r * r) + float(c.lam) * np.sum(np.abs(c.X.astype(np.float64))))


def cdl_obj(c: CDLState) -> float:
    """src/SETUP/CDL_setup.jl:285 -- 0.5*||W*Td - S||^2."""
    r = (c.Td[:, c.gamma:c.gamma + c.L] - c.S).astype(np.float64)
    return float(0.5 * np.sum(r * r))


def sherman_csc(G1h: np.ndarray, RHS: np.ndarray, k) -> np.ndarray:
    """sherman_CSC_dot! + sherman_CSC_combine! (src/CDL/csc_kernels.jl:19-49,
    train.jl:18-25): x = (RHS - conj(a) * sum_m(a/(sum|a|^2 + k)) RHS) / k, which
    solves (conj(a) a^T + k I) x = RHS per frequency.  G1h (M, Lg), RHS (N, M, Lg)."""
    dots = G1h * np.conj(G1h)
    sum_dots = np.sum(dots, axis=0, keepdims=True) + k
    At = G1h / sum_dots
    alpha = np.sum(At[None] * RHS, axis=1)
    return (RHS - alpha[:, None, :] * np.conj(G1h)[None]) / k


def sherman_cdl(Y3h: np.ndarray, RHS: np.ndarray, k) -> np.ndarray:
    """src/CDL/train.jl:52-60 with sherman_CDL_combine (cdl_kernels.jl:24-33): the same
    solve WITHOUT the final division by k (so the result is k times the solution of
    (conj(b) b^T + k I) x = RHS).  Y3h, RHS (N, M, Lg)."""
    dots = Y3h * np.conj(Y3h)
    sum_dots = np.sum(dots, axis=1, keepdims=True) + k
    X_cdl = Y3h / sum_dots
    beta = np.sum(X_cdl * RHS, axis=1)
    return RHS - beta[:, None, :] * np.conj(Y3h)


def code_update(c: CDLState, num_iter: int, sherman_const_csc: float = 2.0) -> None:
    """src/CDL/train.jl:1-44, statement by statement."""
    k = c.dtype(sherman_const_csc)
    for _ in range(num_iter):
        c.Y2 = shrink(c.X + c.y2, c.lam).astype(c.dtype)                     # :7
        c.Y2h = _fft(c.Y2.astype(c.cdtype))                                  # :8
        c.y1 = c.y1 + c.DX - c.Y1; c.y1h = _fft(c.y1.astype(c.cdtype))       # :12
        c.y2 = c.y2 + c.X - c.Y2; c.y2h = _fft(c.y2.astype(c.cdtype))        # :13
        c.y3 = c.y3 + c.X - c.Y3; c.y3h = _fft(c.y3.astype(c.cdtype))        # :14
        RHS = (np.conj(c.G1h)[None] * (c.Y1h - c.y1h)[:, None, :]           # :23 sherman_CSC_RHS!
               + (c.Y2h - c.y2h) + (c.Y3h - c.y3h))
        c.Xh = sherman_csc(c.G1h, RHS, k)                                    # :18-25
        c.X = np.real(_ifft(c.Xh)).astype(c.dtype)                           # :26
        c.DX = np.real(_ifft(np.sum(c.G1h[None] * c.Xh, axis=1))).astype(c.dtype)  # :27
        c.Y1 = ((c.WtS + c.rho * (c.DX + c.y1)) / (c.WtW_diag + c.rho)).astype(c.dtype)  # :35
        c.Y1h = _fft(c.Y1.astype(c.cdtype))                                  # :36
        c.Y3 = projectionX(c.X, c.y3).astype(c.dtype)                        # :40
        c.Y3h = _fft(c.Y3.astype(c.cdtype))                                  # :41
    c.resid[0:5] = x_residuals(c)


def x_residuals(c: CDLState) -> np.ndarray:
    """Primal residuals of the final iterate of a code update, in float64: what the next
    dual updates (src/CDL/train.jl:12-14) would add -- sum (X - shrink(X + y2))^2,
    sum (X - projectionX(X + y3))^2, sum (DX - Y1)^2 -- and sum X^2, sum DX^2."""
    X = c.X.astype(np.float64)
    r2 = X - shrink(c.X + c.y2, c.lam).astype(np.float64)
    r3 = X - projectionX(c.X, c.y3).astype(np.float64)
    r1 = c.DX.astype(np.float64) - c.Y1.astype(np.float64)
    return np.array([np.sum(r2 * r2), np.sum(r3 * r3), np.sum(r1 * r1), np.sum(X * X),
                     np.sum(c.DX.astype(np.float64) ** 2)])


def relative_residuals(r) -> dict:
    """The stopping test's five relative residuals from a 13-value residual record:
    primal of the code update (X - Y2, X - Y3 against |X|; DX - Y1 against |DX|), primal
    of the D-step (the g1, g3 increments against |d|; the g2 increment against |Td|) and
    the D-step's consensus dual residual (the change of G1, G3 against |G|)."""
    tiny = 1e-300
    return {"primal_x": np.sqrt((r[0] + r[1]) / max(r[3], tiny)),
            "primal_dx": np.sqrt(r[2] / max(r[4], tiny)),
            "primal_d": np.sqrt((r[5] + r[6]) / max(2.0 * r[8], tiny)),
            "primal_td": np.sqrt(r[7] / max(r[9], tiny)),
            "dual_d": np.sqrt((r[10] + r[11]) / max(r[12], tiny))}


def dict_update(c: CDLState, num_iter: int, sherman_const_cdl: float = 2.0) -> None:
    """src/CDL/train.jl:46-89, statement by statement (no 1/2 in the combine, cdl_kernels.jl:30)."""
    k = c.dtype(sherman_const_cdl)
    for _ in range(num_iter):
        c.Td = np.real(_ifft(np.sum(c.Y3h * c.dh, axis=1))).astype(c.dtype)  # :56-57 (old d-hat)
        RHS = (np.conj(c.Y3h) * (c.G2h - c.g2h)[:, None, :]                  # :58 sherman_CDL_RHS!
               + (c.G1h[None] - c.g1h) + (c.G3h[None] - c.g3h))
        c.dh = sherman_cdl(c.Y3h, RHS, k)                                    # :52-54,59-60
        c.d = np.real(_ifft(c.dh)).astype(c.dtype)                           # :61
        c.G2 = ((c.WtS + c.sigma * (c.Td + c.g2)) / (c.WtW_diag + c.sigma)).astype(c.dtype)  # :68
        c.G2h = _fft(c.G2.astype(c.cdtype))                                  # :69
        c.g1 = c.g1 + c.d - c.G1[None]; c.g1h = _fft(c.g1.astype(c.cdtype))  # :70
        c.g2 = c.g2 + c.Td - c.G2; c.g2h = _fft(c.g2.astype(c.cdtype))       # :71
        c.g3 = c.g3 + c.d - c.G3[None]; c.g3h = _fft(c.g3.astype(c.cdtype))  # :72
        d64, Td64 = c.d.astype(np.float64), c.Td.astype(np.float64)
        G1o, G3o = c.G1.astype(np.float64), c.G3.astype(np.float64)
        c.resid[5:10] = [np.sum((d64 - G1o[None]) ** 2), np.sum((d64 - G3o[None]) ** 2),
                         np.sum((Td64 - c.G2.astype(np.float64)) ** 2), np.sum(d64 * d64),
                         np.sum(Td64 * Td64)]
        v2 = (np.sum(c.d + c.g3, axis=0) / c.N).astype(c.dtype)              # :76
        c.G3 = projection2box(v2, c.P_D)                                     # :77
        c.G3h = _fft(c.G3.astype(c.cdtype))                                  # :78
        v1 = (np.sum(c.d + c.g1, axis=0) / c.N).astype(c.dtype)              # :83
        c.G1 = prox_simplex_zeros(v1, c.P_D).astype(c.dtype)                 # :84
        c.G1h = _fft(c.G1.astype(c.cdtype))                                  # :85
        G1n, G3n = c.G1.astype(np.float64), c.G3.astype(np.float64)
        c.resid[10:13] = [c.N * np.sum((G1n - G1o) ** 2), c.N * np.sum((G3n - G3o) ** 2),
                          c.N * (np.sum(G1n * G1n) + np.sum(G3n * G3n))]


def update_best(c: CDLState) -> tuple[float, bool]:
    """src/CDL/train.jl:91-98."""
    obj = objective(c)
    improved = obj < c.obj_best
    if improved:
        c.obj_best = obj
        c.D_best = (np.sum(c.d, axis=0) / c.N).astype(c.dtype)
        c.X_best = c.X.copy()
    return obj, improved


def run_outer(c: CDLState, iter_num: int, csc_iter_num: int = 15, cdl_iter_num: int = 1) -> list:
    """The body of ``cdl_optimize``'s loop, src/WRAPPER/wrap.jl:6-11."""
    objs = []
    for _ in range(iter_num):
        code_update(c, csc_iter_num)
        obj, _imp = update_best(c)
        dict_update(c, cdl_iter_num)
        objs.append(obj)
    return objs


def code_threshold(X_best: np.ndarray, multiplier: float = 1.0) -> float:
    """src/WRAPPER/wrap.jl:12 -- std(X_best[X_best .> 0]) (Julia's corrected std, n-1)."""
    v = X_best[X_best > 0].astype(np.float64)
    return float(multiplier * np.std(v, ddof=1))
