"""CPU test of the algebra the CUDA kernels implement.

The kernels do not replay the reference's statement order: they use half spectra,
one real FFT per column per step instead of four complex ones, recompute Y3 from
X + y3 and the consensus spectrum d-hat from d, and reduce each Sherman-Morrison
solve to one cross-filter sum.  This file restates that reduced algebra in numpy
FP64 and checks it against the oracle's literal restatement of
src/CDL/train.jl:1-89 over several outer iterations (agreement to ~1e-13)."""
import numpy as np

from oracle import cdl_oracle as O

from conftest import random_onehot, rel


def _proj(a):
    b = a.copy()
    b[..., (np.arange(a.shape[-1]) % 4) != 0] = 0
    return b


def reduced_xstep(st, c, iters, k=2.0):
    X, y2, y3, Y1, y1, DX = (st[n] for n in ("X", "y2", "y3", "Y1", "y1", "DX"))
    Lg = X.shape[-1]
    a = np.fft.rfft(st["G1"], axis=-1)
    A = np.sum(np.abs(a) ** 2, axis=0)
    for _ in range(iters):
        Y3 = _proj(X + y3)
        Y2 = O.shrink(X + y2, c.lam)
        y2n, y3n = y2 + X - Y2, y3 + X - Y3
        V = (Y2 - y2n) + (Y3 - y3n)
        y1n = y1 + DX - Y1
        U = Y1 - y1n
        Vh, Uh = np.fft.rfft(V, axis=-1), np.fft.rfft(U, axis=-1)
        P = np.sum(a[None] * Vh, axis=1)
        alpha = (A * Uh + P) / (A + k)
        W = Uh - alpha
        Xh = (Vh + np.conj(a)[None] * W[:, None]) / k
        DXh = (P + A * W) / k
        X, DX = np.fft.irfft(Xh, Lg, axis=-1), np.fft.irfft(DXh, Lg, axis=-1)
        Y1 = (c.WtS + c.rho * (DX + y1n)) / (c.WtW_diag + c.rho)
        y1, y2, y3 = y1n, y2n, y3n
    st.update(X=X, y2=y2, y3=y3, Y1=Y1, y1=y1, DX=DX)


def reduced_dstep(st, c, k=2.0):
    X, y3, d, g1, g3, G1, G3, G2, g2 = (st[n] for n in "X y3 d g1 g3 G1 G3 G2 g2".split())
    Lg = X.shape[-1]
    Y3h = np.fft.rfft(_proj(X + y3), axis=-1)
    B = np.sum(np.abs(Y3h) ** 2, axis=1)
    Zh = np.fft.rfft(G2 - g2, axis=-1)
    Hh = np.fft.rfft((G1[None] - g1) + (G3[None] - g3), axis=-1)
    T = np.sum(Y3h * np.fft.rfft(d, axis=-1), axis=1)
    Td = np.fft.irfft(T, Lg, axis=-1)
    Q = np.sum(Y3h * Hh, axis=1)
    beta = (Zh * B + Q) / (B + k)
    d = np.fft.irfft(Hh + np.conj(Y3h) * (Zh - beta)[:, None], Lg, axis=-1)
    G2n = (c.WtS + c.sigma * (Td + g2)) / (c.WtW_diag + c.sigma)
    g2n = g2 + Td - G2n
    g1n, g3n = g1 + d - G1[None], g3 + d - G3[None]
    G3n = O.projection2box(np.mean(d + g3n, axis=0), c.P_D)
    G1n = O.prox_simplex_zeros(np.mean(d + g1n, axis=0), c.P_D)
    st.update(d=d, g1=g1n, g3=g3n, G1=G1n, G3=G3n, G2=G2n, g2=g2n, Td=Td)


def test_reduced_algebra_matches_reference_order():
    rng = np.random.default_rng(11)
    S, _ = random_onehot(rng, 6, 10)
    c = O.init_cdl(S, 3, 2, rho=1.0, sigma=100.0, lam=0.1, rng=rng)
    st = {k: getattr(c, k).copy() for k in "X y2 y3 Y1 y1 DX d g1 g3 G1 G3 G2 g2".split()}
    for _ in range(4):
        O.code_update(c, 15)
        reduced_xstep(st, c, 15)
        assert rel(st["X"], c.X) < 1e-12 and rel(st["DX"], c.DX) < 1e-12
        O.dict_update(c, 1)
        reduced_dstep(st, c)
        assert rel(st["d"], c.d) < 1e-12 and rel(st["Td"], c.Td) < 1e-12
        assert rel(st["G1"], c.G1) < 1e-12 and rel(st["G3"], c.G3) < 1e-12
        # invariants the kernels rely on
        assert rel(_proj(c.X + c.y3), c.Y3) < 1e-14
        np.testing.assert_allclose(np.fft.fft(c.d, axis=-1), c.dh, atol=1e-9)
