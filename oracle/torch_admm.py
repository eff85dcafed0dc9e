"""GPU restatements of the CDL ADMM in torch, for the precision study and the long-run
parity tests.

TEST INFRASTRUCTURE ONLY: the checker the float32 CUDA path is measured against.  Only
``tests/`` and ``bench.py``'s precision study import it; the product never does.

Two restatements, both chunked over sequences so that the 20000-sequence workload fits
next to the CUDA path's own state:

* ``LiteralADMM`` -- ``code_update!`` / ``dict_update!`` / ``update_best!`` / ``objective``
  (src/CDL/train.jl:1-98, src/SETUP/CDL_setup.jl:165-286) statement by statement, as
  ``oracle/cdl_oracle.py`` states them: full complex FFTs of real arrays promoted to
  complex, the inverse scaled by 1/Lg and its real part kept, d-hat kept as state.  In
  ``float32`` it is the reference's own arithmetic order evaluated in FP32 (CUFFT c2c
  plans, broadcasts, sums over filters), which gives the drift that FP32 rounding alone
  causes in the reference; in ``float64`` it is an all-FP64 reference.
* ``HalfSpectrumADMM`` -- the same ADMM in the half-spectrum form the CUDA kernels use
  (one real transform per column for V = (Y2 - y2') + (Y3 - y3'), Y3 recomputed, d-hat =
  rfft(d)), cheaper in FP64; it agrees with the literal form to ~1e-13 in float64
  (tests/test_fp64ref_cpu.py).

Both keep the residual record the CUDA path reports (``RESIDUAL_FIELDS``): after each
code update the primal residuals of the final iterate (what the next dual updates of
src/CDL/train.jl:12-14 would add), after each D-step the increments its dual updates
(train.jl:70-72) added and the change of the consensus dictionary, all in float64.
"""
from __future__ import annotations

import numpy as np

RESIDUAL_FIELDS = (
    "x_y2",     # sum (X - shrink(X + y2, lambda))^2          after a code update
    "x_y3",     # sum (X - projectionX(X + y3))^2
    "x_y1",     # sum (DX - Y1)^2 over all Lg rows
    "x_norm",   # sum X^2
    "dx_norm",  # sum DX^2
    "d_g1",     # sum_n (d - G1_old)^2  = |increment of g1|^2   after a D-step
    "d_g3",     # sum_n (d - G3_old)^2  = |increment of g3|^2
    "d_g2",     # sum (Td - G2)^2       = |increment of g2|^2
    "d_norm",   # sum_n d^2
    "td_norm",  # sum Td^2
    "dual_G1",  # N sum (G1_new - G1_old)^2   (consensus dual residual / sigma^2)
    "dual_G3",  # N sum (G3_new - G3_old)^2
    "G_norm",   # N (sum G1_new^2 + sum G3_new^2)
)


def relative_residuals(r) -> dict:
    """The five relative residuals of the stopping test, from a residual record (13
    float64 values in RESIDUAL_FIELDS order)."""
    r = {k: float(v) for k, v in zip(RESIDUAL_FIELDS, r)}
    tiny = 1e-300
    return {
        "primal_x": np.sqrt((r["x_y2"] + r["x_y3"]) / max(r["x_norm"], tiny)),
        "primal_dx": np.sqrt(r["x_y1"] / max(r["dx_norm"], tiny)),
        "primal_d": np.sqrt((r["d_g1"] + r["d_g3"]) / max(2.0 * r["d_norm"], tiny)),
        "primal_td": np.sqrt(r["d_g2"] / max(r["td_norm"], tiny)),
        "dual_d": np.sqrt((r["dual_G1"] + r["dual_G3"]) / max(r["G_norm"], tiny)),
    }


class _Common:
    def _setup(self, S, X0, D0, M, filter_size, rho, sigma, lam, device, chunk, dtype):
        import torch
        self.t = torch
        self.dt = dtype
        self.cdt = torch.complex64 if dtype == torch.float32 else torch.complex128
        self.dev = device
        self.S = torch.as_tensor(np.asarray(S), device=device).to(dtype)         # (N, 4L)
        self.N, self.L4 = self.S.shape
        self.M = M
        self.gamma = 4 * filter_size
        self.flen = 4 * filter_size
        self.Lg = self.L4 + 2 * self.gamma
        self.rho, self.sigma, self.lam = rho, sigma, lam
        self.chunk = chunk
        self.diag = torch.zeros(self.Lg, dtype=dtype, device=device)
        self.diag[self.gamma:self.gamma + self.L4] = 1.0
        self.mask4 = (torch.arange(self.Lg, device=device) % 4) == 0
        self.zero = torch.zeros((), dtype=dtype, device=device)
        X = torch.as_tensor(np.asarray(X0), device=device).to(dtype).reshape(self.N, M, self.Lg).clone()
        X[:, :, ~self.mask4] = 0.0
        D = torch.as_tensor(np.asarray(D0), device=device).to(dtype).reshape(M, self.Lg).clone()
        D[:, self.flen:] = 0.0
        self.resid = np.zeros(len(RESIDUAL_FIELDS))
        return X, D

    def _chunks(self):
        for n0 in range(0, self.N, self.chunk):
            yield n0, min(self.N, n0 + self.chunk)

    def _wts(self, n0, n1):
        w = self.t.zeros(n1 - n0, self.Lg, dtype=self.dt, device=self.dev)
        w[:, self.gamma:self.gamma + self.L4] = self.S[n0:n1]
        return w

    def _shrink(self, v):
        t = self.t
        return t.sign(v) * t.clamp(v.abs() - self.lam, min=0.0)

    def _proj(self, v):
        return self.t.where(self.mask4, v, self.zero)

    def objective(self) -> float:
        """src/SETUP/CDL_setup.jl:286, accumulated in float64."""
        f64 = self.t.float64
        r = (self.DX[:, self.gamma:self.gamma + self.L4] - self.S).to(f64)
        a = 0.0
        for n0, n1 in self._chunks():
            a += float(self.X[n0:n1].to(f64).abs().sum())
        return float(0.5 * (r * r).sum()) + float(self.lam) * a

    def _x_residuals(self):
        """Primal residuals of the final iterate of a code update (float64 sums)."""
        f64 = self.t.float64
        s = np.zeros(5)
        for n0, n1 in self._chunks():
            X = self.X[n0:n1]
            Y2 = self._shrink(X + self.y2[n0:n1])
            Y3 = self._proj(X + self.y3[n0:n1])
            s[0] += float(((X - Y2).to(f64) ** 2).sum())
            s[1] += float(((X - Y3).to(f64) ** 2).sum())
            s[3] += float((X.to(f64) ** 2).sum())
        s[2] = float(((self.DX - self.Y1).to(f64) ** 2).sum())
        s[4] = float((self.DX.to(f64) ** 2).sum())
        self.resid[0:5] = s

    def _prox(self, v1, v2):
        """projection2box! (cdl_kernels.jl:37-51) of v2 and prox_simplex_zeros! with the
        reference's group index (cdl_kernels.jl:53-66) of v1."""
        t = self.t
        sup = t.zeros_like(v2, dtype=t.bool)
        sup[:, : self.flen] = True
        G3 = t.where(v2 >= 1, sup.to(v2.dtype), t.where(v2 <= 0, t.zeros_like(v2), t.where(sup, v2, t.zeros_like(v2))))
        l0 = t.arange(self.flen, device=self.dev)
        i = 4 * ((l0 + 1) // 4)
        grp = v1[:, i] + v1[:, i + 1] + v1[:, i + 2] + v1[:, i + 3]
        G1 = t.zeros_like(v1)
        G1[:, : self.flen] = v1[:, : self.flen] - 0.25 * (grp - 1.0)
        return G1, G3

    def _dual_d(self, G1o, G3o):
        f64 = self.t.float64
        self.resid[10] = self.N * float(((self.G1 - G1o).to(f64) ** 2).sum())
        self.resid[11] = self.N * float(((self.G3 - G3o).to(f64) ** 2).sum())
        self.resid[12] = self.N * float((self.G1.to(f64) ** 2).sum() + (self.G3.to(f64) ** 2).sum())

    def update_best(self):
        """src/CDL/train.jl:91-98."""
        obj = self.objective()
        imp = obj < self.obj_best
        if imp:
            self.obj_best = obj
            self.D_best = self.dmean.clone()
            self.X_best.copy_(self.X)
        return obj, imp

    def run_outer(self, iters: int, csc: int = 15, cdl: int = 1):
        """cdl_optimize's loop body, src/WRAPPER/wrap.jl:6-11."""
        objs = []
        for _ in range(iters):
            self.code_update(csc)
            o, _ = self.update_best()
            self.dict_update(cdl)
            objs.append(o)
        return objs


class LiteralADMM(_Common):
    """src/CDL/train.jl:1-98 statement by statement (full complex FFTs), in `dtype`."""

    def __init__(self, S, X0, D0, M: int, filter_size: int, rho: float, sigma: float,
                 lam: float, device="cuda:0", chunk: int = 1024, k_csc: float = 2.0,
                 k_cdl: float = 2.0, dtype=None):
        import torch
        dtype = dtype or torch.float32
        X, D = self._setup(S, X0, D0, M, filter_size, rho, sigma, lam, device, chunk, dtype)
        fft = torch.fft
        N, Lg = self.N, self.Lg
        self.kc, self.kd = k_csc, k_cdl
        self.X = X
        # CDL_setup.jl:197-236
        Dh = fft.fft(D.to(self.cdt), dim=-1)
        self.DX = torch.empty(N, Lg, dtype=dtype, device=device)
        for n0, n1 in self._chunks():
            Xh = fft.fft(X[n0:n1].to(self.cdt), dim=-1)
            self.DX[n0:n1] = fft.ifft((Dh.unsqueeze(0) * Xh).sum(1), dim=-1).real
        self.dh = Dh.unsqueeze(0).expand(N, M, Lg).clone()
        self.d = fft.ifft(Dh, dim=-1).real.unsqueeze(0).expand(N, M, Lg).clone()
        self.Td = torch.zeros(N, Lg, dtype=dtype, device=device)
        self.Y1 = torch.zeros_like(self.Td)
        self.y1 = torch.zeros_like(self.Td)
        self.Y3 = X.clone()
        self.y2 = torch.zeros_like(X)
        self.y3 = torch.zeros_like(X)
        self.G1, self.G3 = D.clone(), D.clone()
        self.G2 = self.DX.clone()
        self.g1 = torch.zeros_like(X)
        self.g3 = torch.zeros_like(X)
        self.g2 = torch.zeros_like(self.Td)
        self.dmean = D.clone()
        self.D_best = D.clone()
        self.X_best = X.clone()
        self.obj_best = self.objective()

    def code_update(self, iters: int):
        """src/CDL/train.jl:1-44: Y1-hat and Y3-hat carried from the previous iteration
        are the transforms of the stored Y1, Y3 (CDL_setup.jl:227-230, train.jl:36,41)."""
        t = self.t
        fft = t.fft
        cd = self.cdt
        G1h = fft.fft(self.G1.to(cd), dim=-1)                                  # (M, Lg)
        sum_dots = (G1h * G1h.conj()).sum(0, keepdim=True) + self.kc           # :18-19
        At = G1h / sum_dots                                                    # :20
        for _ in range(iters):
            for n0, n1 in self._chunks():
                X, y2, y3 = self.X[n0:n1], self.y2[n0:n1], self.y3[n0:n1]
                Y1, Y3 = self.Y1[n0:n1], self.Y3[n0:n1]
                Y2 = self._shrink(X + y2)                                      # :7
                Y2h = fft.fft(Y2.to(cd), dim=-1)                               # :8
                y1 = self.y1[n0:n1] + self.DX[n0:n1] - Y1                      # :12
                y2 = y2 + X - Y2                                               # :13
                y3 = y3 + X - Y3                                               # :14
                y1h = fft.fft(y1.to(cd), dim=-1)
                y2h = fft.fft(y2.to(cd), dim=-1)
                y3h = fft.fft(y3.to(cd), dim=-1)
                Y1h = fft.fft(Y1.to(cd), dim=-1)
                Y3h = fft.fft(Y3.to(cd), dim=-1)
                RHS = (G1h.conj().unsqueeze(0) * (Y1h - y1h).unsqueeze(1)     # :21-23
                       + (Y2h - y2h) + (Y3h - y3h))
                alpha = (At.unsqueeze(0) * RHS).sum(1)                          # :24
                Xh = (RHS - alpha.unsqueeze(1) * G1h.conj().unsqueeze(0)) / self.kc   # :25
                X = fft.ifft(Xh, dim=-1).real                                  # :26
                DX = fft.ifft((G1h.unsqueeze(0) * Xh).sum(1), dim=-1).real    # :27
                Y1 = (self._wts(n0, n1) + self.rho * (DX + y1)) / (self.diag + self.rho)   # :35
                self.Y3[n0:n1] = self._proj(X + y3)                            # :40
                self.X[n0:n1], self.DX[n0:n1], self.Y1[n0:n1] = X, DX, Y1
                self.y1[n0:n1], self.y2[n0:n1], self.y3[n0:n1] = y1, y2, y3
        self._x_residuals()

    def dict_update(self, iters: int):
        """src/CDL/train.jl:46-89 (no 1/2 in the combine, cdl_kernels.jl:30)."""
        t = self.t
        fft = t.fft
        cd = self.cdt
        f64 = t.float64
        N = self.N
        for _ in range(iters):
            G1h = fft.fft(self.G1.to(cd), dim=-1)
            G3h = fft.fft(self.G3.to(cd), dim=-1)
            s1 = t.zeros(self.M, self.Lg, dtype=self.dt, device=self.dev)
            s3 = t.zeros_like(s1)
            sd = t.zeros_like(s1)
            r = np.zeros(5)
            for n0, n1 in self._chunks():
                Y3h = fft.fft(self.Y3[n0:n1].to(cd), dim=-1)                   # :52
                sum_dots = (Y3h * Y3h.conj()).sum(1, keepdim=True) + self.kd  # :53
                Xc = Y3h / sum_dots                                            # :54
                Td = fft.ifft((Y3h * self.dh[n0:n1]).sum(1), dim=-1).real      # :56-57 (old d-hat)
                G2h = fft.fft(self.G2[n0:n1].to(cd), dim=-1)
                g2h = fft.fft(self.g2[n0:n1].to(cd), dim=-1)
                g1h = fft.fft(self.g1[n0:n1].to(cd), dim=-1)
                g3h = fft.fft(self.g3[n0:n1].to(cd), dim=-1)
                RHS = (Y3h.conj() * (G2h - g2h).unsqueeze(1)                    # :58
                       + (G1h.unsqueeze(0) - g1h) + (G3h.unsqueeze(0) - g3h))
                beta = (Xc * RHS).sum(1)                                       # :59
                dh = RHS - beta.unsqueeze(1) * Y3h.conj()                      # :60
                d = fft.ifft(dh, dim=-1).real                                  # :61
                G2 = (self._wts(n0, n1) + self.sigma * (Td + self.g2[n0:n1])) / (self.diag + self.sigma)   # :68
                g1 = self.g1[n0:n1] + d - self.G1.unsqueeze(0)                 # :70
                g2 = self.g2[n0:n1] + Td - G2                                  # :71
                g3 = self.g3[n0:n1] + d - self.G3.unsqueeze(0)                 # :72
                r[0] += float(((d - self.G1.unsqueeze(0)).to(f64) ** 2).sum())
                r[1] += float(((d - self.G3.unsqueeze(0)).to(f64) ** 2).sum())
                r[2] += float(((Td - G2).to(f64) ** 2).sum())
                r[3] += float((d.to(f64) ** 2).sum())
                r[4] += float((Td.to(f64) ** 2).sum())
                self.dh[n0:n1], self.d[n0:n1], self.Td[n0:n1] = dh, d, Td
                self.G2[n0:n1], self.g1[n0:n1], self.g2[n0:n1], self.g3[n0:n1] = G2, g1, g2, g3
                s3 += (d + g3).sum(0)                                          # :76
                s1 += (d + g1).sum(0)                                          # :83
                sd += d.sum(0)
            self.resid[5:10] = r
            G1o, G3o = self.G1, self.G3
            self.dmean = sd / N
            self.G1, self.G3 = self._prox(s1 / N, s3 / N)                      # :76-85
            self._dual_d(G1o, G3o)


class HalfSpectrumADMM(_Common):
    """The ADMM in the half-spectrum form of the CUDA kernels (the algebra checked
    against the literal restatement in tests/test_algebra.py), in `dtype`."""

    def __init__(self, S, X0, D0, M: int, filter_size: int, rho: float, sigma: float,
                 lam: float, device="cuda:0", chunk: int = 1024, k_csc: float = 2.0,
                 k_cdl: float = 2.0, dtype=None):
        import torch
        dtype = dtype or torch.float64
        X, D = self._setup(S, X0, D0, M, filter_size, rho, sigma, lam, device, chunk, dtype)
        self.kc, self.kd = float(k_csc), float(k_cdl)
        Lg, N = self.Lg, self.N
        self.X = X
        self.G1, self.G3 = D.clone(), D.clone()
        self.y2 = torch.zeros_like(self.X)
        self.y3 = torch.zeros_like(self.X)
        self.g1 = torch.zeros_like(self.X)
        self.g3 = torch.zeros_like(self.X)
        self.d = D.unsqueeze(0).expand(N, M, Lg).clone()
        self.dmean = D.clone()
        self.Y1 = torch.zeros(N, Lg, dtype=dtype, device=device)
        self.y1 = torch.zeros_like(self.Y1)
        self.g2 = torch.zeros_like(self.Y1)
        self.Td = torch.zeros_like(self.Y1)
        # DX = irfft(sum_m rfft(D) rfft(X)), G2 = DX   (CDL_setup.jl:197-203, :226)
        a = torch.fft.rfft(D, dim=-1)
        self.DX = torch.empty_like(self.Y1)
        for n0, n1 in self._chunks():
            Xh = torch.fft.rfft(self.X[n0:n1], dim=-1)
            self.DX[n0:n1] = torch.fft.irfft((a.unsqueeze(0) * Xh).sum(1), n=Lg, dim=-1)
        self.G2 = self.DX.clone()
        self.X_best = self.X.clone()
        self.D_best = D.clone()
        self.obj_best = self.objective()

    def code_update(self, iters: int):
        t = self.t
        Lg = self.Lg
        a = t.fft.rfft(self.G1, dim=-1)
        A = (a.real ** 2 + a.imag ** 2).sum(0)
        for _ in range(iters):
            for n0, n1 in self._chunks():
                X, y2, y3 = self.X[n0:n1], self.y2[n0:n1], self.y3[n0:n1]
                Y3 = self._proj(X + y3)
                Y2 = self._shrink(X + y2)
                y2n = y2 + X - Y2
                y3n = y3 + X - Y3
                V = (Y2 - y2n) + (Y3 - y3n)
                y1n = self.y1[n0:n1] + self.DX[n0:n1] - self.Y1[n0:n1]
                U = self.Y1[n0:n1] - y1n
                Vh = t.fft.rfft(V, dim=-1)
                Uh = t.fft.rfft(U, dim=-1)
                P = (a.unsqueeze(0) * Vh).sum(1)
                alpha = (A * Uh + P) / (A + self.kc)
                W = Uh - alpha
                Xh = (Vh + a.conj().unsqueeze(0) * W.unsqueeze(1)) / self.kc
                DXh = (P + A * W) / self.kc
                self.X[n0:n1] = t.fft.irfft(Xh, n=Lg, dim=-1)
                DX = t.fft.irfft(DXh, n=Lg, dim=-1)
                self.DX[n0:n1] = DX
                self.Y1[n0:n1] = (self._wts(n0, n1) + self.rho * (DX + y1n)) / (self.diag + self.rho)
                self.y1[n0:n1] = y1n
                self.y2[n0:n1] = y2n
                self.y3[n0:n1] = y3n
        self._x_residuals()

    def dict_update(self, iters: int):
        t = self.t
        f64 = t.float64
        Lg, N = self.Lg, self.N
        for _ in range(iters):
            s1 = t.zeros(self.M, Lg, dtype=self.X.dtype, device=self.dev)
            s3 = t.zeros_like(s1)
            sd = t.zeros_like(s1)
            r = np.zeros(5)
            for n0, n1 in self._chunks():
                X, y3 = self.X[n0:n1], self.y3[n0:n1]
                Y3h = t.fft.rfft(self._proj(X + y3), dim=-1)
                B = (Y3h.real ** 2 + Y3h.imag ** 2).sum(1)
                Zh = t.fft.rfft(self.G2[n0:n1] - self.g2[n0:n1], dim=-1)
                Hh = t.fft.rfft((self.G1.unsqueeze(0) - self.g1[n0:n1]) + (self.G3.unsqueeze(0) - self.g3[n0:n1]), dim=-1)
                T = (Y3h * t.fft.rfft(self.d[n0:n1], dim=-1)).sum(1)
                Td = t.fft.irfft(T, n=Lg, dim=-1)
                Q = (Y3h * Hh).sum(1)
                beta = (Zh * B + Q) / (B + self.kd)
                d = t.fft.irfft(Hh + Y3h.conj() * (Zh - beta).unsqueeze(1), n=Lg, dim=-1)
                G2n = (self._wts(n0, n1) + self.sigma * (Td + self.g2[n0:n1])) / (self.diag + self.sigma)
                r[0] += float(((d - self.G1.unsqueeze(0)).to(f64) ** 2).sum())
                r[1] += float(((d - self.G3.unsqueeze(0)).to(f64) ** 2).sum())
                r[2] += float(((Td - G2n).to(f64) ** 2).sum())
                r[3] += float((d.to(f64) ** 2).sum())
                r[4] += float((Td.to(f64) ** 2).sum())
                self.g2[n0:n1] = self.g2[n0:n1] + Td - G2n
                self.G2[n0:n1] = G2n
                self.Td[n0:n1] = Td
                g1n = self.g1[n0:n1] + d - self.G1.unsqueeze(0)
                g3n = self.g3[n0:n1] + d - self.G3.unsqueeze(0)
                self.g1[n0:n1], self.g3[n0:n1], self.d[n0:n1] = g1n, g3n, d
                s1 += (d + g1n).sum(0)
                s3 += (d + g3n).sum(0)
                sd += d.sum(0)
            self.resid[5:10] = r
            G1o, G3o = self.G1, self.G3
            self.dmean = sd / N
            self.G1, self.G3 = self._prox(s1 / N, s3 / N)
            self._dual_d(G1o, G3o)


def FP64Reference(S, X0, D0, M, filter_size, rho, sigma, lam, device="cuda:0", chunk=1024,
                  k_csc=2.0, k_cdl=2.0):
    """The all-FP64 reference of the precision study (half-spectrum form, float64)."""
    import torch
    return HalfSpectrumADMM(S, X0, D0, M, filter_size, rho, sigma, lam, device=device,
                            chunk=chunk, k_csc=k_csc, k_cdl=k_cdl, dtype=torch.float64)
