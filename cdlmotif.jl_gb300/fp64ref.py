"""All-FP64 GPU reference of the CDL ADMM, for the precision study.

A measurement reference, not a product path: it re-runs the same ADMM as the float32
CUDA kernels in float64 with torch (cuFFT double-precision transforms) so that results
at the full 20000-sequence size can state their error against FP64.  It implements
the half-spectrum form of src/CDL/train.jl:1-98 that the CUDA kernels use (the form
checked against a literal statement-by-statement restatement of the reference to
~1e-13), processing sequences in chunks to bound temporaries.
"""
from __future__ import annotations

import numpy as np


class FP64Reference:
    def __init__(self, S, X0, D0, M: int, filter_size: int, rho: float, sigma: float,
                 lam: float, device="cuda:0", chunk: int = 1024, k_csc: float = 2.0,
                 k_cdl: float = 2.0):
        import torch
        self.t = torch
        f64 = torch.float64
        self.dev = device
        self.S = torch.as_tensor(np.asarray(S), device=device).to(f64)           # (N, 4L)
        self.N, self.L4 = self.S.shape
        self.M = M
        self.gamma = 4 * filter_size
        self.flen = 4 * filter_size
        self.Lg = self.L4 + 2 * self.gamma
        self.rho, self.sigma, self.lam = float(rho), float(sigma), float(lam)
        self.kc, self.kd = float(k_csc), float(k_cdl)
        self.chunk = chunk
        Lg, N = self.Lg, self.N
        self.diag = torch.zeros(Lg, dtype=f64, device=device)
        self.diag[self.gamma:self.gamma + self.L4] = 1.0
        self.mask4 = (torch.arange(Lg, device=device) % 4) == 0
        self.X = torch.as_tensor(np.asarray(X0), device=device).to(f64).reshape(N, M, Lg)
        self.X[:, :, ~self.mask4] = 0.0
        D = torch.as_tensor(np.asarray(D0), device=device).to(f64).reshape(M, Lg).clone()
        D[:, self.flen:] = 0.0
        self.G1, self.G3 = D.clone(), D.clone()
        self.y2 = torch.zeros_like(self.X)
        self.y3 = torch.zeros_like(self.X)
        self.g1 = torch.zeros_like(self.X)
        self.g3 = torch.zeros_like(self.X)
        self.d = D.unsqueeze(0).expand(N, M, Lg).clone()
        self.dmean = D.clone()
        self.Y1 = torch.zeros(N, Lg, dtype=f64, device=device)
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

    def _chunks(self):
        for n0 in range(0, self.N, self.chunk):
            yield n0, min(self.N, n0 + self.chunk)

    def _wts(self, n0, n1):
        w = self.t.zeros(n1 - n0, self.Lg, dtype=self.S.dtype, device=self.dev)
        w[:, self.gamma:self.gamma + self.L4] = self.S[n0:n1]
        return w

    def objective(self) -> float:
        t = self.t
        r = self.DX[:, self.gamma:self.gamma + self.L4] - self.S
        return float(0.5 * (r * r).sum() + self.lam * self.X.abs().sum())

    def code_update(self, iters: int):
        t = self.t
        Lg = self.Lg
        a = t.fft.rfft(self.G1, dim=-1)
        A = (a.real ** 2 + a.imag ** 2).sum(0)
        for _ in range(iters):
            for n0, n1 in self._chunks():
                X, y2, y3 = self.X[n0:n1], self.y2[n0:n1], self.y3[n0:n1]
                Y3 = t.where(self.mask4, X + y3, t.zeros((), dtype=X.dtype, device=self.dev))
                tt = X + y2
                Y2 = t.sign(tt) * t.clamp(tt.abs() - self.lam, min=0.0)
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

    def dict_update(self, iters: int):
        t = self.t
        Lg, N = self.Lg, self.N
        for _ in range(iters):
            s1 = t.zeros(self.M, Lg, dtype=self.X.dtype, device=self.dev)
            s3 = t.zeros_like(s1)
            sd = t.zeros_like(s1)
            for n0, n1 in self._chunks():
                X, y3 = self.X[n0:n1], self.y3[n0:n1]
                Y3h = t.fft.rfft(t.where(self.mask4, X + y3, t.zeros((), dtype=X.dtype, device=self.dev)), dim=-1)
                B = (Y3h.real ** 2 + Y3h.imag ** 2).sum(1)
                Zh = t.fft.rfft(self.G2[n0:n1] - self.g2[n0:n1], dim=-1)
                Hh = t.fft.rfft((self.G1.unsqueeze(0) - self.g1[n0:n1]) + (self.G3.unsqueeze(0) - self.g3[n0:n1]), dim=-1)
                T = (Y3h * t.fft.rfft(self.d[n0:n1], dim=-1)).sum(1)
                Td = t.fft.irfft(T, n=Lg, dim=-1)
                Q = (Y3h * Hh).sum(1)
                beta = (Zh * B + Q) / (B + self.kd)
                d = t.fft.irfft(Hh + Y3h.conj() * (Zh - beta).unsqueeze(1), n=Lg, dim=-1)
                G2n = (self._wts(n0, n1) + self.sigma * (Td + self.g2[n0:n1])) / (self.diag + self.sigma)
                self.g2[n0:n1] = self.g2[n0:n1] + Td - G2n
                self.G2[n0:n1] = G2n
                self.Td[n0:n1] = Td
                g1n = self.g1[n0:n1] + d - self.G1.unsqueeze(0)
                g3n = self.g3[n0:n1] + d - self.G3.unsqueeze(0)
                self.g1[n0:n1], self.g3[n0:n1], self.d[n0:n1] = g1n, g3n, d
                s1 += (d + g1n).sum(0)
                s3 += (d + g3n).sum(0)
                sd += d.sum(0)
            v2, v1 = s3 / N, s1 / N
            self.dmean = sd / N
            sup = t.zeros_like(v2, dtype=t.bool)
            sup[:, : self.flen] = True
            # projection2box! (cdl_kernels.jl:37-51)
            G3 = t.where(v2 >= 1, sup.to(v2.dtype), t.where(v2 <= 0, t.zeros_like(v2), t.where(sup, v2, t.zeros_like(v2))))
            # prox_simplex_zeros! with the reference's group index (cdl_kernels.jl:53-66)
            l0 = t.arange(self.flen, device=self.dev)
            i = 4 * ((l0 + 1) // 4)
            grp = v1[:, i] + v1[:, i + 1] + v1[:, i + 2] + v1[:, i + 3]
            G1 = t.zeros_like(v1)
            G1[:, : self.flen] = v1[:, : self.flen] - 0.25 * (grp - 1.0)
            self.G1, self.G3 = G1, G3

    def update_best(self):
        obj = self.objective()
        imp = obj < self.obj_best
        if imp:
            self.obj_best = obj
            self.D_best = self.dmean.clone()
            self.X_best.copy_(self.X)
        return obj, imp

    def run_outer(self, iters: int, csc: int = 15, cdl: int = 1):
        objs = []
        for _ in range(iters):
            self.code_update(csc)
            o, _ = self.update_best()
            self.dict_update(cdl)
            objs.append(o)
        return objs
