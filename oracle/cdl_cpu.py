"""ctypes wrapper of the float32 C++/OpenMP CPU restatement of the CDL ADMM
(``oracle/cdl_cpu.cpp``).

TEST AND MEASUREMENT INFRASTRUCTURE ONLY: the CPU baseline bench.py times on the host
cores and the CPU tests check against the NumPy oracle; the product never uses it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cdl_cpu.cpp")
LIB = os.path.join(HERE, "_build", "libcdlcpu.so")


def build() -> str:
    """g++ -O3 -fopenmp of cdl_cpu.cpp into oracle/_build/ (rebuilt when the source is
    newer)."""
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    tmp = LIB + ".tmp"
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-fcx-limited-range", "-fPIC", "-shared", SRC,
           "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"building the CPU restatement failed:\n{' '.join(cmd)}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(build())
        fp, dp, vp = C.POINTER(C.c_float), C.POINTER(C.c_double), C.c_void_p
        L.cdlcpu_create.restype = vp
        L.cdlcpu_create.argtypes = [fp, fp, fp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float,
                                    C.c_float, C.c_float, C.c_int]
        L.cdlcpu_destroy.argtypes = [vp]
        L.cdlcpu_obj_best.restype = C.c_double
        L.cdlcpu_obj_best.argtypes = [vp]
        L.cdlcpu_run_outer.argtypes = [vp, C.c_int, C.c_int, C.c_int, dp]
        L.cdlcpu_get.restype = C.c_int
        L.cdlcpu_get.argtypes = [vp, C.c_int, fp]
        L.cdlcpu_threads.restype = C.c_int
        _lib = L
    return _lib


def _p(a, t=C.c_float):
    return a.ctypes.data_as(C.POINTER(t))


class CPUADMM:
    """The float32 CPU restatement: same state, statements and order as the reference
    (src/CDL/train.jl:1-98), arrays in the oracle's layout (N, M, Lg)."""

    FIELDS = {"X": 0, "d": 1, "G1": 2, "D_best": 3, "DX": 4, "X_best": 5, "G3": 6}

    def __init__(self, S, X0, D0, M, filter_size, rho, sigma, lam, threads: int = 0):
        S = np.ascontiguousarray(S, np.float32)
        self.N, self.L4 = S.shape
        self.M = M
        self.Lg = self.L4 + 8 * filter_size
        X0 = np.ascontiguousarray(np.asarray(X0, np.float32).reshape(self.N, M, self.Lg))
        D0 = np.ascontiguousarray(np.asarray(D0, np.float32).reshape(M, self.Lg))
        self._h = lib().cdlcpu_create(_p(S), _p(X0), _p(D0), self.N, self.L4, M, filter_size,
                                      rho, sigma, lam, int(threads))
        if not self._h:
            raise ValueError("transform length has a prime factor above 64")

    @property
    def obj_best(self) -> float:
        return lib().cdlcpu_obj_best(self._h)

    def run_outer(self, iters: int, csc: int = 15, cdl: int = 1) -> np.ndarray:
        objs = np.zeros(iters, np.float64)
        lib().cdlcpu_run_outer(self._h, iters, csc, cdl, _p(objs, C.c_double))
        return objs

    def get(self, name: str) -> np.ndarray:
        shape = {"X": (self.N, self.M, self.Lg), "d": (self.N, self.M, self.Lg),
                 "X_best": (self.N, self.M, self.Lg), "G1": (self.M, self.Lg),
                 "G3": (self.M, self.Lg), "D_best": (self.M, self.Lg), "DX": (self.N, self.Lg)}[name]
        out = np.empty(shape, np.float32)
        lib().cdlcpu_get(self._h, self.FIELDS[name], _p(out))
        return out

    def close(self):
        if getattr(self, "_h", None):
            lib().cdlcpu_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def threads() -> int:
    return lib().cdlcpu_threads()
