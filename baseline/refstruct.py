"""Reference-structured CUDA baseline (baseline/refstruct.cu): the reference's CUDA.jl
CDL ADMM restated statement by statement, as the stand-in for the reference GPU path
(unavailable here).  Measurement infrastructure, not part of the product: used by
bench.py (--impl refstruct) and by its parity test against the oracle."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "refstruct.cu")
LIB = os.path.join(HERE, "lib", "librefstruct.so")

_lib = None


def build(force: bool = False) -> str:
    """nvcc the baseline for sm_103a into baseline/lib/librefstruct.so."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cmd = [os.environ.get("NVCC", "nvcc"), "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
           "-std=c++17", "-shared", "-Xcompiler", "-fPIC", SRC, "-o", LIB, "-lcufft", "-lcublas"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise RuntimeError(f"{LIB} is not built (baseline/refstruct.py build())")
        L = C.CDLL(LIB)
        fp = C.POINTER(C.c_float)
        L.rs_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float,
                                fp, fp, fp, C.POINTER(C.c_void_p)]
        L.rs_create.restype = C.c_int
        L.rs_run_outer.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double)]
        L.rs_run_outer.restype = C.c_int
        L.rs_get.argtypes = [C.c_void_p, C.c_int, fp]
        L.rs_get.restype = C.c_int
        L.rs_destroy.argtypes = [C.c_void_p]
        L.rs_destroy.restype = None
        L.rs_last_error.argtypes = [C.c_void_p]
        L.rs_last_error.restype = C.c_char_p
        _lib = L
    return _lib


FIELDS = {"X": 0, "d": 1, "G1": 2, "D_best": 3, "DX": 4, "X_best": 5}


class RefStruct:
    """One reference-structured CDL state on the current CUDA device."""

    def __init__(self, S, X0, D0, M: int, filter_size: int, rho=1.0, sigma=100.0, lam=0.1):
        L = lib()
        S = np.ascontiguousarray(S, np.float32)
        self.N, self.L4 = S.shape
        self.M = M
        self.Lg = self.L4 + 8 * filter_size
        X0 = np.ascontiguousarray(X0, np.float32).reshape(self.N, M, self.Lg)
        D0 = np.ascontiguousarray(D0, np.float32).reshape(M, self.Lg)
        fp = C.POINTER(C.c_float)
        self.h = C.c_void_p()
        st = L.rs_create(self.L4, self.N, M, filter_size, rho, sigma, lam, S.ctypes.data_as(fp),
                         X0.ctypes.data_as(fp), D0.ctypes.data_as(fp), C.byref(self.h))
        if st != 0:
            msg = L.rs_last_error(self.h).decode() if self.h else "allocation failed"
            self.close()
            raise RuntimeError("refstruct create: " + msg)

    def run_outer(self, iters: int, csc: int = 15, cdl: int = 1) -> np.ndarray:
        objs = np.zeros(iters, np.float64)
        st = lib().rs_run_outer(self.h, iters, csc, cdl, objs.ctypes.data_as(C.POINTER(C.c_double)))
        if st != 0:
            raise RuntimeError("refstruct run: " + lib().rs_last_error(self.h).decode())
        return objs

    def get(self, name: str) -> np.ndarray:
        shape = {"X": (self.N, self.M, self.Lg), "X_best": (self.N, self.M, self.Lg),
                 "d": (self.N, self.M, self.Lg), "G1": (self.M, self.Lg), "D_best": (self.M, self.Lg),
                 "DX": (self.N, self.Lg)}[name]
        out = np.empty(shape, np.float32)
        if lib().rs_get(self.h, FIELDS[name], out.ctypes.data_as(C.POINTER(C.c_float))) != 0:
            raise RuntimeError("refstruct get: " + lib().rs_last_error(self.h).decode())
        return out

    def close(self):
        if getattr(self, "h", None):
            lib().rs_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
