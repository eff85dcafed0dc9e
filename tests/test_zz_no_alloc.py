"""The allocation-free objective entry point (cdlgb_objective_noalloc).

It exists for callers that own their device memory through their own allocator and
must not see the library call cudaMalloc (for example a CUDA.jl memory pool that
holds the free memory): they pass their own device buffers X, DX and S and get the
objective back in host memory.  This test gives it device copies of a context's
state and checks two calls in a row against the context's own objective (the
existing entry point, cdlgb_objective), within the objective tolerance used by the
other GPU tests (1e-5 relative).  It is collected last so that a failure here does
not hide the other tests' results."""
import ctypes as C

import numpy as np
import pytest

from conftest import random_onehot

pytestmark = pytest.mark.gpu

TOL_OBJ = 1e-5


def test_objective_noalloc_matches_context(pkg, built_lib):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(21)
    N, L, M, fs = 40, 50, 6, 3
    S, _ = random_onehot(rng, N, L)
    setup = pkg.CDLSetup(M=M, filter_size=fs, lambda_=0.1, rho=1.0, sigma=100.0)
    with pkg.init_cdl(setup, S, seed=3) as c:
        pkg.run_outer(c, 1)
        pkg.code_update(c, 2)
        ref = pkg.objective(c)
        X, DX = c.X, c.DX
        gamma = c.gamma
    dev = torch.device("cuda:0")
    Xd = torch.from_numpy(X).to(dev)
    DXd = torch.from_numpy(DX).to(dev)
    Sd = torch.from_numpy(np.ascontiguousarray(S)).to(dev)
    torch.cuda.synchronize()
    lib = built_lib

    def call():
        out = C.c_double(0.0)
        st = lib.cdlgb_objective_noalloc(C.c_void_p(Xd.data_ptr()), C.c_void_p(DXd.data_ptr()),
                                         C.c_void_p(Sd.data_ptr()), 4 * L, N, M, gamma, 0.1,
                                         C.byref(out), None)
        assert st == 0
        return out.value

    # after a first call (which may load the module on a lazy-loading driver), further
    # calls must leave the device's free memory unchanged: the entry point allocates
    # nothing
    vals = [call()]
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    vals.append(call())
    vals.append(call())
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    for v in vals:
        assert v == pytest.approx(ref, rel=TOL_OBJ)
    assert vals[0] == vals[1] == vals[2]


def test_objective_noalloc_rejects_oversized(pkg, built_lib):
    out = C.c_double(0.0)
    dummy = C.c_void_p(16)   # never dereferenced: the size check comes first
    st = built_lib.cdlgb_objective_noalloc(dummy, dummy, dummy, 400, 65537, 4, 16, 0.1,
                                           C.byref(out), None)
    assert st == -1
