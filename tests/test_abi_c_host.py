"""The C ABI from a plain C host (tests/host/abi_driver.c), without Python in the
process: host-only calls checked here against the oracle, and (on a GPU) one training
and a scan whose every printed value must equal, bit for bit, what the package's ctypes
path gives for the same inputs."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import search_oracle as SO

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "host", "abi_driver.c")
LIBDIR = os.path.join(ROOT, "cdlmotif.jl_gb300", "lib")


def _driver(built_lib, tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "abi_driver")
    subprocess.run([cc, "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe, "-L", LIBDIR,
                    "-lcdlgb", f"-Wl,-rpath,{LIBDIR}"], check=True, capture_output=True, text=True)
    return exe


def _hexf(tok):
    return float.fromhex(tok)


def test_c_host_cpu_calls(built_lib, tmp_path):
    exe = _driver(built_lib, tmp_path)
    r = subprocess.run([exe, "cpu"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.splitlines()
    d = lines[0].split()
    assert d[1:3] == ["10", "4"] and _hexf(d[3]) == 100.0 and d[6:9] == ["15", "1", "10"]
    pfm = np.array([_hexf(t) for t in lines[1].split()[1:]], np.float32).reshape(3, 4).T
    counts = np.array([7, 1, 1, 1, 0, 10, 0, 0, 2, 2, 3, 3], np.int32).reshape(1, 3, 4)
    ref = SO.counts_to_pfms(counts, np.array([10]), [3], smoothing=False)[0]
    np.testing.assert_array_equal(pfm, ref)
    n = int(lines[2].split()[1])
    text = "\n".join(lines[3:]) + "\n"
    text = text[:n]
    assert text == SO.transfac_text(ref)
    ev = [_hexf(t) for t in r.stdout.split("evalues")[1].split()]
    assert ev[0] == pytest.approx(SO.fisher_evalue_exact(40, 5, 100, 2), rel=1e-12)
    assert ev[1] == pytest.approx(SO.fisher_evalue_exact(3, 3, 100, 2), rel=1e-12)


@pytest.mark.gpu
def test_c_host_training_matches_ctypes_path(pkg, built_lib, tmp_path):
    exe = _driver(built_lib, tmp_path)
    r = subprocess.run([exe, "gpu"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    out = {ln.split()[0]: ln.split()[1:] for ln in r.stdout.splitlines()}
    # the same inputs through the package
    N, L, M, fs = 24, 40, 4, 3
    S = np.zeros((N, 4 * L), np.float32)
    s = 12345
    def lcg():
        nonlocal s
        s = (s * 1664525 + 1013904223) & 0xFFFFFFFF
        return s >> 8
    for n in range(N):
        for l in range(L):
            S[n, 4 * l + (lcg() & 3)] = 1.0
    setup = pkg.CDLSetup(M=M, filter_size=fs, lambda_=0.1, rho=1.0, sigma=100.0,
                         track_residuals=True)
    with pkg.init_cdl(setup, S, seed=7) as c:
        objs = pkg.run_outer(c, 3)
        th = pkg.code_threshold(c)
        Db = c.D_best
        res = c.residuals()
        pwm = np.array([((lcg() % 21) - 10) / 4.0 for _ in range(20)], np.float32)
        # (K=1, 4, 5) column-major -> the (4, 5) matrix
        pw = pwm.reshape(5, 4, 1)[:, :, 0].T.copy()
        pos, score, comp = pkg.overlapping_scan(c, [pw], np.array([0.5], np.float32))
    assert [_hexf(t) for t in out["objs"]] == list(objs)
    assert _hexf(out["thresh"][0]) == th
    np.testing.assert_array_equal(np.array([_hexf(t) for t in out["D_best"]], np.float32),
                                  Db.reshape(-1))
    np.testing.assert_array_equal(np.array([_hexf(t) for t in out["residuals"]]), res)
    got = [t.split(":") for t in out["scan"]]
    assert [int(g[0]) for g in got] == list(pos[:, 0])
    assert [np.float32(_hexf(g[1])) for g in got] == list(score[:, 0])
    assert [int(g[2]) for g in got] == list(comp[:, 0])
