"""CPU tests of the C ABI library: it loads, exports every symbol include/cdlgb.h
declares, and its host-only functions (no GPU needed) match the oracle."""
import os
import re

import numpy as np
import pytest

from oracle import search_oracle as SO

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "cdlgb.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(cdlgb_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(built_lib):
    syms = header_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(built_lib, s)]
    assert not missing, missing


def test_python_binding_covers_header(pkg, built_lib):
    from cdlmotif_gb300 import _lib
    assert set(header_symbols()) == set(_lib.SIGNATURES)


def test_params_default_match_cdl_setup(pkg, built_lib):
    import ctypes as C
    from cdlmotif_gb300._lib import CdlgbParams
    p = CdlgbParams()
    assert built_lib.cdlgb_params_default(C.byref(p)) == 0
    # src/SETUP/WRAPPER_setup.jl:1-13
    assert (p.M, p.filter_size, p.csc_iter_num, p.cdl_iter_num, p.iter_num) == (10, 4, 15, 1, 10)
    assert (p.rho, p.sigma) == (100.0, 100.0)
    assert p.lambda_ == pytest.approx(0.01)
    assert (p.sherman_const_csc, p.sherman_const_cdl) == (2.0, 2.0)


def test_transfac_c_matches_oracle(pkg, built_lib):
    rng = np.random.default_rng(0)
    for t in range(300):
        w = int(rng.integers(1, 25))
        pfm = rng.dirichlet(np.ones(4) * 0.7, size=w).T.astype(np.float32)
        assert pkg.transfac_text(pfm) == SO.transfac_text(pfm)
        assert pkg.transfac_text(pfm, True) == SO.transfac_text(SO.pwm_complement(pfm))


def test_transfac_file_writer(pkg, built_lib, tmp_path):
    pfms = [np.array([[0.25, 0.5], [0.25, 0.25], [0.25, 0.125], [0.25, 0.125]], np.float32),
            np.array([[0.7], [0.1], [0.1], [0.1]], np.float32)]
    pkg.save_pfms_as_transfac(str(tmp_path), pfms, [2, 1])
    assert (tmp_path / "d1.transfac").read_text() == SO.transfac_text(pfms[1])
    assert (tmp_path / "d2_c.transfac").read_text() == SO.transfac_text(SO.pwm_complement(pfms[0]))


def test_counts_to_pfms_c_matches_oracle(pkg, built_lib):
    import ctypes as C
    from cdlmotif_gb300._lib import ptr
    rng = np.random.default_rng(1)
    K, maxlen = 5, 9
    lens = rng.integers(3, maxlen + 1, K).astype(np.int32)
    nseq = rng.integers(1, 5000, K).astype(np.int32)
    counts = np.zeros((K, maxlen, 4), np.int32)
    for k in range(K):
        for i in range(lens[k]):
            counts[k, i] = rng.multinomial(nseq[k], [0.25] * 4)
    for smoothing, less in [(True, False), (False, False), (False, True)]:
        out = np.zeros((K, maxlen, 4), np.float32)
        st = built_lib.cdlgb_counts_to_pfms(ptr(counts, C.c_int32), ptr(nseq, C.c_int32),
                                            ptr(lens, C.c_int32), K, maxlen, 0.0295, 5.0,
                                            int(smoothing), int(less), ptr(out, C.c_float))
        assert st == 0
        ref = SO.counts_to_pfms(counts, nseq, lens, smoothing=smoothing, less_pseudocount=less)
        for k in range(K):
            np.testing.assert_array_equal(out[k, : lens[k]].T, ref[k])


def test_golden_scan_pfms_from_counts(pkg, built_lib):
    g = np.load(os.path.join(ROOT, "tests", "golden", "scan_small.npz"))
    assert SO.transfac_text(g["pfms"][0, :, : g["lens"][0]]) == str(g["transfac"])


@pytest.mark.parametrize("py_name,c_name", [("CdlgbParams", "cdlgb_params"),
                                             ("ServerConfig", "cdlgb_server_config"),
                                             ("RequestInfo", "cdlgb_request_info")])
def test_struct_layouts_match_header(pkg, built_lib, tmp_path, py_name, c_name):
    """The ctypes mirrors of the header's structs have the C structs' sizes and field
    offsets (compiled against include/cdlgb.h)."""
    import ctypes as C
    import shutil
    import subprocess
    from cdlmotif_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    st = getattr(_lib, py_name)
    names = [f[0] for f in st._fields_]
    cnames = ["lambda" if n == "lambda_" else n for n in names]
    src = tmp_path / "layout.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "cdlgb.h"\nint main(void){\n'
                   f'printf("%zu\\n", sizeof({c_name}));\n' +
                   "".join(f'printf("%zu\\n", offsetof({c_name}, {n}));\n' for n in cnames) +
                   "return 0;}\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    vals = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert vals[0] == C.sizeof(st)
    assert vals[1:] == [getattr(st, n).offset for n in names]


def test_fused_path_choice(pkg, built_lib, monkeypatch):
    """Which path a shape takes is host logic, visible without a GPU through
    cdlgb_footprint (the fused path holds other buffers than the cuFFT-transform path):
    at Lg = 832 (L = 200, W = 4) M = 34 fits only the multi-iteration X-step (the generic
    kernel's layout needs 150 KB of shared memory at 2 CTAs of 17 filters, and there is no
    one-X-step variant for 832), so the automatic choice is the fused path while that
    kernel is on and the cuFFT-transform path with CDLGB_XITER=0; M = 32 also fits the
    generic kernel (4 CTAs of 8 filters) and stays fused either way."""
    from cdlmotif_gb300 import serve

    def fp(M, mode):
        return serve.footprint_bytes(pkg.CDLSetup(M=M, filter_size=4), 200, 100, mode)

    monkeypatch.delenv("CDLGB_XITER", raising=False)
    monkeypatch.delenv("CDLGB_GENERIC_FFT", raising=False)
    monkeypatch.delenv("CDLGB_CLUSTER", raising=False)
    fused34, fused32 = fp(34, 2), fp(32, 2)
    assert fp(34, 0) == fused34 and fp(32, 0) == fused32
    monkeypatch.setenv("CDLGB_XITER", "0")
    assert fp(34, 0) != fused34
    assert fp(32, 0) == fp(32, 2) == fused32


_C_SCALARS = {"int32_t": (4, "i"), "uint32_t": (4, "i"), "int64_t": (8, "i"), "uint64_t": (8, "i"),
              "size_t": (8, "i"), "int": (4, "i"), "uint8_t": (1, "i"), "char": (1, "i"),
              "float": (4, "f"), "double": (8, "f")}


def _c_param(decl):
    """(pointer depth, base type) of one parameter declaration"""
    decl = re.sub(r"\bconst\b", "", decl).strip()
    depth = decl.count("*")
    words = decl.replace("*", " ").split()
    base = words[0] if len(words) > 1 or depth else words[0]
    return depth, base


def _header_params():
    txt = open(os.path.join(ROOT, "include", "cdlgb.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    out = {}
    for ret, name, params in re.findall(r"([\w\s\*]+?)\b(cdlgb_\w+)\s*\(([^()]*)\)\s*;", txt):
        ps = [p for p in params.split(",") if p.strip() and p.strip() != "void"]
        out[name] = (_c_param(ret + " r"), [_c_param(p) for p in ps])
    return out


def _ct_kind(t):
    import ctypes as C
    if t is C.c_void_p or t is C.c_char_p:
        return ("ptr", None)
    if isinstance(t, type) and issubclass(t, C._Pointer):
        return ("ptr", t._type_)
    if isinstance(t, type) and issubclass(t, C.Structure):
        return ("struct", t)
    cls = "f" if t in (C.c_float, C.c_double) else "i"
    return ("scalar", (C.sizeof(t), cls))


def _compatible(cparam, ct):
    import ctypes as C
    depth, base = cparam
    kind, info = _ct_kind(ct)
    if depth == 0:
        return kind == "scalar" and _C_SCALARS.get(base) == info
    if kind != "ptr":
        return False
    if info is None:                      # c_void_p / c_char_p: any pointer
        return True
    if depth > 1:                         # T** against POINTER(c_void_p)
        return _ct_kind(info)[0] == "ptr"
    if base in _C_SCALARS:
        pk = _ct_kind(info)
        return pk[0] == "scalar" and pk[1] == _C_SCALARS[base]
    return issubclass(info, C.Structure) or info is C.c_void_p   # struct or opaque pointee


def test_ctypes_signatures_match_header(pkg, built_lib):
    """Every ctypes signature of the binding has the header prototype's parameter count
    and, parameter by parameter, the same kind: scalars of the same size and class,
    pointers to elements of the same size and class (c_void_p for any pointer)."""
    from cdlmotif_gb300 import _lib
    protos = _header_params()
    assert len(protos) == len(_lib.SIGNATURES)
    for name, (res, args) in _lib.SIGNATURES.items():
        cret, cparams = protos[name]
        assert len(args) == len(cparams), name
        for i, (cp, ct) in enumerate(zip(cparams, args)):
            assert _compatible(cp, ct), (name, i, cp, ct)
        assert _compatible(cret, res), (name, "result", cret, res)
