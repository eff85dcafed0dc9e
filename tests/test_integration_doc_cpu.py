"""The Julia shim's ccalls agree with include/cdlgb.h: every symbol is
declared, with as many parameters, each of the same kind (pointer, integer or floating
point) and the same result kind.  Read from the two files; no GPU, no Julia."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _strip_comments(txt):
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return re.sub(r"//[^\n]*", "", txt)


def _c_kind(decl):
    decl = decl.strip()
    if "*" in decl or "[" in decl:
        return "ptr"
    if re.search(r"\b(float|double)\b", decl):
        return "float"
    return "int"


def header_prototypes():
    txt = _strip_comments(open(os.path.join(ROOT, "include", "cdlgb.h")).read())
    out = {}
    for ret, name, params in re.findall(r"([\w\s\*]+?)\b(cdlgb_\w+)\s*\(([^()]*)\)\s*;", txt):
        ps = [p for p in params.split(",") if p.strip() and p.strip() != "void"]
        out[name] = (_c_kind(ret), [_c_kind(p) for p in ps])
    return out


def _jl_kind(t):
    t = t.strip()
    if re.match(r"(Ptr|Ref|CuPtr)\{", t) or t in ("Cstring", "Ptr"):
        return "ptr"
    if t in ("Float32", "Float64", "Cfloat", "Cdouble"):
        return "float"
    return "int"


def doc_ccalls():
    txt = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    calls = re.findall(r"ccall\(\(:(cdlgb_\w+),\s*libcdlgb\),\s*([\w{}]+),\s*\(([^()]*)\)", txt)
    assert len(calls) >= 20
    return calls


def test_ccalls_match_header():
    protos = header_prototypes()
    assert "cdlgb_create" in protos and "cdlgb_scan_fwd" in protos
    for name, ret, args in doc_ccalls():
        assert name in protos, name
        cret, cargs = protos[name]
        jargs = [a for a in args.split(",") if a.strip()]
        assert len(jargs) == len(cargs), (name, jargs, cargs)
        assert [_jl_kind(a) for a in jargs] == cargs, (name, jargs, cargs)
        assert _jl_kind(ret) == cret, (name, ret, cret)
