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


_C_TO_JL = {"int32_t": "Int32", "uint32_t": "UInt32", "int64_t": "Int64", "uint64_t": "UInt64",
            "float": "Float32", "double": "Float64"}
# the Julia mirrors of the header's structs
_MIRRORS = {"CdlgbParams": "cdlgb_params", "ServerConfig": "cdlgb_server_config"}


def header_struct_fields(name):
    txt = _strip_comments(open(os.path.join(ROOT, "include", "cdlgb.h")).read())
    body = re.search(r"typedef struct\s*\{([^}]*)\}\s*" + name + r"\s*;", txt).group(1)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        ctype, names = decl.split(None, 1)
        fields += [(n.strip(), _C_TO_JL[ctype]) for n in names.split(",")]
    return fields


def doc_struct_fields(name):
    txt = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    body = re.search(r"struct " + name + r"\b(.*?)\bend\b", txt, flags=re.S).group(1)
    body = re.sub(r"#[^\n]*", "", body)
    return re.findall(r"(\w+)::(\w+)", body)


def test_struct_mirrors_match_header():
    """Field for field, in order, with the same types: a missing or reordered field
    shifts every later one in the library's view of the struct."""
    for jl, c in _MIRRORS.items():
        assert doc_struct_fields(jl) == header_struct_fields(c), jl


def test_struct_constructor_calls_pass_every_field():
    txt = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    for jl in _MIRRORS:
        n = len(doc_struct_fields(jl))
        for args in re.findall(r"\b" + jl + r"\(([^()]*(?:\([^()]*\)[^()]*)*)\)", txt):
            # split on top-level commas
            depth, count = 0, 1
            for ch in args:
                depth += ch in "([{"
                depth -= ch in ")]}"
                count += ch == "," and depth == 0
            assert count == n, (jl, count, n)
