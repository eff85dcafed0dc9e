"""Every C entry point refuses null handles and null or zero arguments with a status
(or, for the *_last_error functions, a message; the *_destroy functions accept null,
as free does) instead of crashing.  The calls run in a child process that names each
function before calling it, so a crash names the function."""
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_CHILD = r'''
import ctypes as C, importlib.util, sys
sys.path.insert(0, ROOT)
spec = importlib.util.spec_from_file_location("cdlmotif_gb300", ROOT + "/cdlmotif.jl_gb300/__init__.py",
                                              submodule_search_locations=[ROOT + "/cdlmotif.jl_gb300"])
pkg = importlib.util.module_from_spec(spec); sys.modules["cdlmotif_gb300"] = pkg; spec.loader.exec_module(pkg)
from cdlmotif_gb300 import _lib
L = _lib.lib()
for name in sorted(_lib.SIGNATURES):
    res, args = _lib.SIGNATURES[name]
    vals = []
    for t in args:
        if t in (C.c_float, C.c_double):
            vals.append(0.0)
        elif t in (C.c_void_p, C.c_char_p) or (isinstance(t, type) and issubclass(t, C._Pointer)):
            vals.append(None)
        else:
            vals.append(0)
    print("CALL", name, flush=True)
    r = getattr(L, name)(*vals)
    print("RET", name, r.decode() if isinstance(r, bytes) else r, flush=True)
'''


def test_null_arguments_are_refused(pkg, built_lib):
    p = subprocess.run([sys.executable, "-c", "ROOT = %r\n" % ROOT + _CHILD], capture_output=True,
                       text=True, timeout=300)
    calls = [l.split()[1] for l in p.stdout.splitlines() if l.startswith("CALL")]
    assert p.returncode == 0, "crashed in %s: %s" % (calls[-1] if calls else "?", p.stderr[-400:])
    from cdlmotif_gb300 import _lib
    rets = {}
    for l in p.stdout.splitlines():
        if l.startswith("RET"):
            _, name, val = l.split(" ", 2)
            rets[name] = val
    assert set(rets) == set(_lib.SIGNATURES)
    for name, val in rets.items():
        if name.endswith("_last_error"):
            assert val, name
        elif name.endswith("_destroy"):
            assert int(val) == 0, name
        else:
            assert int(val) == -1, (name, val)        # CDLGB_EINVAL
