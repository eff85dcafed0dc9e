"""Every C entry point refuses null handles and null or zero arguments with a status
(or, for the *_last_error functions, a message; the *_destroy functions accept null,
as free does) instead of crashing.  The calls run in a child process that names each
function before calling it, so a crash names the function."""
import os
import subprocess
import sys

import pytest

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


def test_creation_failures_carry_their_message(pkg, built_lib):
    """Failures with no handle to hold the message (creating a context, a record or a
    server; the allocation-free objective) leave it for the calling thread, and the
    Python wrappers raise with it.  The checks below run before any device call."""
    import ctypes as C
    from cdlmotif_gb300 import _lib, serve
    with pytest.raises(pkg.CDLGBError) as e:
        pkg.CDL(pkg.CDLSetup(M=4, filter_size=2), fft_mode=5)
    assert e.value.status == -1 and "fft_mode=5" in str(e.value)
    with pytest.raises(pkg.CDLGBError) as e:
        pkg.ActivationRecord(10, 70000, 4)
    assert e.value.status == -1 and "L <= 65535" in str(e.value)
    with pytest.raises(pkg.CDLGBError) as e:
        serve.Server(pkg.CDLSetup(M=4, filter_size=2), slots=65, hbm_budget=1 << 30)
    assert e.value.status == -1 and "slots=65" in str(e.value)
    L = _lib.lib()
    obj = C.c_double()
    assert L.cdlgb_objective_noalloc(None, None, None, 0, 0, 0, 0, 0.0, C.byref(obj), None) == -1
    assert b"cdlgb_objective_noalloc" in L.cdlgb_last_error(None)
    # the message belongs to the thread that failed
    import threading
    seen = []
    t = threading.Thread(target=lambda: seen.append(L.cdlgb_last_error(None)))
    t.start()
    t.join()
    assert seen == [b"null context"]
