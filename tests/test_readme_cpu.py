"""The README's Python example names only functions, classes and methods the package
has, with parameters they take (no GPU: the calls are not made)."""
import inspect
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _example():
    txt = open(os.path.join(ROOT, "README.md")).read()
    blocks = re.findall(r"```python\n(.*?)```", txt, flags=re.S)
    assert blocks
    return blocks[0]


def _kwargs_ok(fn, names):
    sig = inspect.signature(fn)
    if any(p.kind == p.VAR_KEYWORD for p in sig.parameters.values()):
        return True
    return set(names) <= set(sig.parameters)


def test_readme_example_names_exist(pkg):
    code = _example()
    for name, args in re.findall(r"\bcdl\.(\w+)\(([^()]*(?:\([^()]*\)[^()]*)*)\)", code):
        assert hasattr(pkg, name), name
        kw = re.findall(r"\b(\w+)=", args)
        assert _kwargs_ok(getattr(pkg, name), kw), (name, kw)
    for name, args in re.findall(r"\bc\.(\w+)\(([^()]*)\)", code):
        assert hasattr(pkg.CDL, name), name
        assert _kwargs_ok(getattr(pkg.CDL, name), re.findall(r"\b(\w+)=", args)), name
    for attr in re.findall(r"\bsetup\.(\w+)", code):
        assert attr in inspect.signature(pkg.CDLSetup).parameters, attr
