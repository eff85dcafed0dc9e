import importlib.util
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "cdlmotif.jl_gb300")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libcdlgb.so")


def load_pkg():
    """Import the package directory ``cdlmotif.jl_gb300`` (its name is not a Python
    identifier) as ``cdlmotif_gb300``."""
    name = "cdlmotif_gb300"
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(name, os.path.join(PKG_DIR, "__init__.py"),
                                                  submodule_search_locations=[PKG_DIR])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def pkg():
    return load_pkg()


@pytest.fixture(scope="session")
def built_lib(pkg):
    """libcdlgb.so, built if missing."""
    from cdlmotif_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pkg.build()
    return _lib.lib()


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def random_onehot(rng, N, L):
    bases = rng.integers(0, 4, size=(N, L))
    S = np.zeros((N, L, 4), np.float32)
    S[np.arange(N)[:, None], np.arange(L)[None, :], bases] = 1.0
    return S.reshape(N, 4 * L), bases
