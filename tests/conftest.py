"""Shared test set-up: the `gpu` marker, the package loader and the oracle build.

The package directory is named ``eulerian-liquid_gb300`` (not an importable identifier), so it
is loaded as the package ``eulerian_liquid_gb300`` from its path.
"""

import importlib.util
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def load_package():
    name = "eulerian_liquid_gb300"
    if name in sys.modules:
        return sys.modules[name]
    pkg_dir = os.path.join(ROOT, "eulerian-liquid_gb300")
    spec = importlib.util.spec_from_file_location(name, os.path.join(pkg_dir, "__init__.py"),
                                                  submodule_search_locations=[pkg_dir])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")


@pytest.fixture(scope="session")
def el():
    return load_package()


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.lib()
    return oracle


def rel_err(a, b):
    """max |a - b| / max |b|, the norm-wise relative error used throughout the parity tests."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (den if den > 0 else 1.0))
