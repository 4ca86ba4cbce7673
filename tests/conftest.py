"""Shared test setup: the `gpu` marker, and loaders for the engine package and the oracle.

The engine package directory is named coupled-cluster-nuclearmatter_gb300 (not a
Python identifier), so it is loaded by path under the module name ccnm_gb300.
"""
import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "coupled-cluster-nuclearmatter_gb300")
ORACLE_DIR = os.path.join(ROOT, "oracle")
if ORACLE_DIR not in sys.path:
    sys.path.insert(0, ORACLE_DIR)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def load_pkg():
    if "ccnm_gb300" in sys.modules:
        return sys.modules["ccnm_gb300"]
    spec = importlib.util.spec_from_file_location(
        "ccnm_gb300", os.path.join(PKG_DIR, "__init__.py"), submodule_search_locations=[PKG_DIR])
    m = importlib.util.module_from_spec(spec)
    sys.modules["ccnm_gb300"] = m
    spec.loader.exec_module(m)
    return m


def build_pkg():
    spec = importlib.util.spec_from_file_location("ccnm_gb300_build", os.path.join(PKG_DIR, "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    return b.build()


@pytest.fixture(scope="session")
def ccx():
    build_pkg()
    return load_pkg()


@pytest.fixture(scope="session")
def O():
    import oracle
    oracle.build()
    return oracle


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
