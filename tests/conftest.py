"""Shared fixtures: the package (directory name has hyphens, so it is loaded
with importlib), the CPU oracle binding, and the ``gpu`` marker."""
from __future__ import annotations

import importlib
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]
if str(REPO) not in sys.path:
    sys.path.insert(0, str(REPO))
if str(REPO / "oracle") not in sys.path:
    sys.path.insert(0, str(REPO / "oracle"))

PKG_NAME = "d3q19-single-phase_gb300"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built liblbm_gb300.so")


def load_pkg():
    return importlib.import_module(PKG_NAME)


@pytest.fixture(scope="session")
def pkg():
    return load_pkg()


@pytest.fixture(scope="session")
def orc():
    import oracle as o  # noqa: WPS433  (test infrastructure)
    o.build()
    return o


@pytest.fixture(scope="session")
def lib(pkg):
    """The built C ABI library; tests that need it fail loudly if it is missing."""
    return pkg.load_library()
