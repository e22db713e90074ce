"""Shared fixtures: the package (under the import name cfd_gb300), the CPU
oracle, and the ``gpu`` marker for tests that need a CUDA device."""
from __future__ import annotations

import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import __graft_entry__  # noqa: E402

__graft_entry__.load_package()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def pkg():
    return sys.modules["cfd_gb300"]


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def ctx(pkg):
    from cfd_gb300 import runtime
    c = runtime.Context(0)
    yield c
    c.close()
