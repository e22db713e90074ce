"""The C-ABI library loads on a host without a GPU and exports every entry
point that include/cfd_rhs.h declares (no compute calls)."""
from __future__ import annotations

import ctypes
import pathlib
import re

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]


def declared_functions():
    names = []
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(cfd_[a-z_0-9]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for required in ("cfd_uq", "cfd_viscous", "cfd_weno", "cfd_ctx_create", "cfd_solver_create",
                     "cfd_solver_step", "cfd_buffer_alloc"):
        assert required in names


def test_library_exports_every_declared_symbol(pkg):
    from cfd_gb300 import abi
    lib = abi.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_bindings_cover_header(pkg):
    from cfd_gb300 import abi
    assert set(declared_functions()) <= set(abi.PROTOTYPES)


def test_missing_library_fails_loudly(pkg, tmp_path, monkeypatch):
    from cfd_gb300 import abi
    monkeypatch.setattr(abi, "_lib", None)
    monkeypatch.setattr(abi._build, "build", lambda *a, **k: None)
    with pytest.raises(RuntimeError):
        abi.load(tmp_path / "absent.so")


def test_struct_sizes_match_reference(pkg):
    from cfd_gb300 import abi, layout
    assert layout.GRID_DTYPE.itemsize == 56
    assert layout.BYTES_PER_NODE_REFERENCE == 1376
    assert ctypes.sizeof(abi.Params) == 56
