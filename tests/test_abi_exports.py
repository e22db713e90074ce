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
    assert ctypes.sizeof(abi.Params) == 64   # 5 doubles, 4 int32, smagorinsky_cs


@pytest.mark.parametrize("lang,compiler", [("c", "gcc"), ("c++", "g++")])
def test_header_compiles_standalone(tmp_path, lang, compiler):
    """include/cfd_rhs.h is self-contained C (no CUDA or torch types)."""
    import shutil
    import subprocess
    if shutil.which(compiler) is None:
        pytest.skip(f"{compiler} not available")
    src = tmp_path / ("t.c" if lang == "c" else "t.cpp")
    src.write_text('#include "cfd_rhs.h"\n'
                   '_Static_assert(sizeof(cfd_grid_t) == 56, "GRID");\n' if lang == "c" else
                   '#include "cfd_rhs.h"\n'
                   'static_assert(sizeof(cfd_grid_t) == 56, "GRID");\n'
                   'static_assert(sizeof(cfd_flow_t) == 72, "FLOW");\n'
                   'static_assert(sizeof(cfd_column_t) == 40, "column");\n'
                   'static_assert(sizeof(cfd_metric_t) == 504, "metric");\n'
                   'static_assert(sizeof(cfd_determ_t) == 48, "determ");\n'
                   'static_assert(sizeof(cfd_roe_t) == 288, "roe");\n'
                   'int main() { cfd_params_t p; cfd_params_default(&p); return 0; }\n')
    r = subprocess.run([compiler, "-fsyntax-only", "-Wall", "-Werror", f"-I{ROOT / 'include'}", str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_static_node_limit_comes_from_the_header(pkg):
    from cfd_gb300 import abi
    text = (ROOT / "include" / "cfd_rhs.h").read_text()
    m = re.search(r"^#define\s+CFD_STATIC_MAX_NODES\s+(\d+)", text, flags=re.M)
    assert m and int(m.group(1)) == abi.STATIC_MAX_NODES


def test_ctypes_mirrors_match_the_header(pkg, tmp_path):
    """The Python mirrors of the header's structs (abi.Params, Geometry,
    KernelTime, SolverInfo, BatchInfo) have the C layout: size and every
    field's offset, as a C compiler lays out include/cfd_rhs.h."""
    import shutil
    import subprocess
    from cfd_gb300 import abi
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    mirrors = {"cfd_params_t": abi.Params, "cfd_geometry_t": abi.Geometry, "cfd_kernel_time_t": abi.KernelTime,
               "cfd_solver_info_t": abi.SolverInfo, "cfd_batch_info_t": abi.BatchInfo}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "cfd_rhs.h"', "int main(void) {"]
    for cname, py in mirrors.items():
        lines.append(f'    printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'    printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["    return 0;", "}"]
    src, exe = tmp_path / "layout.c", tmp_path / "layout"
    src.write_text("\n".join(lines) + "\n")
    r = subprocess.run(["gcc", "-Wall", "-Werror", f"-I{ROOT / 'include'}", str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = dict(((ln.split()[0], ln.split()[1]), int(ln.split()[2]))
               for ln in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines())
    for cname, py in mirrors.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)
