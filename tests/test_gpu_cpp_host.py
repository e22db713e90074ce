"""A C++ host drives the drop-in entry points with no Python in the loop:
tests/cpp/host_loop.cpp, built against include/cfd_rhs.h and
libcfd_gb300.so, runs the reference host loop's stage sequence (cfd_uq ->
cfd_viscous -> cfd_weno(j) -> cfd_boundary_fill) on a case written to disk
-- on device buffers, on its host vectors directly, and as one cfd_rk3_step
call; its FLOW must match the oracle (relative L2 <= 1e-12)."""
from __future__ import annotations

import pathlib
import shutil
import subprocess

import numpy as np
import pytest

from helpers import rel_l2

pytestmark = pytest.mark.gpu
ROOT = pathlib.Path(__file__).resolve().parents[1]


def _build(tmp):
    from cfd_gb300 import abi, build
    abi.load()
    lib = build.LIB
    exe = tmp / "host_loop"
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    subprocess.run([cxx, "-std=c++17", "-O2", str(ROOT / "tests" / "cpp" / "host_loop.cpp"), "-I", str(ROOT / "include"),
                    "-L", str(lib.parent), "-lcfd_gb300", f"-Wl,-rpath,{lib.parent}", "-o", str(exe)], check=True)
    return exe


def _write_case(c, d):
    a = c.arrays
    for k in ("grid", "det", "deter", "metric", "flow"):
        np.ascontiguousarray(a[k]).tofile(d / f"{k}.bin")
    bc = c.bc
    n = []
    for t in ("outlet", "inlet", "boundary", "wall"):
        rows = getattr(bc, t) if bc is not None else np.zeros(0, np.int32)
        np.ascontiguousarray(rows, dtype=np.int32).tofile(d / f"{t}.bin")
        n.append(len(rows))
    p = c.params
    (d / "meta.txt").write_text(" ".join(str(x) for x in (
        c.g_node + 1, c.sd_node, repr(p.mach), repr(p.reynolds), repr(p.prandtl), repr(p.t_inf), repr(p.weno_eps),
        int(p.viscous), int(p.les), repr(c.dt), *n)) + "\n")


@pytest.mark.parametrize("mode", ["device", "host", "rk3"])
@pytest.mark.parametrize("name", ["channel", "vortex"])
def test_cpp_host_loop_matches_oracle(name, mode, oracle_mod, tmp_path):
    from cfd_gb300 import cases
    c = cases.channel(ni=12, nj=10, nk=6) if name == "channel" else cases.isentropic_vortex(n=12)
    exe = _build(tmp_path)
    _write_case(c, tmp_path)
    steps = 2
    r = subprocess.run([str(exe), str(tmp_path), str(steps), mode], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(tmp_path / "flow_out.bin").reshape(-1, 9)
    a = c.copy().arrays
    if c.bc is not None:
        oracle_mod.rk3_steps_bc(a, c.g_node, c.sd_node, c.params, c.dt, steps, c.bc)
    else:
        oracle_mod.rk3_steps(a, c.g_node, c.sd_node, c.params, c.dt, steps)
    assert rel_l2(got[1:], a["flow"][1:]) <= 1e-12
