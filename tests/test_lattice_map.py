"""Host-side lattice detection (csrc/lattice_host.h) on the CPU: the checks
that decide whether a reference neighbour table runs on the face-based
lattice kernels, and the geometry conversion, compiled with g++ and run on
the case generators' tables.  These per-node passes run on several host
threads; the test covers natural and shuffled row orders, ghost layers,
tables that are not lattices, and a corrupted neighbour index."""
from __future__ import annotations

import pathlib
import shutil
import subprocess

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
CSRC = ROOT / "high-order-accurate-cfd-solver-code-for-heterogenous-hardware-cpu-and-gpgpu-_gb300" / "csrc"
PRIME = (1 << 61) - 1


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path_factory.mktemp("latmap") / "lattice_map_check"
    subprocess.run([cxx, "-std=c++17", "-O2", "-pthread", "-I", str(ROOT / "include"), "-I", str(CSRC),
                    str(ROOT / "tests" / "cpp" / "lattice_map_check.cpp"), "-o", str(exe)], check=True)
    return exe


def run(checker, tmp_path, arrays, g_node, sd_node):
    for k in ("grid", "metric", "deter", "det"):
        np.ascontiguousarray(arrays[k]).tofile(tmp_path / f"{k}.bin")
    out = subprocess.run([str(checker), str(tmp_path), str(g_node), str(sd_node)], capture_output=True, text=True,
                         check=True).stdout.split()
    assert out[0] == "ok" and out[7] == "faces"
    return {"ok": int(out[1]), "dims": tuple(int(x) for x in out[2:5]), "per": int(out[5]), "locdirs": int(out[6]),
            "faces": int(out[8]), "row_hash": int(out[9]), "soa": float(out[10])}


def row_hash(row_of):
    n = np.arange(len(row_of), dtype=object)
    return int(sum(int(a) * int(b) for a, b in zip(n, row_of)) % PRIME)


def soa_sum(arrays, row_of):
    """Sum of the lattice geometry (node metrics, det, +1/2 face metrics, face
    dets) for the rows in lattice order."""
    m = arrays["metric"][row_of]
    d = arrays["deter"][row_of]
    total = m[:, :9].sum() + arrays["det"][row_of].sum()
    for k in range(3):
        total += m[:, 9 * (1 + 2 * k) + 3 * k: 9 * (1 + 2 * k) + 3 * k + 3].sum() + d[:, 2 * k].sum()
    return float(total)


def test_periodic_lattice_in_row_order(pkg, checker, tmp_path):
    from cfd_gb300 import cases
    c = cases.isentropic_vortex(n=12, shape=(12, 10, 8))
    r = run(checker, tmp_path, c.arrays, c.g_node, c.sd_node)
    rows = np.arange(1, c.g_node + 1)
    assert r["ok"] == 1 and r["dims"] == (12, 10, 8) and r["per"] == 7 and r["faces"] == 1
    assert r["row_hash"] == row_hash(rows)
    assert r["soa"] == pytest.approx(soa_sum(c.arrays, rows), rel=1e-9)


def shuffled(c, seed):
    """The same table with rows 1..g_node renumbered by a random permutation."""
    rng = np.random.default_rng(seed)
    R = c.g_node
    new_of_old = np.zeros(R + 1, dtype=np.int64)
    new_of_old[1:] = rng.permutation(R) + 1
    a = {k: v.copy() for k, v in c.arrays.items()}
    old_of_new = np.zeros(R + 1, dtype=np.int64)
    old_of_new[new_of_old] = np.arange(R + 1)
    for k in ("grid", "metric", "deter", "det"):
        a[k] = c.arrays[k][old_of_new]
    for s in ("N0", "N1", "N2", "N3", "N4", "N5"):
        a["grid"][s] = new_of_old[a["grid"][s]]
    return a, new_of_old, old_of_new


@pytest.mark.parametrize("shape", [(9, 7, 6), (64, 48, 48)])
def test_periodic_lattice_with_shuffled_rows(pkg, checker, tmp_path, shape):
    """The lattice is found from whichever node is row 1: node (i, j, k) of
    the map is the original node shifted by that node's coordinates.  The
    larger table (147,456 nodes) runs the per-node passes on several
    threads."""
    from cfd_gb300 import cases
    c = cases.isentropic_vortex(n=shape[0], shape=shape)
    a, new_of_old, old_of_new = shuffled(c, 3)
    r = run(checker, tmp_path, a, c.g_node, c.sd_node)
    assert r["ok"] == 1 and r["dims"] == shape and r["per"] == 7 and r["faces"] == 1
    o = old_of_new[1] - 1                            # original node now numbered row 1
    oi, oj, ok_ = o % shape[0], (o // shape[0]) % shape[1], o // (shape[0] * shape[1])
    k, j, i = np.meshgrid(np.arange(shape[2]), np.arange(shape[1]), np.arange(shape[0]), indexing="ij")
    orig = ((i + oi) % shape[0]) + shape[0] * (((j + oj) % shape[1]) + shape[1] * ((k + ok_) % shape[2]))
    expect = new_of_old[orig.ravel() + 1]
    assert r["row_hash"] == row_hash(expect)
    assert r["soa"] == pytest.approx(soa_sum(a, expect), rel=1e-9)   # summation order differs


def test_corrupted_neighbour_is_not_a_lattice(pkg, checker, tmp_path):
    from cfd_gb300 import cases
    c = cases.isentropic_vortex(n=8, shape=(8, 8, 6))
    a = {k: v.copy() for k, v in c.arrays.items()}
    a["grid"]["N0"][100] = a["grid"]["N0"][101]      # row 100's +j neighbour now wrong
    assert run(checker, tmp_path, a, c.g_node, c.sd_node)["ok"] == 0


@pytest.mark.parametrize("maker,per,locdirs,faces", [("channel", 5, 2, 1), ("naca", 5, 2, 1), ("ghost_box", 0, 7, 0)])
def test_lattices_with_ghost_layers(pkg, checker, tmp_path, maker, per, locdirs, faces):
    """Walls in y (channel), wall and far field in the O-grid's radial
    direction (NACA0012), ghosts on every side of a box whose ghosts carry
    their own metrics (a lattice, but faces not single-valued)."""
    from cfd_gb300 import cases
    c = {"channel": lambda: cases.channel(ni=16, nj=12, nk=8),
         "naca": lambda: cases.naca0012(ni=64, nj=24, nk=4),
         "ghost_box": lambda: cases.ghost_box(shape=(9, 8, 7), seed=5)}[maker]()
    r = run(checker, tmp_path, c.arrays, c.g_node, c.sd_node)
    assert r["ok"] == 1 and r["per"] == per and r["locdirs"] == locdirs and r["faces"] == faces
    assert r["dims"][0] * r["dims"][1] * r["dims"][2] == c.g_node
