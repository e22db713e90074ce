"""Restart pair and Tecplot output in the reference's formats
(Tecplot_output_files.cpp:92-123, presolver.cpp:86-183)."""
from __future__ import annotations

import numpy as np


def _flow(seed=0, n=50):
    from cfd_gb300 import layout
    rng = np.random.default_rng(seed)
    f = np.zeros((n + 1, layout.NFLOW))
    f[1:] = rng.uniform(0.5, 2.0, (n, layout.NFLOW))
    return f


def test_restart_round_trip_is_exact(pkg, tmp_path):
    from cfd_gb300 import files, layout
    f = _flow()
    files.write_restart(tmp_path, f, 50, 1234, 1)
    values, it, nxt = files.read_restart(tmp_path, 50)
    assert it == 1234 and nxt == 2
    g = files.restart_flow(np.zeros_like(f), values, mach=0.5)
    for k in files.RESTART_FIELDS:
        assert np.array_equal(g[1:, layout.FLOW[k]], f[1:, layout.FLOW[k]])
    lines = (tmp_path / "restart_file_1.neu").read_text().splitlines()
    assert len(lines) == 50 and len(lines[0].split("\t")) == 9 and lines[0].split("\t")[-1] == "1234"


def test_newest_complete_file_wins(pkg, tmp_path):
    from cfd_gb300 import files
    f1, f2 = _flow(1), _flow(2)
    files.write_restart(tmp_path, f1, 50, 100, 1)
    files.write_restart(tmp_path, f2, 50, 200, 2)
    values, it, nxt = files.read_restart(tmp_path, 50)
    assert it == 200 and nxt == 1
    # an interrupted write of file 2 (truncated) falls back to file 1
    p2 = tmp_path / "restart_file_2.neu"
    p2.write_text("\n".join(p2.read_text().splitlines()[:20]) + "\n")
    values, it, nxt = files.read_restart(tmp_path, 50)
    assert it == 100 and nxt == 2
    # mixed iterations inside a file make it incomplete too
    files.write_restart(tmp_path, f2, 50, 300, 2)
    lines = p2.read_text().splitlines()
    lines[-1] = "\t".join(lines[-1].split("\t")[:-1] + ["299"])
    p2.write_text("\n".join(lines) + "\n")
    assert files.read_restart(tmp_path, 50)[1] == 100
    (tmp_path / "empty").mkdir()
    assert files.read_restart(tmp_path / "empty", 50) is None


def test_tecplot_file_and_ducros_sensor(pkg, tmp_path):
    """Variables in the reference's order; the Ducros sensor is 0 for a
    divergence-free field and 1 for a curl-free compressive one."""
    from cfd_gb300 import cases, files, layout
    c = cases.taylor_green(n=8)
    p = files.write_tecplot(tmp_path / "nodefile_7.dat", c, c.arrays["flow"], 7)
    lines = p.read_text().splitlines()
    assert lines[1] == "VARIABLES = X, Y, Z, U, V, W, RHO, P, T, e, mu, loc, Proc, DUCROS,"
    assert "I= 8 J= 8 K= 8" in lines[2] and "SOLUTIONTIME= 7" in lines[2]
    assert len(lines) == 3 + 8 ** 3 and len(lines[3].split("\t")) == 14
    # Taylor-Green velocity is solenoidal (up to truncation error)
    c16 = cases.taylor_green(n=16)
    d = files.ducros_sensor(c16.arrays["flow"], c16.arrays["metric"], c16.shape)
    assert np.median(d) < 1e-6 and np.percentile(d, 99) < 0.05   # ill-defined only at stagnation points
    # radial compression u = -x on a uniform periodic-looking patch: curl free
    f = c.arrays["flow"].copy()
    x, y, z = (c.arrays["grid"][k][1:] for k in ("x", "y", "z"))
    f[1:, layout.FLOW["u"]] = np.sin(x)
    f[1:, layout.FLOW["v"]] = np.sin(y)
    f[1:, layout.FLOW["w"]] = np.sin(z)
    d = files.ducros_sensor(f, c.arrays["metric"], c.shape)
    assert np.median(d) > 0.9


def test_tecplot_of_a_ghosted_lattice(pkg, tmp_path):
    from cfd_gb300 import cases, files
    c = cases.channel(ni=8, nj=6, nk=4)
    p = files.write_tecplot(tmp_path / "nodefile_0.dat", c, c.arrays["flow"], 0)
    lines = p.read_text().splitlines()
    assert "I= 8 J= 6 K= 4" in lines[2] and len(lines) == 3 + 8 * 6 * 4
    locs = {int(l.split("\t")[11]) for l in lines[3:]}
    assert locs == {0, 1, 3}
