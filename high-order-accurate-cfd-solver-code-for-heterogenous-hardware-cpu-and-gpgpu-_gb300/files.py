"""Restart and Tecplot files in the reference's formats (host side).

* Restart pair ``restart_file_1.neu`` / ``restart_file_2.neu``
  (Tecplot_output_files.cpp:112-123 writes one, presolver.cpp:86-183 picks
  one on start-up): one line per owned node 1..NUMNP,
  ``u v w rho p t e mu iter`` separated by tabs.  Writes alternate between
  the two files, so an interrupted write leaves the other one whole; on
  start-up the file whose lines are complete and carry the newest iteration
  is used.  Values are written with 17 significant digits (the reference
  writes C++ stream defaults, 6 digits), so a restart reproduces the state
  bit for bit; the reference's reader takes either.
* Tecplot ASCII ``nodefile_<iter>.dat`` (Tecplot_output_files.cpp:92-110):
  the reference's variable list X, Y, Z, U, V, W, RHO, P, T, e, mu, loc,
  Proc, DUCROS in POINT packing.  The reference writes a FEBRICK zone from
  the element list of its mesh file; lattice cases have no element list and
  are written as the equivalent ordered zone (I, J, K = the owned box).
  DUCROS is the Ducros shock sensor of viscous_terms.cpp:260-266,
  div^2 / (div^2 + |curl|^2 + 1e-29), with velocity gradients from the
  fourth-order index derivatives and node metrics of the viscous terms.
"""
from __future__ import annotations

import os
import pathlib

import numpy as np

from . import layout as L

RESTART_FIELDS = ("u", "v", "w", "rho", "p", "t", "e", "mu")


def restart_path(directory, num: int) -> pathlib.Path:
    return pathlib.Path(directory) / f"restart_file_{num}.neu"


def write_restart(directory, flow: np.ndarray, sd_node: int, iteration: int, restart_num: int) -> pathlib.Path:
    """Writes rows 1..sd_node of FLOW to restart_file_<restart_num>.neu
    (written to a temporary name, then renamed into place).  Returns the
    path; the next write should go to the other number."""
    if restart_num not in (1, 2):
        raise ValueError("restart_num is 1 or 2")
    cols = [L.FLOW[k] for k in RESTART_FIELDS]
    rows = flow[1:sd_node + 1][:, cols]
    path = restart_path(directory, restart_num)
    tmp = path.with_suffix(".neu.tmp")
    it = np.full((rows.shape[0], 1), int(iteration), dtype=np.int64)
    with open(tmp, "w") as fp:
        for r, i in zip(rows, it[:, 0]):
            fp.write("\t".join(f"{x:.17g}" for x in r) + f"\t{i}\n")
    os.replace(tmp, path)
    return path


def _read_one(path: pathlib.Path, sd_node: int):
    """(values (sd_node, 8), iteration) of a complete restart file, else None."""
    if not path.exists():
        return None
    try:
        data = np.loadtxt(path, ndmin=2)
    except ValueError:
        return None
    if data.shape != (sd_node, 9):
        return None
    its = data[:, 8]
    if not np.all(its == its[0]) or its[0] < 0:
        return None
    return data[:, :8], int(its[0])


def read_restart(directory, sd_node: int):
    """The newest complete file of the pair: (values (sd_node, 8) in
    RESTART_FIELDS order, iteration, number to write next), or None when
    neither file is complete (presolver.cpp:86-183 semantics)."""
    got = {n: _read_one(restart_path(directory, n), sd_node) for n in (1, 2)}
    valid = {n: g for n, g in got.items() if g is not None}
    if not valid:
        return None
    num = max(valid, key=lambda n: valid[n][1])
    values, iteration = valid[num]
    return values, iteration, 3 - num


def restart_flow(template: np.ndarray, values: np.ndarray, mach: float) -> np.ndarray:
    """FLOW rows 0..g_node: `template` with rows 1..sd_node replaced by a
    restart's values; the sound speed follows from p and rho."""
    flow = template.copy()
    n = values.shape[0]
    for k, name in enumerate(RESTART_FIELDS):
        flow[1:n + 1, L.FLOW[name]] = values[:, k]
    rows = flow[1:n + 1]
    rows[:, L.FLOW["a"]] = np.sqrt(1.4 * rows[:, L.FLOW["p"]] / rows[:, L.FLOW["rho"]])
    return flow


def _index_derivative(f: np.ndarray, axis: int, periodic: bool) -> np.ndarray:
    """4th-order central index derivative (one-sided 2nd order at the two
    outermost layers of a non-periodic direction)."""
    if periodic:
        r = lambda o: np.roll(f, -o, axis=axis)   # noqa: E731
        return (1.0 / 12.0) * (8.0 * (r(1) - r(-1)) - (r(2) - r(-2)))
    g = np.moveaxis(f, axis, 0)
    n = g.shape[0]
    d = np.empty_like(g)
    if n >= 5:
        d[2:n - 2] = (1.0 / 12.0) * (8.0 * (g[3:n - 1] - g[1:n - 3]) - (g[4:n] - g[0:n - 4]))
    d[0] = g[1] - g[0]
    d[n - 1] = g[n - 1] - g[n - 2]
    if n >= 3:
        d[1] = 0.5 * (g[2] - g[0])
        d[n - 2] = 0.5 * (g[n - 1] - g[n - 3])
    return np.moveaxis(d, 0, axis)


def ducros_sensor(flow: np.ndarray, metric: np.ndarray, shape, periodic=(True, True, True)) -> np.ndarray:
    """Ducros sensor of the owned box (rows 1..ni*nj*nk in i-fastest order)."""
    ni, nj, nk = shape
    n = ni * nj * nk
    f = flow[1:n + 1].reshape(nk, nj, ni, L.NFLOW)
    m = metric[1:n + 1, :9].reshape(nk, nj, ni, 3, 3)   # m[..., d, b] = d zeta_d / d x_b
    u = np.stack([f[..., L.FLOW["u"]], f[..., L.FLOW["v"]], f[..., L.FLOW["w"]]], axis=-1)
    axes = (2, 1, 0)                                    # zeta ~ i, eta ~ j, xi ~ k
    grad = np.zeros(u.shape + (3,))                     # grad[..., a, b] = d u_a / d x_b
    for d in range(3):
        du = _index_derivative(u, axes[d], periodic[d])
        grad += du[..., :, None] * m[..., d, None, :]
    div = grad[..., 0, 0] + grad[..., 1, 1] + grad[..., 2, 2]
    curl2 = ((grad[..., 1, 2] - grad[..., 2, 1]) ** 2 + (grad[..., 0, 2] - grad[..., 2, 0]) ** 2
             + (grad[..., 0, 1] - grad[..., 1, 0]) ** 2)
    return ((div * div) / ((div * div) + curl2 + 10e-30)).reshape(-1)


def write_tecplot(path, case, flow: np.ndarray, iteration: int, proc: int = 0) -> pathlib.Path:
    """Tecplot ASCII of the owned rows 1..sd_node of a case on a lattice
    (case.shape = the owned box)."""
    path = pathlib.Path(path)
    g = case.arrays["grid"]
    ni, nj, nk = case.shape
    n = case.sd_node
    if ni * nj * nk != n:
        raise ValueError("write_tecplot needs a case whose owned rows form its lattice box")
    # a direction is non-periodic when the owned box ends in boundary nodes
    loc = g["loc"][1:n + 1].reshape(nk, nj, ni)
    periodic = (not (loc[:, :, 0] > 0).all(), not (loc[:, 0, :] > 0).all(), not (loc[0, :, :] > 0).all())
    duc = ducros_sensor(flow, case.arrays["metric"], case.shape, periodic)
    f = flow[1:n + 1]
    cols = [f[:, L.FLOW[k]] for k in ("u", "v", "w", "rho", "p", "t", "e", "mu")]
    with open(path, "w") as fp:
        fp.write("TITLE = Node file\n")
        fp.write("VARIABLES = X, Y, Z, U, V, W, RHO, P, T, e, mu, loc, Proc, DUCROS,\n")
        fp.write(f"ZONE I= {ni} J= {nj} K= {nk} DATAPACKING=POINT, ZONETYPE=ORDERED, SOLUTIONTIME= {iteration}\n")
        x, y, z, loc = g["x"][1:n + 1], g["y"][1:n + 1], g["z"][1:n + 1], g["loc"][1:n + 1]
        for r in range(n):
            vals = [x[r], y[r], z[r]] + [c[r] for c in cols]
            fp.write("\t".join(f"{v:.10g}" for v in vals) + f"\t{int(loc[r])}\t{proc}\t{duc[r]:.10g}\n")
    return path
