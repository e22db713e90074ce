"""Synthetic cases in the reference layout (the inputs of the RHS path).

The reference reads Gambit/ICEM meshes that are not shipped, so the cases its
benchmark configurations describe are generated here, deterministically:

* ``isentropic_vortex`` -- periodic Cartesian box [0, L)^3, inviscid
  isentropic vortex advected in x (uniform in z).
* ``taylor_green``      -- periodic [0, 2 pi)^3 with sinusoidally perturbed
  node positions x_i = xi_i + A sin(xi_j) sin(xi_k) (cyclic), analytic
  metrics, Taylor-Green vortex initial condition.
* ``shock_slab``        -- the perturbed periodic lattice of the Taylor-Green
  case with a high-pressure, high-density slab drifting along x: shocks
  from its edges (the shocked curvilinear workload's discontinuity).
* ``ghost_box``         -- a non-periodic box surrounded by three layers of
  ghost nodes (loc = 100) with boundary codes on the faces, edges and corners,
  used to exercise the one-sided stencil branches keyed on ``loc``.

Every generator fills the arrays the reference's host hands to its kernels:
GRID (neighbour table, loc codes), det, TRANSFORMED (node metrics and the
half-point metrics of Main.cpp:2369-2440), DETERM, and FLOW.  Row 0 is the
reference's dummy row; it is given a benign state whose neighbours point to
itself so that computing it (the reference's NDRange includes it) stays finite.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from . import layout as L


@dataclasses.dataclass
class Params:
    """Physical and numerical constants of the RHS path.

    The reference hard-codes mach/reynolds/prandtl/t_inf in Viscous.cl:30-33
    (1.5, 500, 0.72, 273) and weno_eps in Weno.cl:59 (10e-8); Weno takes Mach
    as an argument (Weno.cl:36).  ``viscous=0`` zeroes Fv/Ev/Gv (inviscid
    runs); ``les`` selects the SGS model: 0 none, 1 the reference's mixed
    time scale, 2 Smagorinsky with ``smagorinsky_cs`` (no counterpart in the
    reference).
    """
    mach: float = 1.5
    reynolds: float = 500.0
    prandtl: float = 0.72
    t_inf: float = 273.0
    weno_eps: float = 1e-7
    viscous: int = 1
    les: int = 1
    smagorinsky_cs: float = 0.1


@dataclasses.dataclass
class BoundaryLists:
    """Node lists of the reference's boundary routine intialise()
    (Flow_Initialisation.cpp:23-1394): row indices, visited in order,
    outlet, then inlet, boundary (mirror copy) and wall (no-slip).

    ``singular`` (rows x 6, int32) is the reference's singular-node table of
    a wake cut (functions.h ``singul``, filled in Main.cpp:1612-1700): the
    neighbours across the cut that the wall rules of ID 10 and codes 29/30,
    33..52 read.  ``tips`` are the trailing-edge rows the solver fixes after
    the routine (Solver.cpp:660-683)."""
    outlet: np.ndarray
    inlet: np.ndarray
    boundary: np.ndarray
    wall: np.ndarray
    singular: np.ndarray | None = None
    tips: np.ndarray | None = None

    def __post_init__(self):
        for k in ("outlet", "inlet", "boundary", "wall"):
            setattr(self, k, np.ascontiguousarray(getattr(self, k), dtype=np.int32))
        if self.singular is not None:
            self.singular = np.ascontiguousarray(self.singular, dtype=np.int32).reshape(-1, 6)
        if self.tips is not None:
            self.tips = np.ascontiguousarray(self.tips, dtype=np.int32)


@dataclasses.dataclass
class Case:
    name: str
    shape: tuple            # (ni, nj, nk) of owned nodes for structured cases
    periodic: bool
    sd_node: int            # owned nodes 1..sd_node
    g_node: int             # owned + ghost nodes 1..g_node
    arrays: dict            # layout.empty_arrays(g_node + 1) filled
    params: Params
    dt: float
    bc: BoundaryLists | None = None   # boundary routine lists (non-periodic cases)

    @property
    def n_rows(self) -> int:
        return self.g_node + 1

    def copy(self) -> "Case":
        return dataclasses.replace(self, arrays={k: v.copy() for k, v in self.arrays.items()},
                                   params=dataclasses.replace(self.params))


# --------------------------------------------------------------- helpers ---

def _flow_from_primitives(flow, rho, u, v, w, p, mach):
    f = L.FLOW
    flow[:, f["rho"]] = rho
    flow[:, f["u"]] = u
    flow[:, f["v"]] = v
    flow[:, f["w"]] = w
    flow[:, f["p"]] = p
    flow[:, f["t"]] = (1.4 * mach * mach) * (p / rho)
    flow[:, f["a"]] = np.sqrt(1.4 * p / rho)
    flow[:, f["e"]] = p / (0.4 * rho)
    flow[:, f["mu"]] = 0.0


def _set_dummy_row(a):
    """Row 0: neighbours to itself, unit metrics, quiescent unit state."""
    g = a["grid"][0]
    for k in ("N0", "N1", "N2", "N3", "N4", "N5", "ID", "loc"):
        g[k] = 0
    a["det"][0] = 1.0
    a["deter"][0, :] = 1.0
    m = np.zeros(63)
    for b in range(7):
        m[9 * b + 0] = m[9 * b + 4] = m[9 * b + 8] = 1.0
    a["metric"][0] = m
    a["flow"][0] = 0.0
    _flow_from_primitives(a["flow"][0:1], 1.0, 0.0, 0.0, 0.0, 1.0, 1.0)


def _periodic_index(ni, nj, nk):
    """Row number (1-based) of node (i, j, k), i fastest."""
    i, j, k = np.meshgrid(np.arange(ni), np.arange(nj), np.arange(nk), indexing="ij")
    return (1 + i + ni * (j + nj * k)), i, j, k


def _fill_periodic_grid(a, ni, nj, nk, x, y, z):
    """Wrap-around neighbour table; arrays x,y,z are (ni,nj,nk)."""
    row, i, j, k = _periodic_index(ni, nj, nk)
    rows = row.transpose(2, 1, 0).ravel()  # i fastest -> rows 1..n in order
    assert np.array_equal(rows, np.arange(1, ni * nj * nk + 1))

    def rid(ii, jj, kk):
        return (1 + (ii % ni) + ni * ((jj % nj) + nj * (kk % nk))).transpose(2, 1, 0).ravel()

    g = a["grid"][1:]
    g["x"] = x.transpose(2, 1, 0).ravel()
    g["y"] = y.transpose(2, 1, 0).ravel()
    g["z"] = z.transpose(2, 1, 0).ravel()
    g["N0"] = rid(i, j + 1, k)
    g["N1"] = rid(i + 1, j, k)
    g["N2"] = rid(i, j - 1, k)
    g["N3"] = rid(i - 1, j, k)
    g["N4"] = rid(i, j, k + 1)
    g["N5"] = rid(i, j, k - 1)
    g["ID"] = rows
    g["loc"] = 0


def _node_metrics(jac):
    """jac[..., a, b] = d x_a / d zeta_b (index coordinates).  Returns the
    9 node metrics (zeta_x, zeta_y, zeta_z, eta_x, ..., xi_z) = the inverse
    Jacobian (cofactors / det, as Grid_Transformation.cpp:1029-1037 forms
    them) and det."""
    J = jac
    c00 = J[..., 1, 1] * J[..., 2, 2] - J[..., 1, 2] * J[..., 2, 1]
    c01 = J[..., 1, 2] * J[..., 2, 0] - J[..., 1, 0] * J[..., 2, 2]
    c02 = J[..., 1, 0] * J[..., 2, 1] - J[..., 1, 1] * J[..., 2, 0]
    det = J[..., 0, 0] * c00 + J[..., 0, 1] * c01 + J[..., 0, 2] * c02
    inv = np.empty(J.shape)
    inv[..., 0, 0] = c00
    inv[..., 1, 0] = c01
    inv[..., 2, 0] = c02
    inv[..., 0, 1] = J[..., 0, 2] * J[..., 2, 1] - J[..., 0, 1] * J[..., 2, 2]
    inv[..., 1, 1] = J[..., 0, 0] * J[..., 2, 2] - J[..., 0, 2] * J[..., 2, 0]
    inv[..., 2, 1] = J[..., 0, 1] * J[..., 2, 0] - J[..., 0, 0] * J[..., 2, 1]
    inv[..., 0, 2] = J[..., 0, 1] * J[..., 1, 2] - J[..., 0, 2] * J[..., 1, 1]
    inv[..., 1, 2] = J[..., 0, 2] * J[..., 1, 0] - J[..., 0, 0] * J[..., 1, 2]
    inv[..., 2, 2] = J[..., 0, 0] * J[..., 1, 1] - J[..., 0, 1] * J[..., 1, 0]
    inv /= det[..., None, None]       # inv[..., b, a] = d zeta_b / d x_a
    m9 = inv.reshape(inv.shape[:-2] + (9,))
    return m9, det


def _lattice_half_points(a, m9_kji, det_kji):
    """Half-point metrics and face determinants of a periodic lattice from
    node values held in row order as [k, j, i, ...] arrays: the six-point
    midpoint rule (3, -25, 150, 150, -25, 3)/256 of Main.cpp:2369-2440 with
    the same operand order as half_point_metrics, evaluated on wrap-padded
    slices instead of neighbour chains."""
    nk, nj, ni = det_kji.shape
    for d in range(3):
        axis = 2 - d                      # i -> axis 2, j -> axis 1, k -> axis 0
        n = det_kji.shape[axis]
        for src, dst_cols in ((m9_kji, None), (det_kji, None)):
            pad = [(0, 0)] * src.ndim
            pad[axis] = (3, 3)
            v = np.pad(src, pad, mode="wrap")

            def sl(o):
                idx = [slice(None)] * src.ndim
                idx[axis] = slice(3 + o, 3 + o + n)
                return v[tuple(idx)]
            for side in (0, 1):            # +1/2 face uses offsets -2..3, -1/2 face -3..2
                o0 = -2 - side
                # ((((3 f0 - 25 f1) + 150 f2) + 150 f3) - 25 f4) + 3 f5, then x 1/256,
                # accumulated in place (same order and rounding as the expression)
                out = np.multiply(sl(o0), 3.0)
                tmp = np.empty_like(out)
                for o, cst, sub in ((1, 25.0, True), (2, 150.0, False), (3, 150.0, False), (4, 25.0, True),
                                    (5, 3.0, False)):
                    np.multiply(sl(o0 + o), cst, out=tmp)
                    (np.subtract if sub else np.add)(out, tmp, out=out)
                out *= (1.0 / 256.0)
                if src is m9_kji:
                    b = 1 + 2 * d + side
                    a["metric"][1:, 9 * b:9 * b + 9] = out.reshape(-1, 9)
                else:
                    a["deter"][1:, 2 * d + side] = out.ravel()


def half_point_metrics(a, n_rows_owned: int):
    """Face metrics and face determinants by the six-point midpoint rule
    (3, -25, 150, 150, -25, 3)/256 of node values along each direction,
    Main.cpp:2369-2440, for rows 1..n_rows_owned.  Uses the neighbour table,
    so it works for any layout whose neighbours of owned nodes exist."""
    g = a["grid"]
    rows = np.arange(1, n_rows_owned + 1)
    node_m = a["metric"][:, 0:9]
    det = a["det"]
    plus = [g[n] for n in L.PLUS]
    minus = [g[n] for n in L.MINUS]
    for d in range(3):
        P, M = plus[d], minus[d]
        im1 = M[rows]
        im2 = M[im1]
        im3 = M[im2]
        ip1 = P[rows]
        ip2 = P[ip1]
        ip3 = P[ip2]

        def interp(v, s0, s1, s2, s3, s4, s5):
            return (1.0 / 256.0) * (3.0 * (v[s0]) - 25.0 * (v[s1]) + 150.0 * (v[s2]) + 150.0 * (v[s3])
                                    - 25.0 * (v[s4]) + 3.0 * (v[s5]))

        bp = 1 + 2 * d
        bm = 2 + 2 * d
        a["metric"][rows, 9 * bp:9 * bp + 9] = interp(node_m, im2, im1, rows, ip1, ip2, ip3)
        a["metric"][rows, 9 * bm:9 * bm + 9] = interp(node_m, im3, im2, im1, rows, ip1, ip2)
        a["deter"][rows, 2 * d] = interp(det, im2, im1, rows, ip1, ip2, ip3)
        a["deter"][rows, 2 * d + 1] = interp(det, im3, im2, im1, rows, ip1, ip2)


def cfl_dt(a, rows, cfl: float) -> float:
    """Builder-defined time step: cfl / max over nodes and directions of
    |U . grad zeta_d| + c |grad zeta_d| (unit computational spacing).  The
    reference itself uses a fixed del_t (Main.cpp:47)."""
    f = a["flow"][rows]
    m = a["metric"][rows, 0:9].reshape(-1, 3, 3)
    u = f[:, [L.FLOW["u"], L.FLOW["v"], L.FLOW["w"]]]
    c = np.sqrt(1.4 * f[:, L.FLOW["p"]] / f[:, L.FLOW["rho"]])
    un = np.abs(np.einsum("nda,na->nd", m, u))
    gn = np.linalg.norm(m, axis=2)
    lam = (un + c[:, None] * gn).max()
    return float(cfl / lam)


# ------------------------------------------------------------- generators --

def isentropic_vortex(n=64, length=10.0, beta=5.0, u_inf=0.5, center=(5.0, 5.0),
                      weno_eps=1e-7, cfl=0.5, shape=None) -> Case:
    """Inviscid isentropic vortex on a periodic Cartesian grid.

    Nodes x_i = i*D, D = length/n, identity-direction metrics zeta_x = eta_y =
    xi_z = 1/D in all seven metric blocks and det = D^3 (the reference's flux
    difference has unit computational spacing, Weno.cl:3060-3082).  gamma=1.4,
    rho_inf = p_inf = 1, vortex of strength beta centred at ``center`` in x-y,
    uniform in z.  ``viscous=0``: Fv, Ev, Gv are zeroed.
    """
    ni, nj, nk = shape if shape is not None else (n, n, n)
    D = length / ni
    a = L.empty_arrays(ni * nj * nk + 1)
    _set_dummy_row(a)
    xs = np.arange(ni) * D
    ys = np.arange(nj) * (length / nj)
    zs = np.arange(nk) * (length / nk)
    X, Y, Z = np.meshgrid(xs, ys, zs, indexing="ij")
    _fill_periodic_grid(a, ni, nj, nk, X, Y, Z)
    Dy, Dz = length / nj, length / nk
    m = np.zeros(63)
    for b in range(7):
        m[9 * b + 0] = 1.0 / D
        m[9 * b + 4] = 1.0 / Dy
        m[9 * b + 8] = 1.0 / Dz
    a["metric"][1:] = m
    a["det"][1:] = D * Dy * Dz
    a["deter"][1:] = D * Dy * Dz

    gam = 1.4
    xr = a["grid"]["x"][1:] - center[0]
    yr = a["grid"]["y"][1:] - center[1]
    r2 = xr * xr + yr * yr
    ex = np.exp(0.5 * (1.0 - r2))
    du = -beta / (2 * math.pi) * ex * yr
    dv = beta / (2 * math.pi) * ex * xr
    T = 1.0 - (gam - 1.0) * beta * beta / (8.0 * gam * math.pi ** 2) * np.exp(1.0 - r2)
    rho = T ** (1.0 / (gam - 1.0))
    p = rho ** gam
    mach = u_inf / math.sqrt(gam)
    _flow_from_primitives(a["flow"][1:], rho, u_inf + du, dv, np.zeros_like(rho), p, mach)
    rows = np.arange(1, ni * nj * nk + 1)
    prm = Params(mach=mach, weno_eps=weno_eps, viscous=0, les=0)
    return Case("isentropic_vortex", (ni, nj, nk), True, ni * nj * nk, ni * nj * nk, a, prm,
                cfl_dt(a, rows, cfl))


def _perturbed_periodic_box(ni, nj, nk, amp):
    """Reference arrays of a periodic [0, 2 pi)^3 lattice with perturbed nodes
    x = xi1 + A sin xi2 sin xi3, y = xi2 + A sin xi3 sin xi1,
    z = xi3 + A sin xi1 sin xi2: the neighbour table, node metrics and det
    from the analytic Jacobian (index coordinates, spacing h = 2 pi / n per
    direction), face metrics and face determinants by the reference's
    six-point midpoint rule.  Returns the arrays and the node coordinates
    (flattened in row order)."""
    hs = (2 * math.pi / ni, 2 * math.pi / nj, 2 * math.pi / nk)
    # arrays in row order [k, j, i] (i fastest)
    x3, x2, x1 = np.meshgrid(np.arange(nk) * hs[2], np.arange(nj) * hs[1], np.arange(ni) * hs[0], indexing="ij")
    A = amp
    s1, c1, s2, c2, s3, c3 = np.sin(x1), np.cos(x1), np.sin(x2), np.cos(x2), np.sin(x3), np.cos(x3)
    X = x1 + A * s2 * s3
    Y = x2 + A * s3 * s1
    Z = x3 + A * s1 * s2
    a = L.empty_arrays(ni * nj * nk + 1)
    _set_dummy_row(a)
    _fill_periodic_grid(a, ni, nj, nk, X.transpose(2, 1, 0), Y.transpose(2, 1, 0), Z.transpose(2, 1, 0))
    jac = np.empty(x1.shape + (3, 3))
    jac[..., 0, 0] = 1.0
    jac[..., 0, 1] = A * c2 * s3
    jac[..., 0, 2] = A * s2 * c3
    jac[..., 1, 0] = A * s3 * c1
    jac[..., 1, 1] = 1.0
    jac[..., 1, 2] = A * c3 * s1
    jac[..., 2, 0] = A * c1 * s2
    jac[..., 2, 1] = A * s1 * c2
    jac[..., 2, 2] = 1.0
    jac *= np.array(hs)[None, None, None, None, :]
    m9, det = _node_metrics(jac)
    del jac
    a["metric"][1:, 0:9] = m9.reshape(-1, 9)
    a["det"][1:] = det.ravel()
    _lattice_half_points(a, m9, det)
    return a, X.ravel(), Y.ravel(), Z.ravel()


def taylor_green(n=128, amp=0.05, mach=0.1, reynolds=1600.0, prandtl=0.72, t_inf=273.0,
                 weno_eps=1e-7, cfl=0.5, les=1, shape=None) -> Case:
    """Taylor-Green vortex on the perturbed periodic [0, 2 pi)^3 lattice
    (_perturbed_periodic_box).  Initial state u = sin x cos y cos z,
    v = -cos x sin y cos z, w = 0, rho = 1,
    p = 1/(gamma M^2) + (cos 2x + cos 2y)(cos 2z + 2)/16."""
    ni, nj, nk = shape if shape is not None else (n, n, n)
    a, xx, yy, zz = _perturbed_periodic_box(ni, nj, nk, amp)
    gam = 1.4
    u = np.sin(xx) * np.cos(yy) * np.cos(zz)
    v = -np.cos(xx) * np.sin(yy) * np.cos(zz)
    w = np.zeros_like(u)
    rho = np.ones_like(u)
    p = 1.0 / (gam * mach * mach) + (np.cos(2 * xx) + np.cos(2 * yy)) * (np.cos(2 * zz) + 2.0) / 16.0
    _flow_from_primitives(a["flow"][1:], rho, u, v, w, p, mach)
    rows = np.arange(1, ni * nj * nk + 1)
    prm = Params(mach=mach, reynolds=reynolds, prandtl=prandtl, t_inf=t_inf, weno_eps=weno_eps,
                 viscous=1, les=les)
    return Case("taylor_green", (ni, nj, nk), True, ni * nj * nk, ni * nj * nk, a, prm,
                cfl_dt(a, rows, cfl))


def shock_slab(shape=(256, 64, 64), amp=0.05, mach=0.8, reynolds=5e5, prandtl=0.72, t_inf=273.0,
               p_ratio=10.0, rho_ratio=4.0, drift=1.5, weno_eps=1e-7, cfl=0.5, les=1) -> Case:
    """A shocked flow on the perturbed periodic lattice (_perturbed_periodic_box,
    the same curvilinear geometry as the Taylor-Green case): the slab
    pi/2 <= x < 3 pi/2 starts at p_ratio times the free-stream pressure
    1/(gamma M^2) and rho_ratio times its density (rho = 1 outside), with
    discontinuous edges; every node moves with u = drift x the free-stream
    sound speed 1/M along x.  Each slab edge is a Riemann problem: shocks and
    contacts run out from both edges from the first step.  The drift keeps
    u > 0 throughout, so the contravariant velocity along i is positive and
    the reference's LLF speed (lambda_5 = U.grad(zeta) + c|grad(zeta)| only,
    Weno.cl:2859-2911) bounds the wave speeds there.  Viscous with the MTS
    LES model at the NACA0012 workload's Mach and Reynolds numbers."""
    ni, nj, nk = shape
    a, xx, yy, zz = _perturbed_periodic_box(ni, nj, nk, amp)
    gam = 1.4
    p_inf = 1.0 / (gam * mach * mach)
    inside = (xx >= 0.5 * math.pi) & (xx < 1.5 * math.pi)
    rho = np.where(inside, rho_ratio, 1.0)
    p = np.where(inside, p_ratio * p_inf, p_inf)
    u = np.full_like(rho, drift / mach)
    z0 = np.zeros_like(rho)
    _flow_from_primitives(a["flow"][1:], rho, u, z0, z0, p, mach)
    rows = np.arange(1, ni * nj * nk + 1)
    prm = Params(mach=mach, reynolds=reynolds, prandtl=prandtl, t_inf=t_inf, weno_eps=weno_eps,
                 viscous=1, les=les)
    return Case("shock_slab", (ni, nj, nk), True, ni * nj * nk, ni * nj * nk, a, prm, cfl_dt(a, rows, cfl))


# Boundary codes of owned nodes by the box faces they lie on, in the
# reference's convention: a face code names the missing neighbour
# (Flow_Initialisation.cpp:55-89: 1 no +j, 2 no +i, 3 no -j, 4 no -i,
# 5 no -k, 6 no +k); edge and corner codes are those whose copy chains
# (:139-340) step from the node into the interior.
_EDGE_CODES = {("jmin", "kmax"): 15, ("imin", "jmin"): 16, ("jmin", "kmin"): 17, ("imax", "jmin"): 18,
               ("jmax", "kmax"): 19, ("imin", "jmax"): 20, ("jmax", "kmin"): 21, ("imax", "jmax"): 22,
               ("imin", "kmax"): 23, ("imin", "kmin"): 24, ("imax", "kmin"): 25, ("imax", "kmax"): 26}
_CORNER_CODES = {("imin", "jmax", "kmax"): 7, ("imin", "jmax", "kmin"): 8, ("imax", "jmax", "kmin"): 9,
                 ("imax", "jmax", "kmax"): 10, ("imin", "jmin", "kmax"): 11, ("imin", "jmin", "kmin"): 12,
                 ("imax", "jmin", "kmin"): 13, ("imax", "jmin", "kmax"): 14}
_FACE_CODES = {"jmax": 1, "imax": 2, "jmin": 3, "imin": 4, "kmin": 5, "kmax": 6}


def reference_loc_codes(imin, imax, jmin, jmax, kmin, kmax) -> np.ndarray:
    """loc of nodes from boolean masks of the six box faces (0 = interior)."""
    flags = {"imin": imin, "imax": imax, "jmin": jmin, "jmax": jmax, "kmin": kmin, "kmax": kmax}
    loc = np.zeros(np.shape(imin), dtype=np.int64)
    count = sum(np.asarray(f, dtype=int) for f in flags.values())
    for name, code in _FACE_CODES.items():
        loc = np.where((count == 1) & flags[name], code, loc)
    for names, code in _EDGE_CODES.items():
        m = (count == 2) & np.logical_and.reduce([flags[n] for n in names])
        loc = np.where(m, code, loc)
    for names, code in _CORNER_CODES.items():
        m = (count == 3) & np.logical_and.reduce([flags[n] for n in names])
        loc = np.where(m, code, loc)
    return loc


def box_mesh(shape=(12, 10, 8), amp=0.04, lengths=(1.0, 0.8, 0.6)):
    """A curvilinear box as the reference's mesh tools hand it to its
    geometry routines: rows 1..N in lattice order (i fastest), neighbour 0
    where the box ends, the reference's loc codes on its faces, edges and
    corners, ID 0.  Nodes x = L1 (s1 + A sin(pi s2) sin(pi s3)), y and z
    alike (cyclic), s_d = index / (n_d - 1).  Returns the GRID array and the
    analytic node metrics [N, 9] and det [N] (index coordinates)."""
    ni, nj, nk = shape
    k, j, i = np.meshgrid(np.arange(nk), np.arange(nj), np.arange(ni), indexing="ij")
    s1, s2, s3 = i / (ni - 1), j / (nj - 1), k / (nk - 1)
    A, pi = amp, math.pi
    L1, L2, L3 = lengths
    X = L1 * (s1 + A * np.sin(pi * s2) * np.sin(pi * s3))
    Y = L2 * (s2 + A * np.sin(pi * s3) * np.sin(pi * s1))
    Z = L3 * (s3 + A * np.sin(pi * s1) * np.sin(pi * s2))
    N = ni * nj * nk
    g = np.zeros(N + 1, L.GRID_DTYPE)
    g["x"][1:], g["y"][1:], g["z"][1:] = X.ravel(), Y.ravel(), Z.ravel()
    row = (i + ni * (j + nj * k)) + 1

    def nb(di, dj, dk):
        ii, jj, kk = i + di, j + dj, k + dk
        inside = (ii >= 0) & (ii < ni) & (jj >= 0) & (jj < nj) & (kk >= 0) & (kk < nk)
        return np.where(inside, (ii + ni * (jj + nj * kk)) + 1, 0).ravel()

    g["N0"][1:], g["N1"][1:], g["N2"][1:] = nb(0, 1, 0), nb(1, 0, 0), nb(0, -1, 0)
    g["N3"][1:], g["N4"][1:], g["N5"][1:] = nb(-1, 0, 0), nb(0, 0, 1), nb(0, 0, -1)
    g["ID"][1:] = 0
    g["loc"][1:] = reference_loc_codes(i == 0, i == ni - 1, j == 0, j == nj - 1, k == 0, k == nk - 1).ravel()
    assert (row.ravel() == np.arange(1, N + 1)).all()
    # analytic Jacobian d(x, y, z)/d(i, j, k)
    c1, c2, c3 = np.cos(pi * s1), np.cos(pi * s2), np.cos(pi * s3)
    n1, n2, n3 = np.sin(pi * s1), np.sin(pi * s2), np.sin(pi * s3)
    h = (1.0 / (ni - 1), 1.0 / (nj - 1), 1.0 / (nk - 1))
    jac = np.empty(X.shape + (3, 3))
    jac[..., 0, 0] = L1 * h[0]
    jac[..., 0, 1] = L1 * A * pi * c2 * n3 * h[1]
    jac[..., 0, 2] = L1 * A * pi * n2 * c3 * h[2]
    jac[..., 1, 0] = L2 * A * pi * n3 * c1 * h[0]
    jac[..., 1, 1] = L2 * h[1]
    jac[..., 1, 2] = L2 * A * pi * c3 * n1 * h[2]
    jac[..., 2, 0] = L3 * A * pi * c1 * n2 * h[0]
    jac[..., 2, 1] = L3 * A * pi * n1 * c2 * h[1]
    jac[..., 2, 2] = L3 * h[2]
    m9, det = _node_metrics(jac)
    return g, m9.reshape(-1, 9), det.ravel()


def ghost_box(shape=(10, 9, 8), seed=0, mach=1.5, amp=0.05, bc: bool = False) -> Case:
    """Non-periodic box of owned nodes with three ghost layers on every side.

    Owned nodes carry ``loc`` = 0 in the interior and a code in 1..26 on the
    boundary (faces, edges, corners), ghosts carry 100, as in
    node_locations.cpp and Main.cpp:1426-2300.  Ghost neighbour chains that
    would leave the padded box point back to the ghost itself.  The flow is
    a smooth perturbation of a uniform state (seeded), the geometry a mildly
    perturbed Cartesian grid with analytic metrics."""
    ni, nj, nk = shape
    G = 3
    pi_, pj, pk = ni + 2 * G, nj + 2 * G, nk + 2 * G
    ii, jj, kk = np.meshgrid(np.arange(pi_), np.arange(pj), np.arange(pk), indexing="ij")
    owned = (ii >= G) & (ii < G + ni) & (jj >= G) & (jj < G + nj) & (kk >= G) & (kk < G + nk)
    n_owned = int(owned.sum())
    n_all = pi_ * pj * pk
    # row numbers: owned first (i fastest), then ghosts
    order = np.zeros((pi_, pj, pk), dtype=np.int64)
    own_idx = np.argwhere(owned.transpose(2, 1, 0))[:, ::-1]  # (i,j,k) with i fastest
    order[own_idx[:, 0], own_idx[:, 1], own_idx[:, 2]] = np.arange(1, n_owned + 1)
    gh_idx = np.argwhere((~owned).transpose(2, 1, 0))[:, ::-1]
    order[gh_idx[:, 0], gh_idx[:, 1], gh_idx[:, 2]] = np.arange(n_owned + 1, n_all + 1)

    a = L.empty_arrays(n_all + 1)
    _set_dummy_row(a)
    h = 1.0 / max(ni, nj, nk)
    x1, x2, x3 = ii * h, jj * h, kk * h
    A = amp * h * 4
    X = x1 + A * np.sin(7 * x2) * np.sin(5 * x3)
    Y = x2 + A * np.sin(6 * x3) * np.sin(5 * x1)
    Z = x3 + A * np.sin(5 * x1) * np.sin(6 * x2)

    def nb(di, dj, dk):
        ti, tj, tk = ii + di, jj + dj, kk + dk
        inside = (ti >= 0) & (ti < pi_) & (tj >= 0) & (tj < pj) & (tk >= 0) & (tk < pk)
        ti = np.where(inside, ti, ii)
        tj = np.where(inside, tj, jj)
        tk = np.where(inside, tk, kk)
        return order[ti, tj, tk]

    def put(field, vals):
        a["grid"][field][order.ravel()] = vals.ravel()

    put("x", X)
    put("y", Y)
    put("z", Z)
    put("N0", nb(0, 1, 0))
    put("N1", nb(1, 0, 0))
    put("N2", nb(0, -1, 0))
    put("N3", nb(-1, 0, 0))
    put("N4", nb(0, 0, 1))
    put("N5", nb(0, 0, -1))
    put("ID", order)
    loc = reference_loc_codes(ii == G, ii == G + ni - 1, jj == G, jj == G + nj - 1, kk == G, kk == G + nk - 1)
    loc = np.where(owned, loc, 100)
    put("loc", loc)

    jac = np.zeros(ii.shape + (3, 3))
    jac[..., 0, 0] = h
    jac[..., 0, 1] = A * 7 * h * np.cos(7 * x2) * np.sin(5 * x3)
    jac[..., 0, 2] = A * 5 * h * np.sin(7 * x2) * np.cos(5 * x3)
    jac[..., 1, 0] = A * 5 * h * np.sin(6 * x3) * np.cos(5 * x1)
    jac[..., 1, 1] = h
    jac[..., 1, 2] = A * 6 * h * np.cos(6 * x3) * np.sin(5 * x1)
    jac[..., 2, 0] = A * 5 * h * np.cos(5 * x1) * np.sin(6 * x2)
    jac[..., 2, 1] = A * 6 * h * np.sin(5 * x1) * np.cos(6 * x2)
    jac[..., 2, 2] = h
    m9, det = _node_metrics(jac)
    a["metric"][order.ravel(), 0:9] = m9.reshape(-1, 9)
    a["det"][order.ravel()] = det.ravel()
    # ghosts carry their own node metrics in every half-point block
    for b in range(1, 7):
        a["metric"][1:, 9 * b:9 * b + 9] = a["metric"][1:, 0:9]
    a["deter"][1:, :] = a["det"][1:, None]
    half_point_metrics(a, n_owned)

    rng = np.random.default_rng(seed)
    ph = rng.uniform(0, 2 * math.pi, size=6)
    rho = 1.0 + 0.1 * np.sin(2 * math.pi * x1 + ph[0]) * np.cos(2 * math.pi * x2 + ph[1])
    u = 0.6 + 0.1 * np.sin(2 * math.pi * x2 + ph[2])
    v = 0.1 * np.cos(2 * math.pi * x3 + ph[3])
    w = 0.05 * np.sin(2 * math.pi * x1 + ph[4])
    p = 1.0 / (1.4 * mach * mach) * (1.0 + 0.05 * np.cos(2 * math.pi * (x1 + x2 + x3) + ph[5]))
    flow = np.zeros((n_all, 9))
    _flow_from_primitives(flow, rho.ravel(), u.ravel(), v.ravel(), w.ravel(), p.ravel(), mach)
    a["flow"][order.ravel()] = flow
    rows = np.arange(1, n_owned + 1)
    prm = Params(mach=mach)
    c = Case("ghost_box", (ni, nj, nk), False, n_owned, n_all, a, prm, cfl_dt(a, rows, 0.3))
    if bc:
        # ID 10 marks the reference's singular wall nodes; the box has none
        a["grid"]["ID"][:] = 0
        c.bc = box_boundary_lists(a["grid"]["loc"], n_owned)
    return c


# Codes of the reference's singular wall branches: 29/30 (a node beyond
# the cut), 33..52 (the multi-pass corner codes; Flow_Initialisation.cpp
# :1276-1392).  53..56 are left out: the routine never sets their slots.
SINGULAR_CODES = (29, 30) + tuple(range(33, 53))


def with_singular_nodes(c: Case, seed: int = 0, n_tips: int = 4, face_code: int | None = None) -> Case:
    """Relabels wall nodes of ``c`` (a case with boundary lists) as the
    reference's singular wall nodes, in place: rows of one wall face code
    (the most common one unless given) take every singular code of the
    routine, some with ID 10 (over the face code and over codes 33..52),
    plus a wall edge or corner with ID 10 where the case has one; a
    singular-node table whose slots name seeded owned rows (in a C-grid they
    are the nodes across the wake cut; here any owned row exercises the same
    index chains); and ``n_tips`` tip rows.  Every loc code stays in 1..52,
    so the kernels' boundary branches treat the relabelled nodes as the face
    nodes they were."""
    g = c.arrays["grid"]
    rng = np.random.default_rng(seed + 17)
    wall = np.asarray(c.bc.wall)
    codes = g["loc"][wall]
    if face_code is None:
        faces = codes[(codes >= 1) & (codes <= 6)]
        face_code = int(np.bincount(faces).argmax())
    rows = wall[codes == face_code]
    edges = wall[(codes >= 7) & (codes <= 26)]
    need = len(SINGULAR_CODES) + 6
    if rows.size < need:
        raise ValueError(f"{rows.size} wall rows with code {face_code}; the relabelling needs {need}")
    chosen = rows[rng.choice(rows.size, size=need, replace=False)]
    g["ID"][wall] = 0
    for r, code in zip(chosen, SINGULAR_CODES):
        g["loc"][r] = code
    marked = list(chosen[2:8]) + list(chosen[len(SINGULAR_CODES):])   # over 33..52 and over the face code
    if edges.size:
        marked.append(edges[0])
    g["ID"][marked] = 10
    owned = np.arange(1, c.sd_node + 1)
    sing = np.zeros((c.g_node + 1, 6), dtype=np.int32)
    for r in list(chosen) + marked:
        sing[r] = rng.choice(owned, size=6)
    tips = rng.choice(owned, size=n_tips, replace=False).astype(np.int32)
    c.bc = BoundaryLists(c.bc.outlet, c.bc.inlet, c.bc.boundary, c.bc.wall, singular=sing, tips=tips)
    return c


def singular_box(shape=(10, 9, 8), seed=0, mach=1.5, n_tips: int = 4) -> Case:
    """ghost_box(bc=True) with singular wall nodes on its south (-j) wall
    (with_singular_nodes)."""
    c = with_singular_nodes(ghost_box(shape=shape, seed=seed, mach=mach, bc=True), seed, n_tips, face_code=3)
    c.name = "singular_box"
    return c


# Boundary type of each box face for ghost_box(bc=True): every type of the
# boundary routine appears, edges and corners included.
_BOX_FACE_TYPE = {4: "inlet", 2: "outlet", 3: "wall", 1: "boundary", 5: "wall", 6: "outlet"}
_TYPES = ("outlet", "inlet", "boundary", "wall")


def box_boundary_lists(loc: np.ndarray, sd_node: int) -> BoundaryLists:
    """Lists of the owned boundary rows 1..sd_node by their loc code: face
    codes by _BOX_FACE_TYPE, edge and corner codes 7..26 round-robin over
    the four types."""
    lists = {t: [] for t in _TYPES}
    for r in range(1, sd_node + 1):
        code = int(loc[r])
        if 1 <= code <= 6:
            lists[_BOX_FACE_TYPE[code]].append(r)
        elif 7 <= code <= 26:
            lists[_TYPES[code % 4]].append(r)
    return BoundaryLists(**{t: np.array(v) for t, v in lists.items()})


# ------------------------------------------------- ghosted lattices ---

GHOSTS = 3   # ghost layers beyond the owned nodes of a non-periodic direction


def _index_derivative(X: np.ndarray, axis: int, periodic: bool, period: float = 0.0) -> np.ndarray:
    """d X / d (index) along `axis`, 4th order: central (wrapped when
    periodic, X(c + n) = X(c) + period), one-sided at the two outermost
    layers of a non-periodic direction."""
    n = X.shape[axis]
    if periodic:
        c = np.arange(n).reshape([-1 if a == axis else 1 for a in range(X.ndim)])

        def r(s):   # X[c + s] continued across the wrap
            return np.roll(X, -s, axis=axis) + period * np.floor_divide(c + s, n)
        return (r(-2) - 8.0 * r(-1) + 8.0 * r(1) - r(2)) / 12.0
    Xt = np.moveaxis(X, axis, 0)
    D = np.empty_like(Xt)
    D[2:n - 2] = (Xt[0:n - 4] - 8.0 * Xt[1:n - 3] + 8.0 * Xt[3:n - 1] - Xt[4:n]) / 12.0
    D[0] = (-25.0 * Xt[0] + 48.0 * Xt[1] - 36.0 * Xt[2] + 16.0 * Xt[3] - 3.0 * Xt[4]) / 12.0
    D[1] = (-3.0 * Xt[0] - 10.0 * Xt[1] + 18.0 * Xt[2] - 6.0 * Xt[3] + Xt[4]) / 12.0
    D[n - 1] = -(-25.0 * Xt[n - 1] + 48.0 * Xt[n - 2] - 36.0 * Xt[n - 3] + 16.0 * Xt[n - 4] - 3.0 * Xt[n - 5]) / 12.0
    D[n - 2] = -(-3.0 * Xt[n - 1] - 10.0 * Xt[n - 2] + 18.0 * Xt[n - 3] - 6.0 * Xt[n - 4] + Xt[n - 5]) / 12.0
    return np.moveaxis(D, 0, axis)


def _mirror_pad(A: np.ndarray, axis: int, G: int, point: bool) -> np.ndarray:
    """A padded by G layers on both ends of `axis`: the mirror image about
    the end layer (point=True: point reflection 2 A[0] - A[m], for
    coordinates; else the even copy A[m])."""
    At = np.moveaxis(A, axis, 0)
    lo = At[1:G + 1][::-1]
    hi = At[-G - 1:-1][::-1]
    if point:
        lo = 2.0 * At[0] - lo
        hi = 2.0 * At[-1] - hi
    return np.moveaxis(np.concatenate([lo, At, hi], axis=0), 0, axis)


def ghosted_lattice(name: str, X, Y, Z, periodic, prims, params: Params, mach: float, bc_type=None,
                    cfl: float = 0.5, periods=None) -> Case:
    """A case on an (i, j, k) lattice of owned nodes whose non-periodic
    directions get GHOSTS ghost layers on each side, in the reference layout.

    X, Y, Z: coordinates of the owned nodes [i, j, k]; periodic: three
    flags; periods[d]: the (x, y, z) shift across one period of direction d;
    prims: (rho, u, v, w, p) over the owned nodes; bc_type(i, j, k, loc) ->
    "outlet" | "inlet" | "boundary" | "wall" | None classifies each owned
    boundary node (indices of the padded lattice) into the boundary
    routine's lists.  Rows: owned nodes first (i fastest), then ghosts, as
    the reference numbers them; the outermost ghosts of a non-periodic
    direction point at themselves.  Node metrics come from 4th-order index
    derivatives over the owned nodes; ghosts carry the mirror image of the
    owned metrics and state about the boundary node (their coordinates are
    the point reflection); half-point metrics follow by the six-point rule
    on every row, so the faces of the owned nodes are single-valued."""
    G = GHOSTS
    periods = periods or ((0.0, 0.0, 0.0),) * 3
    jac = np.empty(X.shape + (3, 3))
    for axis in range(3):
        for comp, V in enumerate((X, Y, Z)):
            jac[..., comp, axis] = _index_derivative(V, axis, periodic[axis], periods[axis][comp])
    m9, det = _node_metrics(jac)
    if not np.all(det > 0):
        raise ValueError(f"{name}: the mapping folds (det <= 0 at {int((det <= 0).sum())} nodes)")
    fields = [np.broadcast_to(q, X.shape).astype(np.float64) for q in prims]
    for d in range(3):
        if periodic[d]:
            continue
        X, Y, Z = (_mirror_pad(V, d, G, True) for V in (X, Y, Z))
        m9 = _mirror_pad(m9, d, G, False)
        det = _mirror_pad(det, d, G, False)
        fields = [_mirror_pad(q, d, G, False) for q in fields]
    pi_, pj, pk = X.shape
    ext = (pi_, pj, pk)
    ii, jj, kk = np.meshgrid(np.arange(pi_), np.arange(pj), np.arange(pk), indexing="ij")
    cc = (ii, jj, kk)
    owned = np.ones(X.shape, dtype=bool)
    for d in range(3):
        if not periodic[d]:
            owned &= (cc[d] >= G) & (cc[d] < ext[d] - G)
    n_owned = int(owned.sum())
    n_all = pi_ * pj * pk
    order = np.zeros(X.shape, dtype=np.int64)
    own_idx = np.argwhere(owned.transpose(2, 1, 0))[:, ::-1]
    order[own_idx[:, 0], own_idx[:, 1], own_idx[:, 2]] = np.arange(1, n_owned + 1)
    gh_idx = np.argwhere((~owned).transpose(2, 1, 0))[:, ::-1]
    order[gh_idx[:, 0], gh_idx[:, 1], gh_idx[:, 2]] = np.arange(n_owned + 1, n_all + 1)

    a = L.empty_arrays(n_all + 1)
    _set_dummy_row(a)

    def nb(d, o):
        t = [ii, jj, kk]
        c = cc[d] + o
        t[d] = c % ext[d] if periodic[d] else np.clip(c, 0, ext[d] - 1)
        return order[t[0], t[1], t[2]]

    def put(field, vals):
        a["grid"][field][order.ravel()] = np.asarray(vals).ravel()

    put("x", X)
    put("y", Y)
    put("z", Z)
    put("N1", nb(0, 1))
    put("N3", nb(0, -1))
    put("N0", nb(1, 1))
    put("N2", nb(1, -1))
    put("N4", nb(2, 1))
    put("N5", nb(2, -1))
    put("ID", np.zeros(X.shape, dtype=np.int64))
    lo = [(cc[d] == G) & (not periodic[d]) for d in range(3)]
    hi = [(cc[d] == ext[d] - G - 1) & (not periodic[d]) for d in range(3)]
    loc = reference_loc_codes(lo[0], hi[0], lo[1], hi[1], lo[2], hi[2])
    loc = np.where(owned, loc, 100)
    put("loc", loc)
    a["metric"][order.ravel(), 0:9] = m9.reshape(-1, 9)
    a["det"][order.ravel()] = det.ravel()
    half_point_metrics(a, n_all)

    rho, u, v, w, p = fields
    flow = np.zeros((n_all, 9))
    _flow_from_primitives(flow, rho.ravel(), u.ravel(), v.ravel(), w.ravel(), p.ravel(), mach)
    a["flow"][order.ravel()] = flow
    rows = np.arange(1, n_owned + 1)
    shape = tuple(ext[d] if periodic[d] else ext[d] - 2 * G for d in range(3))
    c = Case(name, shape, False, n_owned, n_all, a, params, cfl_dt(a, rows, cfl))
    if bc_type is not None:
        lists = {t: [] for t in _TYPES}
        bidx = np.argwhere(owned & (loc > 0))
        rws = order[bidx[:, 0], bidx[:, 1], bidx[:, 2]]
        for (i, j, k), r in sorted(zip(map(tuple, bidx), rws), key=lambda t: t[1]):
            t = bc_type(int(i), int(j), int(k), int(loc[i, j, k]))
            if t is not None:
                lists[t].append(int(r))
        c.bc = BoundaryLists(**{t: np.array(v, dtype=np.int32) for t, v in lists.items()})
    return c


def channel(ni=16, nj=12, nk=8, mach=0.5, reynolds=500.0, amp=0.05, les=1, seed=0) -> Case:
    """Wall-bounded channel on a perturbed grid: periodic in x (i) and z (k),
    no-slip walls at y = 0 (j-min) and the upper boundary (j-max) split into
    inlet (x < L/2) and outlet nodes, so the lattice path, the loc-code
    branches and every face rule of the boundary routine run together.
    Parabolic streamwise profile with a seeded perturbation."""
    Lx, H, Lz = 2.0, 1.0, 1.0
    hx, hy, hz = Lx / ni, H / (nj - 1), Lz / nk
    i, j, k = np.meshgrid(np.arange(ni), np.arange(nj), np.arange(nk), indexing="ij")
    xi, eta, zeta = i * hx, j * hy, k * hz
    X = xi + amp * hx * np.sin(2 * np.pi * eta / H) * np.cos(2 * np.pi * zeta / Lz)
    Y = eta + amp * hy * np.sin(2 * np.pi * xi / Lx) * np.cos(2 * np.pi * zeta / Lz)
    Z = zeta + amp * hz * np.sin(2 * np.pi * xi / Lx) * np.sin(np.pi * eta / H)
    rng = np.random.default_rng(seed)
    yn = np.clip(Y / H, 0.0, 1.0)
    u = 4.0 * yn * (1.0 - yn) + 0.02 * rng.standard_normal(X.shape)
    v = 0.02 * rng.standard_normal(X.shape)
    w = 0.02 * rng.standard_normal(X.shape)
    p = 1.0 / (1.4 * mach * mach) * (1.0 + 0.01 * np.sin(2 * np.pi * X / Lx))
    rho = np.ones(X.shape)
    prm = Params(mach=mach, reynolds=reynolds, viscous=1, les=les)

    def bc_type(ii, jj, kk, loc):
        if loc == 3:
            return "wall"
        if loc == 1:
            return "inlet" if ii < ni // 2 else "outlet"
        return None

    return ghosted_lattice("channel", X, Y, Z, (True, False, True), (rho, u, v, w, p), prm, mach, bc_type,
                           periods=((Lx, 0.0, 0.0), (0.0, 0.0, 0.0), (0.0, 0.0, Lz)))


def naca0012_thickness(x: np.ndarray, t: float = 0.12) -> np.ndarray:
    """Half thickness of the NACA 4-digit symmetric section, closed trailing
    edge (last coefficient -0.1036), chord 1."""
    return 5.0 * t * (0.2969 * np.sqrt(x) - 0.1260 * x - 0.3516 * x**2 + 0.2843 * x**3 - 0.1036 * x**4)


def naca0012(ni=512, nj=128, nk=32, mach=0.8, aoa_deg=1.25, reynolds=5e5, span=0.2, radius=15.0, beta=6.0,
             les=1, cfl=0.5) -> Case:
    """Shocked transonic case: an algebraic O-grid around a NACA0012 section.

    i (periodic) runs clockwise around the section from the trailing edge
    over the lower surface, x = (1 + cos phi)/2 (cosine clustering at both
    edges);
    j runs from the wall to a circle of `radius` chords about mid-chord with
    exponential clustering s = (e^(beta eta) - 1)/(e^beta - 1); k is the
    periodic span; three ghost layers mirror the first and last owned
    layers (ghosted_lattice).  The grid is rotated by -aoa about the
    quarter chord, so the reference's free stream (u = 1, v = 0, its inlet
    state) meets the section at the angle of attack.  Wall nodes are
    no-slip walls; far-field nodes upstream of mid-chord are inlets, the
    rest outlets.  Initial state: the free stream."""
    i = np.arange(ni)
    phi = -2.0 * np.pi * i / ni          # clockwise: (i, j, k) right-handed
    xs = 0.5 * (1.0 + np.cos(phi))
    ys = np.sign(np.sin(phi)) * naca0012_thickness(xs)
    xo = 0.5 + radius * np.cos(phi)
    yo = radius * np.sin(phi)
    eta = np.arange(nj) / (nj - 1)
    s = np.expm1(beta * eta) / np.expm1(beta)
    X2 = xs[:, None] + s[None, :] * (xo - xs)[:, None]
    Y2 = ys[:, None] + s[None, :] * (yo - ys)[:, None]
    a = math.radians(aoa_deg)
    Xr = 0.25 + (X2 - 0.25) * math.cos(a) + Y2 * math.sin(a)
    Yr = -(X2 - 0.25) * math.sin(a) + Y2 * math.cos(a)
    z = np.arange(nk) * span / nk
    X = np.repeat(Xr[:, :, None], nk, axis=2)
    Y = np.repeat(Yr[:, :, None], nk, axis=2)
    Z = np.broadcast_to(z[None, None, :], X.shape).copy()
    p_inf = 1.0 / (1.4 * mach * mach)
    prims = (np.ones(X.shape), np.ones(X.shape), np.zeros(X.shape), np.zeros(X.shape), np.full(X.shape, p_inf))
    prm = Params(mach=mach, reynolds=reynolds, viscous=1, les=les)
    upstream = np.cos(phi) < 0.0

    def bc_type(ii, jj, kk, loc):
        if loc == 3:
            return "wall"
        if loc == 1:
            return "inlet" if upstream[ii] else "outlet"
        return None

    return ghosted_lattice("naca0012", X, Y, Z, (True, False, True), prims, prm, mach, bc_type, cfl=cfl,
                           periods=((0.0, 0.0, 0.0), (0.0, 0.0, 0.0), (0.0, 0.0, span)))


def duct(ni=12, nj=10, nk=9, mach=0.5, reynolds=500.0, amp=0.04, seed=1) -> Case:
    """Square duct on a perturbed grid: periodic in x (i), no-slip walls on
    all four sides in y (j) and z (k), so the lattice path carries edge
    codes (15, 17, 19, 21) next to the face codes and the boundary
    routine's wall list mixes face and edge entries."""
    Lx, H, W = 2.0, 1.0, 1.0
    hx, hy, hz = Lx / ni, H / (nj - 1), W / (nk - 1)
    i, j, k = np.meshgrid(np.arange(ni), np.arange(nj), np.arange(nk), indexing="ij")
    xi, eta, zeta = i * hx, j * hy, k * hz
    X = xi + amp * hx * np.sin(np.pi * eta / H) * np.sin(np.pi * zeta / W)
    Y = eta + amp * hy * np.sin(2 * np.pi * xi / Lx) * np.sin(np.pi * zeta / W)
    Z = zeta + amp * hz * np.cos(2 * np.pi * xi / Lx) * np.sin(np.pi * eta / H)
    rng = np.random.default_rng(seed)
    u = 16.0 * (Y / H) * (1 - Y / H) * (Z / W) * (1 - Z / W) + 0.02 * rng.standard_normal(X.shape)
    v = 0.02 * rng.standard_normal(X.shape)
    w = 0.02 * rng.standard_normal(X.shape)
    p = np.full(X.shape, 1.0 / (1.4 * mach * mach))
    prm = Params(mach=mach, reynolds=reynolds, viscous=1, les=1)
    return ghosted_lattice("duct", X, Y, Z, (True, False, False), (np.ones(X.shape), u, v, w, p), prm, mach,
                           lambda ii, jj, kk, loc: "wall", periods=((Lx, 0.0, 0.0), (0.0, 0.0, 0.0), (0.0, 0.0, 0.0)))
