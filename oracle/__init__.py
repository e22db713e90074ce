"""CPU oracle for the RHS path -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
bench.py may import this package; the product never does.  It wraps two
shared libraries through ctypes:

* ``liboracle.so`` -- the C restatement in cfd_oracle.c (always built;
  plain C + OpenMP, portable to the Arm GPU host), compiled -O2 without
  FMA contraction: the parity build, bit-exact against the reference's own
  kernels on x86;
* ``liboracle_timed.so`` -- the same source compiled for speed (-O3, FMA
  contraction allowed, the host core named when it is a Neoverse V2): the
  CPU baseline that bench.py times, never a parity checker;
* ``_ref/libcfd_ref.so`` -- the reference's own kernel sources compiled as
  host C++ (build_ref.sh; only where the reference checkout exists).  It pins
  the restatement; golden vectors committed under tests/golden/ were made
  with it.

Arrays follow the reference layout documented in the product's layout module
(float64 row-major, row 0 = dummy row).
"""
from __future__ import annotations

import ctypes as C
import os
import pathlib
import subprocess

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
TIMED_LIB = HERE / "liboracle_timed.so"
REF_LIB = HERE / "_ref" / "libcfd_ref.so"
REF_GEOM_LIB = HERE / "_ref" / "libcfd_ref_geom.so"
# The reference checkout: CFD_REFERENCE_DIR, else a directory named
# "reference" beside this repository.
REFERENCE_DIR = pathlib.Path(os.environ.get("CFD_REFERENCE_DIR", HERE.parent.parent / "reference"))

_dp = C.POINTER(C.c_double)
_vp = C.c_void_p


class OrParams(C.Structure):
    _fields_ = [("mach", C.c_double), ("reynolds", C.c_double), ("prandtl", C.c_double),
                ("t_inf", C.c_double), ("weno_eps", C.c_double), ("viscous", C.c_int),
                ("les", C.c_int), ("smagorinsky_cs", C.c_double)]


class OrCase(C.Structure):
    _fields_ = [("g_node", C.c_int), ("sd_node", C.c_int)] + [
        (n, _vp) for n in ("grid", "det", "deter", "metric", "flow", "U0", "U1", "U2", "Q",
                           "F", "E", "G", "Fv", "Ev", "Gv", "roe")]


class OrBcLists(C.Structure):
    _fields_ = [("outlet", _vp), ("inlet", _vp), ("boundary", _vp), ("wall", _vp),
                ("n_outlet", C.c_int), ("n_inlet", C.c_int), ("n_boundary", C.c_int), ("n_wall", C.c_int),
                ("singular", _vp), ("tips", _vp), ("n_tips", C.c_int)]


def make_bc(bc) -> OrBcLists:
    """ctypes view of a cases.BoundaryLists (the arrays must stay alive)."""
    sing = getattr(bc, "singular", None)
    tips = getattr(bc, "tips", None)
    return OrBcLists(_p(bc.outlet), _p(bc.inlet), _p(bc.boundary), _p(bc.wall),
                     len(bc.outlet), len(bc.inlet), len(bc.boundary), len(bc.wall),
                     _p(sing) if sing is not None else None, _p(tips) if tips is not None and len(tips) else None,
                     0 if tips is None else len(tips))


def _host_core_flags() -> list[str]:
    """-mcpu for the timed build: Grace's Neoverse V2 named explicitly when
    /proc/cpuinfo reports that core (CPU part 0xd4f); nothing elsewhere."""
    import platform
    if platform.machine() not in ("aarch64", "arm64"):
        return []
    try:
        info = pathlib.Path("/proc/cpuinfo").read_text()
    except OSError:
        return []
    return ["-mcpu=neoverse-v2"] if "0xd4f" in info else []


TIMED_FLAGS = ["-std=gnu11", "-O3", "-ffp-contract=fast", "-fopenmp"]


def timed_build_flags() -> str:
    return " ".join(TIMED_FLAGS + _host_core_flags())


def build(force: bool = False) -> None:
    """Compile the restatement (parity and timed builds) and the reference
    pin where the reference checkout exists."""
    src = HERE / "cfd_oracle.c"
    newest = max(src.stat().st_mtime, (HERE / "cfd_oracle.h").stat().st_mtime)
    if force or not LIB.exists() or LIB.stat().st_mtime < newest:
        subprocess.run(["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
                        str(src), "-o", str(LIB), "-lm"], check=True)
    if force or not TIMED_LIB.exists() or TIMED_LIB.stat().st_mtime < newest:
        subprocess.run(["gcc", *TIMED_FLAGS, *_host_core_flags(), "-fPIC", "-shared", str(src), "-o",
                        str(TIMED_LIB), "-lm"], check=True)
    ref_dir = REFERENCE_DIR
    ref_srcs = [HERE / n for n in ("build_ref.sh", "ref_kernels.cpp", "ref_bc.cpp", "ref_shim.h", "bc_ref_shim.h",
                                   "ref_metrics.cpp", "metric_ref_shim.h")]
    stale = not REF_GEOM_LIB.exists() or REF_LIB.stat().st_mtime < max(p.stat().st_mtime for p in ref_srcs)
    if (ref_dir / "Weno.cl").exists() and (force or stale):
        subprocess.run(["bash", str(HERE / "build_ref.sh")], check=True)


_lib = None
_timed = None
_ref = None
_ref_geom = None


def lib():
    """The parity build."""
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        _lib = _declare(C.CDLL(str(LIB)))
    return _lib


def timed_lib():
    """The build that bench.py times as the CPU baseline."""
    global _timed
    if _timed is None:
        if not TIMED_LIB.exists():
            build()
        _timed = _declare(C.CDLL(str(TIMED_LIB)))
    return _timed


def _declare(L):
    """Argument and result types of the restatement's entry points."""
    L.oracle_stage.argtypes = [C.POINTER(OrCase), C.POINTER(OrParams), C.c_int, C.c_double, _vp]
    L.oracle_rk3_steps.argtypes = [C.POINTER(OrCase), C.POINTER(OrParams), C.c_double, C.c_int]
    L.oracle_uq.argtypes = [C.c_int] + [_vp] * 6
    L.oracle_viscous.argtypes = [C.c_int, C.POINTER(OrParams)] + [_vp] * 11
    L.oracle_weno.argtypes = ([C.c_int, C.c_int, C.c_double, C.c_double, C.POINTER(OrParams)]
                                 + [_vp] * 17)
    L.oracle_boundary_fill.argtypes = [_vp, _vp, C.POINTER(OrBcLists), C.c_double, C.c_int, C.c_int]
    L.oracle_boundary_fill.restype = C.c_int
    L.oracle_rk3_steps_bc.argtypes = [C.POINTER(OrCase), C.POINTER(OrParams), C.c_double, C.c_int,
                                         C.POINTER(OrBcLists)]
    L.oracle_rk3_steps_bc.restype = C.c_int
    L.oracle_set_threads.argtypes = [C.c_int]
    L.oracle_set_poison.argtypes = [C.c_int]
    L.oracle_get_threads.restype = C.c_int
    L.oracle_compact_metrics.argtypes = [_vp, C.c_int, C.c_double, _vp, _vp]
    L.oracle_compact_metrics.restype = C.c_int
    L.oracle_half_point_metrics.argtypes = [_vp, C.c_int, _vp, _vp, _vp]
    return L


def ref_available() -> bool:
    return REF_LIB.exists()


def ref():
    global _ref
    if _ref is None:
        _ref = C.CDLL(str(REF_LIB))
        _ref.ref_uq.argtypes = [C.c_int] + [_vp] * 6
        _ref.ref_viscous.argtypes = [C.c_int] + [_vp] * 11
        _ref.ref_viscous_param.argtypes = [C.c_int] + [C.c_double] * 4 + [_vp] * 11
        _ref.ref_weno.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double] + [_vp] * 16
        _ref.ref_boundary_fill.argtypes = ([_vp, _vp, C.c_int] + [_vp, C.c_int] * 4
                                           + [C.c_double, C.c_int, C.c_int, _vp])
    return _ref


def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_vp)


def make_params(p) -> OrParams:
    return OrParams(p.mach, p.reynolds, p.prandtl, p.t_inf, p.weno_eps, int(p.viscous), int(p.les),
                    float(getattr(p, "smagorinsky_cs", 0.1)))


def make_case(arrays: dict, g_node: int, sd_node: int) -> OrCase:
    c = OrCase()
    c.g_node = g_node
    c.sd_node = sd_node
    for name, _ in OrCase._fields_[2:]:
        setattr(c, name, _p(arrays[name]))
    return c


def set_poison(on: bool) -> None:
    lib().oracle_set_poison(1 if on else 0)


def set_threads(n: int) -> None:
    lib().oracle_set_threads(int(n))


# ------------------------------------------------------------ restatement --

def stage(arrays: dict, g_node: int, sd_node: int, params, j: int, dt: float, want_L: bool = False):
    """One RK stage (U_Q, Viscous, Weno(j)) in place; returns L (rows x 5)."""
    Lout = np.zeros((g_node + 1, 5)) if want_L else None
    c = make_case(arrays, g_node, sd_node)
    pr = make_params(params)
    lib().oracle_stage(C.byref(c), C.byref(pr), int(j), float(dt), _p(Lout) if want_L else None)
    return Lout


def rk3_steps(arrays: dict, g_node: int, sd_node: int, params, dt: float, nsteps: int, timed: bool = False) -> None:
    """nsteps whole SSP-RK3 steps in place (timed: through the timed build)."""
    c = make_case(arrays, g_node, sd_node)
    pr = make_params(params)
    (timed_lib() if timed else lib()).oracle_rk3_steps(C.byref(c), C.byref(pr), float(dt), int(nsteps))


def boundary_fill(arrays: dict, bc, mach: float, initial: int = 1, sd_node: int = 0) -> None:
    """The boundary routine (intialise) on arrays["flow"] in place."""
    lists = make_bc(bc)
    rc = lib().oracle_boundary_fill(_p(arrays["grid"]), _p(arrays["flow"]), C.byref(lists), float(mach),
                                    int(initial), int(sd_node))
    if rc != 0:
        raise ValueError("a wall node needs the singular-node table (none given) or has code 53..56")


def rk3_steps_bc(arrays: dict, g_node: int, sd_node: int, params, dt: float, nsteps: int, bc) -> None:
    """rk3_steps with the boundary routine after every stage."""
    c = make_case(arrays, g_node, sd_node)
    pr = make_params(params)
    lists = make_bc(bc)
    if lib().oracle_rk3_steps_bc(C.byref(c), C.byref(pr), float(dt), int(nsteps), C.byref(lists)) != 0:
        raise ValueError("a wall node needs the singular-node table (none given) or has code 53..56")


def uq(a: dict, n_items: int, U_out: np.ndarray) -> None:
    lib().oracle_uq(n_items, _p(U_out), _p(a["Q"]), _p(a["grid"]), _p(a["det"]), _p(a["flow"]), _p(a["roe"]))


def viscous(a: dict, n_items: int, params, U_in: np.ndarray) -> None:
    pr = make_params(params)
    lib().oracle_viscous(n_items, C.byref(pr), _p(U_in), _p(a["F"]), _p(a["E"]), _p(a["G"]), _p(a["Fv"]),
                         _p(a["Ev"]), _p(a["Gv"]), _p(a["grid"]), _p(a["metric"]), _p(a["det"]), _p(a["flow"]))


def weno(a: dict, n_items: int, params, j: int, dt: float, want_L: bool = False):
    Lout = np.zeros((a["det"].shape[0], 5)) if want_L else None
    pr = make_params(params)
    lib().oracle_weno(n_items, int(j), params.mach, float(dt), C.byref(pr), _p(a["deter"]), _p(a["det"]),
                      _p(a["U0"]), _p(a["U1"]), _p(a["U2"]), _p(a["grid"]), _p(a["Q"]), _p(a["metric"]),
                      _p(a["roe"]), _p(a["Fv"]), _p(a["Ev"]), _p(a["Gv"]), _p(a["F"]), _p(a["E"]), _p(a["G"]),
                      _p(a["flow"]), _p(Lout) if want_L else None)
    return Lout


# ------------------------------------------------- reference (pin) build --

def ref_uq(a: dict, n_items: int, U_out: np.ndarray) -> None:
    ref().ref_uq(n_items, _p(U_out), _p(a["Q"]), _p(a["grid"]), _p(a["det"]), _p(a["flow"]), _p(a["roe"]))


def ref_viscous(a: dict, n_items: int, params, U_in: np.ndarray) -> None:
    """The reference Viscous kernel; with its own constants when ``params``
    carries them (1.5, 500, 0.72, 273), else the constant-substituted copy."""
    args = (_p(U_in), _p(a["F"]), _p(a["E"]), _p(a["G"]), _p(a["Fv"]), _p(a["Ev"]), _p(a["Gv"]),
            _p(a["grid"]), _p(a["metric"]), _p(a["det"]), _p(a["flow"]))
    if (params.mach, params.reynolds, params.prandtl, params.t_inf) == (1.5, 500.0, 0.72, 273.0):
        ref().ref_viscous(n_items, *args)
    else:
        ref().ref_viscous_param(n_items, params.mach, params.reynolds, params.prandtl, params.t_inf, *args)
    if not params.viscous:
        for k in ("Fv", "Ev", "Gv"):
            a[k][:n_items] = 0.0


def ref_weno(a: dict, n_items: int, mach: float, j: int, dt: float) -> None:
    ref().ref_weno(n_items, int(j), float(mach), float(dt), _p(a["deter"]), _p(a["det"]), _p(a["U0"]),
                   _p(a["U1"]), _p(a["U2"]), _p(a["grid"]), _p(a["Q"]), _p(a["metric"]), _p(a["roe"]),
                   _p(a["Fv"]), _p(a["Ev"]), _p(a["Gv"]), _p(a["F"]), _p(a["E"]), _p(a["G"]), _p(a["flow"]))


def ref_boundary_fill(arrays: dict, bc, mach: float, initial: int = 1, sd_node: int = 0) -> None:
    """The reference's own intialise() on arrays["flow"] in place, with the
    singular-node table of ``bc`` when it has one (the tip fix-ups belong to
    the solver loop, not to intialise, and are not applied here)."""
    n = arrays["flow"].shape[0]
    sing = getattr(bc, "singular", None)
    ref().ref_boundary_fill(_p(arrays["grid"]), _p(arrays["flow"]), n, _p(bc.outlet), len(bc.outlet),
                            _p(bc.inlet), len(bc.inlet), _p(bc.boundary), len(bc.boundary), _p(bc.wall),
                            len(bc.wall), float(mach), int(initial), int(sd_node),
                            _p(sing) if sing is not None else None)


def ref_stage(a: dict, g_node: int, sd_node: int, params, j: int, dt: float) -> None:
    """Solver.cpp:365-541 sequencing with the reference kernels themselves.
    The reference kernels use eps = 1e-7 (Weno.cl:59) and always run MTS."""
    Uj = a[("U0", "U1", "U2")[j]]
    ref_uq(a, g_node + 1, Uj)
    ref_viscous(a, g_node + 1, params, Uj)
    ref_weno(a, sd_node + 1, params.mach, j, dt)


# ------------------------------------------------------- geometry producer --

def compact_metrics(grid: np.ndarray, det: np.ndarray, metric: np.ndarray, del_zeta: float = 1.0) -> None:
    """Node metrics (metric[:, 0:9]) and det by the compact scheme, in place."""
    if lib().oracle_compact_metrics(_p(grid), int(grid.shape[0]), float(del_zeta), _p(det), _p(metric)) != 0:
        raise ValueError("table has ID 10 rows or a line shorter than three rows")


def half_point_metrics(grid: np.ndarray, n_owned: int, det: np.ndarray, metric: np.ndarray, deter: np.ndarray) -> None:
    """Face metrics and face dets of rows 1..n_owned, in place."""
    lib().oracle_half_point_metrics(_p(grid), int(n_owned), _p(det), _p(metric), _p(deter))


def ref_geom_available() -> bool:
    return REF_GEOM_LIB.exists()


def ref_geom():
    global _ref_geom
    if _ref_geom is None:
        _ref_geom = C.CDLL(str(REF_GEOM_LIB))
        _ref_geom.ref_compact_metrics.argtypes = [_vp, C.c_int, _vp, _vp]
        _ref_geom.ref_half_point_metrics.argtypes = [_vp, C.c_int, C.c_int, _vp, _vp, _vp]
    return _ref_geom


def ref_compact_metrics(grid: np.ndarray, det: np.ndarray, metric: np.ndarray) -> None:
    """The reference's own metric_term() (node block of metric, det), in place."""
    ref_geom().ref_compact_metrics(_p(grid), int(grid.shape[0]), _p(det), _p(metric))


def ref_half_point_metrics(grid: np.ndarray, n_owned: int, det: np.ndarray, metric: np.ndarray,
                           deter: np.ndarray) -> None:
    """The reference's own half-point block of Main.cpp, in place."""
    ref_geom().ref_half_point_metrics(_p(grid), int(grid.shape[0]), int(n_owned), _p(det), _p(metric), _p(deter))
