"""Host-side mirror of the reference's RHS interface over the C ABI.

``Context`` mirrors the reference's OpenCL objects: device buffers
(``cl::Buffer``, Solver.cpp:232-273), copies (``cl::copy``) and the three
kernel launches with the reference's argument order (``uq``, ``viscous``,
``weno``; Solver.cpp:277-315, 377, 440, 521).  ``Solver`` is the resident
form of the reference host loop (Solver.cpp:356-658): the state stays on the
device and whole SSP-RK3 steps run without host round trips.

Errors surface as ``CfdError`` carrying the library's status code, instead of
the reference's print-and-exit.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import weakref

import numpy as np

from . import abi
from . import layout as L

# per-row sizes (bytes) of every reference buffer
ROW_BYTES = {"grid": 56, "det": 8, "deter": 48, "metric": 504, "flow": 72, "U0": 40, "U1": 40, "U2": 40,
             "Q": 40, "F": 40, "E": 40, "G": 40, "Fv": 40, "Ev": 40, "Gv": 40, "roe": 288, "L": 40}


def to_params(p) -> abi.Params:
    out = abi.Params()
    abi.load().cfd_params_default(C.byref(out))
    if p is None:
        return out
    out.mach, out.reynolds, out.prandtl, out.t_inf = p.mach, p.reynolds, p.prandtl, p.t_inf
    out.weno_eps = p.weno_eps
    out.viscous, out.les = int(p.viscous), int(p.les)
    out.precision = int(getattr(p, "precision", 0))
    out.smagorinsky_cs = float(getattr(p, "smagorinsky_cs", 0.1))
    return out


def _ptr(a: np.ndarray) -> int:
    assert a.flags["C_CONTIGUOUS"], "arrays must be C-contiguous"
    return a.ctypes.data


class Context:
    """One CUDA device + stream; owns the error state of its launches."""

    def __init__(self, device: int = 0):
        self.lib = abi.load()
        h = C.c_void_p()
        s = self.lib.cfd_ctx_create(C.byref(h), int(device))
        if s != abi.OK:
            raise abi.CfdError(s, "cfd_ctx_create")
        self.h = h
        self._buffers = []
        # solvers, batches and boundary plans of this context: closed before
        # the context itself (they hold device memory and use its stream)
        self._children = weakref.WeakSet()

    # -- errors --
    def check(self, status: int, where: str):
        if status != abi.OK:
            detail = self.lib.cfd_last_error(self.h)
            raise abi.CfdError(status, where, detail.decode() if detail else "")

    def close(self):
        if self.h:
            for ch in list(self._children):
                ch.close()
            for p in self._buffers:
                self.lib.cfd_buffer_free(self.h, p)
            self._buffers = []
            self.lib.cfd_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, cuda_stream: int):
        """Launch on a caller-owned cudaStream_t (e.g. a torch stream)."""
        self.check(self.lib.cfd_ctx_set_stream(self.h, C.c_void_p(cuda_stream)), "cfd_ctx_set_stream")

    def probe_flops(self, fp64: bool) -> float:
        out = C.c_double()
        self.check(self.lib.cfd_probe_flops(self.h, 1 if fp64 else 0, C.byref(out)), "cfd_probe_flops")
        return out.value

    def probe_emu64(self, n_per_class: int = 1 << 22, seed: int = 1) -> tuple:
        """Mismatch counts (f2d, d2f, add/sub, mul, shared-reciprocal
        division) of the integer-pipe binary64 routines against the device's
        instructions (cfd_probe_emu64); all zero on a correct build."""
        out = (C.c_int64 * 5)()
        self.check(self.lib.cfd_probe_emu64(self.h, int(n_per_class), int(seed), out), "cfd_probe_emu64")
        return tuple(int(v) for v in out)

    def set_rows(self, n_rows: int):
        self.check(self.lib.cfd_ctx_set_rows(self.h, int(n_rows)), "cfd_ctx_set_rows")

    def set_face_reuse(self, on: bool):
        """cfd_weno: share each interior face between its two rows (default)
        or evaluate both faces at every row as the reference does."""
        self.check(self.lib.cfd_ctx_set_face_reuse(self.h, 1 if on else 0), "cfd_ctx_set_face_reuse")

    def set_async(self, on: bool):
        self.check(self.lib.cfd_ctx_set_async(self.h, 1 if on else 0), "cfd_ctx_set_async")

    def synchronize(self):
        self.check(self.lib.cfd_ctx_synchronize(self.h), "cfd_ctx_synchronize")

    @property
    def launch_count(self) -> int:
        return int(self.lib.cfd_ctx_launch_count(self.h))

    # -- buffers (cl::Buffer / cl::copy) --
    def alloc(self, nbytes: int) -> int:
        p = C.c_void_p()
        self.check(self.lib.cfd_buffer_alloc(self.h, int(nbytes), C.byref(p)), "cfd_buffer_alloc")
        self._buffers.append(p.value)
        return p.value

    def free(self, ptr: int):
        self.check(self.lib.cfd_buffer_free(self.h, C.c_void_p(ptr)), "cfd_buffer_free")
        self._buffers.remove(ptr)

    def write(self, dev: int, host: np.ndarray):
        self.check(self.lib.cfd_buffer_write(self.h, C.c_void_p(dev), C.c_void_p(_ptr(host)), host.nbytes),
                   "cfd_buffer_write")

    def read(self, host: np.ndarray, dev: int):
        self.check(self.lib.cfd_buffer_read(self.h, C.c_void_p(_ptr(host)), C.c_void_p(dev), host.nbytes),
                   "cfd_buffer_read")

    def upload_case(self, arrays: dict, names=None) -> dict:
        """Device copies of the reference buffers of a case (plus L)."""
        names = names or list(arrays) + ["L"]
        n_rows = arrays["det"].shape[0]
        dev = {}
        for k in names:
            dev[k] = self.alloc(ROW_BYTES[k] * n_rows)
            if k in arrays:
                self.write(dev[k], np.ascontiguousarray(arrays[k]))
        self.set_rows(n_rows)
        return dev

    def download(self, dev: dict, name: str, like: np.ndarray) -> np.ndarray:
        out = np.empty_like(like)
        self.read(out, dev[name])
        return out

    # -- the three reference kernels (device pointers, reference arg order) --
    def uq(self, U_C, Q_C, Grid_P, det, FLOW, ROE_AVER, n_items: int):
        self.check(self.lib.cfd_uq(self.h, U_C, Q_C, Grid_P, det, FLOW, ROE_AVER, int(n_items)), "cfd_uq")

    def viscous(self, U_C, F_C, E_C, G_C, Fv_C, Ev_C, Gv_C, Grid_P, metric, det, FLOW, n_items: int, params=None):
        pr = to_params(params)
        self.check(self.lib.cfd_viscous(self.h, U_C, F_C, E_C, G_C, Fv_C, Ev_C, Gv_C, Grid_P, metric, det, FLOW,
                                        int(n_items), C.byref(pr)), "cfd_viscous")

    def weno(self, j, Mach, del_t, deter, det, U0, U1, U2, Grid_P, Q_C, metric, ROE_AVER, Fv, Ev, Gv, F, E, G,
             FLOW, n_items: int, params=None, L_out=None):
        pr = to_params(params)
        self.check(self.lib.cfd_weno(self.h, int(j), float(Mach), float(del_t), deter, det, U0, U1, U2, Grid_P, Q_C,
                                     metric, ROE_AVER, Fv, Ev, Gv, F, E, G, FLOW, int(n_items), C.byref(pr), L_out),
                   "cfd_weno")

    def rk3_step(self, bufs: dict, g_node: int, sd_node: int, params, dt: float, nsteps: int = 1, bc=None):
        """cfd_rk3_step: nsteps SSP-RK3 steps on the reference buffers in one
        call.  bufs maps buffer names to device pointers (ints) or host numpy
        arrays of g_node + 1 rows (copied in and back by the library); bc is
        an optional Boundary."""
        def ptr(x):
            if isinstance(x, np.ndarray):
                assert x.flags["C_CONTIGUOUS"]
                return C.c_void_p(x.ctypes.data)
            return C.c_void_p(x)
        b = {k: ptr(v) for k, v in bufs.items()}
        pr = to_params(params)
        self.check(self.lib.cfd_rk3_step(self.h, float(params.mach), float(dt), b["deter"], b["det"], b["U0"], b["U1"],
                                         b["U2"], b["grid"], b["Q"], b["metric"], b["roe"], b["Fv"], b["Ev"], b["Gv"],
                                         b["F"], b["E"], b["G"], b["flow"], int(g_node), int(sd_node), C.byref(pr),
                                         bc.h if bc is not None else None, int(nsteps)), "cfd_rk3_step")

    def stage(self, dev: dict, g_node: int, sd_node: int, params, j: int, dt: float, want_L: bool = False):
        """One stage of the reference host loop (Solver.cpp:365-541) through
        the three drop-in entry points; U_Q writes U_j, Viscous reads U_j."""
        Uj = dev[("U0", "U1", "U2")[j]]
        self.uq(Uj, dev["Q"], dev["grid"], dev["det"], dev["flow"], dev["roe"], g_node + 1)
        self.viscous(Uj, dev["F"], dev["E"], dev["G"], dev["Fv"], dev["Ev"], dev["Gv"], dev["grid"], dev["metric"],
                     dev["det"], dev["flow"], g_node + 1, params)
        self.weno(j, params.mach, dt, dev["deter"], dev["det"], dev["U0"], dev["U1"], dev["U2"], dev["grid"],
                  dev["Q"], dev["metric"], dev["roe"], dev["Fv"], dev["Ev"], dev["Gv"], dev["F"], dev["E"], dev["G"],
                  dev["flow"], sd_node + 1, params, dev["L"] if want_L else None)


@dataclasses.dataclass
class SolverInfo:
    path: str
    shape: tuple
    precision: str
    device_bytes: int
    face_tiles: tuple = (0, 0)     # (along i, along j and k); mixed/split lattices
    face_blocks: tuple = (0, 0, 0)  # blocks per SM of the i, j, k face passes; FP64 lattices


class Boundary:
    """The reference's boundary routine for one table (cfd_bc_*): the plan of
    a cases.BoundaryLists resolved against the neighbour table.  A
    BoundaryLists with a singular-node table or tip rows goes through
    cfd_bc_create_singular."""

    def __init__(self, ctx: Context, grid: np.ndarray, bc):
        self.ctx = ctx
        self.lib = ctx.lib
        self._lists = tuple(np.ascontiguousarray(getattr(bc, t), dtype=np.int32)
                            for t in ("outlet", "inlet", "boundary", "wall"))
        args = []
        for a in self._lists:
            args += [_ptr(a) if a.size else None, int(a.size)]
        h = C.c_void_p()
        sing = getattr(bc, "singular", None)
        tips = getattr(bc, "tips", None)
        if sing is None and tips is None:
            ctx.check(self.lib.cfd_bc_create(ctx.h, _ptr(grid), int(grid.shape[0]), *args, C.byref(h)),
                      "cfd_bc_create")
        else:
            self._sing = None if sing is None else np.ascontiguousarray(sing, dtype=np.int32).reshape(-1, 6)
            if self._sing is not None and self._sing.shape[0] != grid.shape[0]:
                raise ValueError("singular table needs one row of six slots per grid row")
            self._tips = np.ascontiguousarray(tips if tips is not None else [], dtype=np.int32)
            ctx.check(self.lib.cfd_bc_create_singular(
                ctx.h, _ptr(grid), int(grid.shape[0]), *args, _ptr(self._sing) if self._sing is not None else None,
                _ptr(self._tips) if self._tips.size else None, int(self._tips.size), C.byref(h)),
                "cfd_bc_create_singular")
        self.h = h
        ctx._children.add(self)

    def fill(self, flow_dev: int, mach: float, initial: int = 1, sd_node: int = 0):
        """intialise() on a device FLOW buffer (reference layout)."""
        self.ctx.check(self.lib.cfd_boundary_fill(self.ctx.h, self.h, C.c_void_p(flow_dev), float(mach), int(initial),
                                                  int(sd_node)), "cfd_boundary_fill")

    def close(self):
        if self.h and self.ctx.h:
            self.lib.cfd_bc_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Solver:
    """Resident RHS solver for one grid (cfd_solver_*).  A case with boundary
    lists (case.bc) gets the reference's boundary routine after every stage
    unless ``boundary=False``."""

    def __init__(self, ctx: Context, case, params=None, force_path: int = -1, precision: int = 0,
                 boundary: bool = True):
        self.ctx = ctx
        self.lib = ctx.lib
        a = case.arrays
        self._geom_arrays = (a["grid"], a["det"], a["deter"], a["metric"])
        self.g_node, self.sd_node = case.g_node, case.sd_node
        geom = abi.Geometry(case.g_node, case.sd_node, _ptr(a["grid"]), _ptr(a["det"]), _ptr(a["deter"]),
                            _ptr(a["metric"]))
        pr = to_params(params if params is not None else case.params)
        pr.precision = int(precision)
        h = C.c_void_p()
        ctx.check(self.lib.cfd_solver_create(ctx.h, C.byref(geom), C.byref(pr), int(force_path), C.byref(h)),
                  "cfd_solver_create")
        self.h = h
        ctx._children.add(self)
        self.boundary = None
        if boundary and getattr(case, "bc", None) is not None:
            self.set_boundary(Boundary(ctx, a["grid"], case.bc))

    def set_boundary(self, bnd: "Boundary | None"):
        """Run the boundary routine after every stage (None: off)."""
        self.ctx.check(self.lib.cfd_solver_set_boundary(self.h, bnd.h if bnd is not None else None),
                       "cfd_solver_set_boundary")
        self.boundary = bnd

    def close(self):
        if self.h and self.ctx.h:
            self.lib.cfd_solver_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self) -> SolverInfo:
        i = abi.SolverInfo()
        self.ctx.check(self.lib.cfd_solver_info(self.h, C.byref(i)), "cfd_solver_info")
        return SolverInfo("structured" if i.path == abi.PATH_STRUCTURED else "gather", (i.ni, i.nj, i.nk),
                          abi.PREC_NAMES[i.precision], int(i.device_bytes), (int(i.face_tile_i), int(i.face_tile_jk)),
                          tuple(int(b) for b in i.face_blocks))

    def set_face_tiles(self, tile_i: int = 0, tile_jk: int = 0):
        """Fix the face-tile widths of a mixed or split lattice solver."""
        self.ctx.check(self.lib.cfd_solver_set_face_tiles(self.h, int(tile_i), int(tile_jk)),
                       "cfd_solver_set_face_tiles")

    def set_face_blocks(self, blocks_i: int = 0, blocks_j: int = 0, blocks_k: int = 0):
        """Fix the register budgets (blocks per SM) of an FP64 lattice solver's
        face passes."""
        self.ctx.check(self.lib.cfd_solver_set_face_blocks(self.h, int(blocks_i), int(blocks_j), int(blocks_k)),
                       "cfd_solver_set_face_blocks")

    def set_flow(self, flow: np.ndarray):
        assert flow.shape == (self.g_node + 1, L.NFLOW) and flow.dtype == np.float64
        self.ctx.check(self.lib.cfd_solver_set_flow(self.h, C.c_void_p(_ptr(flow))), "cfd_solver_set_flow")

    def get_flow(self, out: np.ndarray | None = None) -> np.ndarray:
        out = np.empty((self.g_node + 1, L.NFLOW)) if out is None else out
        self.ctx.check(self.lib.cfd_solver_get_flow(self.h, C.c_void_p(_ptr(out))), "cfd_solver_get_flow")
        return out

    def get_u0(self) -> np.ndarray:
        out = np.empty((self.g_node + 1, L.NCOL))
        self.ctx.check(self.lib.cfd_solver_get_u0(self.h, C.c_void_p(_ptr(out))), "cfd_solver_get_u0")
        return out

    def step(self, dt: float, nsteps: int = 1):
        self.ctx.check(self.lib.cfd_solver_step(self.h, float(dt), int(nsteps)), "cfd_solver_step")

    def profile_stage(self, j: int, dt: float) -> list:
        """One stage with per-launch device times: [(name, ms), ...]."""
        buf = (abi.KernelTime * 16)()
        n = C.c_int32()
        self.ctx.check(self.lib.cfd_solver_profile_stage(self.h, int(j), float(dt), buf, 16, C.byref(n)),
                       "cfd_solver_profile_stage")
        return [(buf[i].name.decode(), buf[i].ms) for i in range(n.value)]

    def stage(self, j: int, dt: float, want_L: bool = True):
        out = np.zeros((self.g_node + 1, L.NCOL)) if want_L else None
        self.ctx.check(self.lib.cfd_solver_stage(self.h, int(j), float(dt), C.c_void_p(_ptr(out)) if want_L else None),
                       "cfd_solver_stage")
        return out


@dataclasses.dataclass
class BatchInfo:
    n_active: int
    tile_nodes: int
    blocks: int
    graph: bool
    precision: str
    nodes_total: int
    device_bytes: int
    capacity_bytes: int
    n_held: int = 0
    face_tiles: bool = False


class StagedInstance:
    """A batch instance converted on the host (Batch.stage), not yet added;
    freed if it is never added."""

    def __init__(self, lib, h, rows: int):
        self.lib, self.h, self.rows = lib, h, rows

    def take(self):
        h, self.h = self.h, None
        if h is None:
            raise ValueError("staged instance already added")
        return h

    def __del__(self):
        try:
            if getattr(self, "h", None) is not None:
                self.lib.cfd_batch_staged_free(self.h)
                self.h = None
        except Exception:
            pass


class Batch:
    """Many periodic-lattice instances advanced together (cfd_batch_*): one
    persistent launch per RK stage over all instances, CUDA-graph replay."""

    def __init__(self, ctx: Context, precision: int = 0, capacity_bytes: int = 0):
        self.ctx = ctx
        self.lib = ctx.lib
        h = C.c_void_p()
        ctx.check(self.lib.cfd_batch_create(ctx.h, int(precision), int(capacity_bytes), C.byref(h)), "cfd_batch_create")
        self.h = h
        self.rows = {}
        ctx._children.add(self)

    @staticmethod
    def instance_bytes(precision: int, nodes: int) -> int:
        return int(abi.load().cfd_batch_instance_bytes(int(precision), int(nodes)))

    def close(self):
        if self.h and self.ctx.h:
            self.lib.cfd_batch_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, case, flow=None, dt=None, params=None) -> int:
        a = case.arrays
        geom = abi.Geometry(case.g_node, case.sd_node, _ptr(a["grid"]), _ptr(a["det"]), _ptr(a["deter"]),
                            _ptr(a["metric"]))
        pr = to_params(params if params is not None else case.params)
        f = np.ascontiguousarray(a["flow"] if flow is None else flow)
        slot = C.c_int32()
        self.ctx.check(self.lib.cfd_batch_add(self.h, C.byref(geom), C.byref(pr), C.c_void_p(_ptr(f)),
                                              float(case.dt if dt is None else dt), C.byref(slot)), "cfd_batch_add")
        self.rows[slot.value] = case.g_node + 1
        return slot.value

    @staticmethod
    def stage(case, flow=None, dt=None, params=None) -> "StagedInstance":
        """The host half of add() (cfd_batch_stage): checks the table and
        converts geometry and FLOW into library-owned host memory.  Uses no
        device, context or batch, and releases the GIL, so it can run on a
        worker thread while the batch steps."""
        lib = abi.load()
        a = case.arrays
        geom = abi.Geometry(case.g_node, case.sd_node, _ptr(a["grid"]), _ptr(a["det"]), _ptr(a["deter"]),
                            _ptr(a["metric"]))
        pr = to_params(params if params is not None else case.params)
        f = np.ascontiguousarray(a["flow"] if flow is None else flow)
        h = C.c_void_p()
        st = lib.cfd_batch_stage(C.byref(geom), C.byref(pr), C.c_void_p(_ptr(f)),
                                 float(case.dt if dt is None else dt), C.byref(h))
        if not h.value:
            raise abi.CfdError(st, "cfd_batch_stage: out of host memory")
        return StagedInstance(lib, h, case.g_node + 1)

    def add_staged(self, staged: "StagedInstance") -> int:
        """The device half of add(): allocates, uploads and prepares a staged
        instance (consumed, also on failure)."""
        h = staged.take()
        slot = C.c_int32()
        self.ctx.check(self.lib.cfd_batch_add_staged(self.h, h, C.byref(slot)), "cfd_batch_add_staged")
        self.rows[slot.value] = staged.rows
        return slot.value

    def remove(self, slot: int):
        self.ctx.check(self.lib.cfd_batch_remove(self.h, int(slot)), "cfd_batch_remove")
        self.rows.pop(slot, None)

    def step(self, nsteps: int = 1):
        self.ctx.check(self.lib.cfd_batch_step(self.h, int(nsteps)), "cfd_batch_step")

    def step_async(self, nsteps: int = 1):
        """Queues the steps; returns once the previous call's steps are done."""
        self.ctx.check(self.lib.cfd_batch_step_async(self.h, int(nsteps)), "cfd_batch_step_async")

    def sync(self):
        """Waits for every queued step; raises on their errors."""
        self.ctx.check(self.lib.cfd_batch_sync(self.h), "cfd_batch_sync")

    def set_hold(self, slot: int, hold: bool):
        """A held instance stays resident but is not advanced by step()."""
        self.ctx.check(self.lib.cfd_batch_set_hold(self.h, int(slot), 1 if hold else 0), "cfd_batch_set_hold")

    def get_flow(self, slot: int) -> np.ndarray:
        out = np.empty((self.rows[slot], L.NFLOW))
        self.ctx.check(self.lib.cfd_batch_get_flow(self.h, int(slot), C.c_void_p(_ptr(out))), "cfd_batch_get_flow")
        return out

    def get_u0(self, slot: int) -> np.ndarray:
        out = np.empty((self.rows[slot], L.NCOL))
        self.ctx.check(self.lib.cfd_batch_get_u0(self.h, int(slot), C.c_void_p(_ptr(out))), "cfd_batch_get_u0")
        return out

    def slot_status(self, slot: int) -> int:
        return int(self.lib.cfd_batch_slot_status(self.h, int(slot)))

    def set_flow(self, slot: int, flow: np.ndarray):
        """Replace an instance's state (FLOW rows 0..g_node) and prepare its
        next step; the recovery path after a barrier timeout."""
        f = np.ascontiguousarray(flow, dtype=np.float64)
        assert f.shape == (self.rows[slot], L.NFLOW)
        self.ctx.check(self.lib.cfd_batch_set_flow(self.h, int(slot), C.c_void_p(_ptr(f))), "cfd_batch_set_flow")

    def set_wait_limit(self, limit_ns: int = -1):
        """Grid-barrier deadline in ns (< 0: the library default)."""
        self.ctx.check(self.lib.cfd_batch_set_wait_limit(self.h, int(limit_ns)), "cfd_batch_set_wait_limit")

    def set_tiling(self, tile_nodes: int = 0, max_blocks: int = 0, use_graph: bool = True):
        """tile_nodes: 64/128/256 (1-D tiles), abi.BATCH_FACE_TILES (shared-memory
        face tiles, mixed and split batches), 0 keeps the current choice."""
        self.ctx.check(self.lib.cfd_batch_set_tiling(self.h, int(tile_nodes), int(max_blocks), 1 if use_graph else 0),
                       "cfd_batch_set_tiling")

    def tune(self, steps_per_trial: int = 2):
        self.ctx.check(self.lib.cfd_batch_tune(self.h, int(steps_per_trial)), "cfd_batch_tune")

    def info(self) -> BatchInfo:
        i = abi.BatchInfo()
        self.ctx.check(self.lib.cfd_batch_info(self.h, C.byref(i)), "cfd_batch_info")
        return BatchInfo(i.n_active, i.tile_nodes, i.blocks, bool(i.graph), abi.PREC_NAMES[i.precision],
                         int(i.nodes_total), int(i.device_bytes), int(i.capacity_bytes), int(i.n_held),
                         bool(i.face_tiles))
