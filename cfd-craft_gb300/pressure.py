"""The pressure API of crates/cfd-craft/src/pressure.rs, served by the GB300 engine.

Same names, argument meanings and error behaviour as the reference:

    project(grid, u, p, dt, tol, max, control)        -> LinearInfo   (pressure.rs:469)
    solve_scaled(grid, b, scale, tol, max, control)   -> (x, LinearInfo) (pressure.rs:342)
    solve(grid, b, tol, max, control)                 -> (x, LinearInfo) (pressure.rs:329)
    apply(grid, x)                                    -> y            (pressure.rs:293)
    center_nullspaces(grid, x)                        (in place)      (pressure.rs:316)
    multigrid_stats(grid)                             -> dict | None  (pressure.rs:100)

Errors raise ``PressureError`` whose message is the reference's string
("CFD-E031: ...", "cancelled", ...); on error ``u`` and ``p`` are unchanged.
``grid`` is a :class:`grid.Grid`; its device state (topology, IC(0) factor,
multigrid hierarchy) is opened on first use and cached on the grid object, the
way the reference caches ``Grid::pressure_factor`` and the multigrid hierarchy.
"""
from __future__ import annotations

import atexit
import ctypes as C
import json
import threading
import time
import weakref
from dataclasses import dataclass

import numpy as np

from . import engine as E


class PressureError(RuntimeError):
    """A failed pressure solve; ``code`` is the engine's return code."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


@dataclass
class LinearInfo:
    """pressure.rs:30-36, plus the profile work counters of the solve."""

    iterations: int = 0
    relative_residual: float = 0.0
    work: dict = None


class Control:
    """solver::Control (solver.rs:75-188): cooperative cancellation and a wall-time limit.

    ``poll`` is an optional callable; raising or returning a string stops the solve
    as "cancelled" (or "wall_time_limit" when that is the text)."""

    def __init__(self, seconds: float = 1e9, poll=None):
        self.start = time.monotonic()
        self.limit = seconds
        self.cancelled = threading.Event()
        self.poll = poll
        self.polls = 0

    def check(self) -> int:
        self.polls += 1
        if self.poll is not None:
            try:
                r = self.poll()
            except Exception as e:  # an external poll error stops as cancelled
                r = str(e) or "cancelled"
            if r:
                return E.CFDG_WALL_TIME if r == "wall_time_limit" else E.CFDG_CANCELLED
        if self.cancelled.is_set():
            return E.CFDG_CANCELLED
        if time.monotonic() - self.start >= self.limit:
            return E.CFDG_WALL_TIME
        return 0


class Context:
    """One CUDA device with an HBM budget (cfdg_context)."""

    _default = None
    _lock = threading.Lock()

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0):
        L = E.load()
        h = C.c_void_p()
        rc = L.cfdg_context_create(device, hbm_budget_bytes, C.byref(h))
        if rc:
            raise PressureError(rc, E.last_error())
        self.h = h
        self.device = device

    @classmethod
    def default(cls) -> "Context":
        with cls._lock:
            if cls._default is None:
                cls._default = Context()
            return cls._default

    def close(self):
        h = getattr(self, "h", None)
        if h and E._lib is not None:
            E._lib.cfdg_context_destroy(h)
        self.h = None

    def __del__(self):
        self.close()


def _vp(a):
    return a.ctypes.data_as(C.c_void_p)


_open_grids = weakref.WeakSet()
_open_groups = weakref.WeakSet()  # batches and servers: closed before their grids and context


@atexit.register
def _close_all():
    # Release device state before the interpreter (and then the CUDA runtime) shut down:
    # batches and servers first (they use their grids' state), then grids, then contexts.
    for b in list(_open_groups):
        b.close()
    for dg in list(_open_grids):
        dg.close()
    if Context._default is not None:
        Context._default.close()
        Context._default = None


class DeviceGrid:
    """A grid opened on the engine (cfdg_grid): topology and caches resident in HBM."""

    def __init__(self, grid, ctx: Context = None, preconditioner: str = None, precision: str = "plain"):
        self.ctx = ctx or Context.default()
        L = E.load()
        self.grid = grid
        self._keep = dict(
            fluid=np.ascontiguousarray(grid.fluid, np.uint8),
            kind=np.ascontiguousarray(grid.face_kind, np.uint8),
            lo=np.ascontiguousarray(grid.face_lo, np.int64),
            hi=np.ascontiguousarray(grid.face_hi, np.int64),
            area=np.ascontiguousarray(grid.face_area, np.float64),
            dist=np.ascontiguousarray(grid.face_distance, np.float64),
            comp=np.ascontiguousarray(grid.component, np.int32),
            anch=np.ascontiguousarray(grid.anchored, np.uint8),
        )
        k = self._keep
        d = E.GridDesc()
        for a in range(3):
            d.n[a] = grid.n[a]
            d.dx[a] = grid.dx[a]
            d.periodic[a] = 1 if grid.periodic[a] else 0
        d.volume = grid.volume
        d.n_faces = grid.n_faces
        d.fluid, d.face_kind, d.face_lo, d.face_hi = _vp(k["fluid"]), _vp(k["kind"]), _vp(k["lo"]), _vp(k["hi"])
        d.face_area, d.face_distance = _vp(k["area"]), _vp(k["dist"])
        d.component, d.n_components = _vp(k["comp"]), grid.n_components
        d.anchored = _vp(k["anch"]) if grid.n_components else None
        d.preconditioner = E.PRECOND[preconditioner or grid.preconditioner]
        d.precision = E.PRECISION[precision]
        h = C.c_void_p()
        rc = L.cfdg_grid_open(self.ctx.h, C.byref(d), C.byref(h))
        if rc:
            raise PressureError(rc, E.last_error())
        self.h = h
        self.L = L
        _open_grids.add(self)

    def close(self):
        if getattr(self, "h", None):
            self.L.cfdg_grid_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def configure(self, preconditioner: str, precision: str = "plain"):
        self._check(self.L.cfdg_grid_configure(self.h, E.PRECOND[preconditioner], E.PRECISION[precision]))

    def update_faces(self, area=None, distance=None):
        a = None if area is None else np.ascontiguousarray(area, np.float64)
        d = None if distance is None else np.ascontiguousarray(distance, np.float64)
        self._check(self.L.cfdg_grid_update_faces(self.h, None if a is None else _vp(a), None if d is None else _vp(d)))

    def set_flow(self, case: dict):
        """The case's laminar flow terms for step_device (cfdg_grid_set_flow)."""
        bnd = {"periodic": 0, "open": 1, "wall": 2, "slip": 3, "ground_open_top": 4}
        flow = case["flow"]
        if flow["kind"] != "laminar":
            raise PressureError(E.CFDG_ERR_UNSUPPORTED, "laminar stepping: the case flow is not laminar")
        d = E.FlowDesc()
        for a in range(3):
            d.boundary[a] = bnd[case["boundaries"]["xyz"[a]]]
            d.size_m[a] = float(case["domain"]["size_m"][a])
            d.velocity[a] = float(flow.get("initial_velocity_m_s", [0.0, 0.0, 0.0])[a])
            d.acceleration[a] = float(flow.get("acceleration_m_s2", [0.0, 0.0, 0.0])[a])
        d.viscosity = float(flow.get("viscosity_m2_s", 1.5e-5))
        self._check(self.L.cfdg_grid_set_flow(self.h, C.byref(d)))

    def step_device(self, u_ptr: int, p_ptr: int, dt, tol, max_iter, control=None) -> LinearInfo:
        """One SSPRK2 step with a projection per stage, in place on device arrays (cfdg_step_device)."""
        info = E.Info()
        cb = self._poll_fn(control)
        rc = self.L.cfdg_step_device(self.h, C.c_void_p(u_ptr), C.c_void_p(p_ptr), float(dt), float(tol),
                                     int(max_iter), cb, None, C.byref(info))
        self._check(rc)
        return LinearInfo(info.iterations, info.relative_residual, info.as_dict())

    def scalar_step_budget(self, u_ptr: int, c_ptr: int, d_ptr: int, source_ptr: int, dt, budget_ptr: int):
        """The step and its budget increments (emitted, inflow, outflow in kg) into the three
        device doubles at budget_ptr (cfdg_scalar_step_budget)."""
        self._check(self.L.cfdg_scalar_step_budget(self.h, C.c_void_p(u_ptr), C.c_void_p(c_ptr), C.c_void_p(d_ptr),
                                                   C.c_void_p(source_ptr), float(dt), C.c_void_p(budget_ptr)))

    def set_advection(self, scheme: str):
        """Advection of the scalar steps and rates: "linear_upwind" or "muscl"
        (cfdg_grid_set_advection; transport.rs Advection)."""
        schemes = {"linear_upwind": 0, "muscl": 1}
        if scheme not in schemes:
            raise ValueError(f"advection is one of {sorted(schemes)}, not {scheme!r}")
        self._check(self.L.cfdg_grid_set_advection(self.h, schemes[scheme]))

    def scalar_rates(self, u_ptr: int, c_ptr: int, d_ptr: int, source_ptr: int):
        """(emitted, inflow, outflow) rates in kg/s of the device field at c_ptr (cfdg_scalar_rates)."""
        r = (C.c_double * 3)()
        self._check(self.L.cfdg_scalar_rates(self.h, C.c_void_p(u_ptr), C.c_void_p(c_ptr), C.c_void_p(d_ptr),
                                             C.c_void_p(source_ptr), r))
        return float(r[0]), float(r[1]), float(r[2])

    def scalar_step_device(self, u_ptr: int, c_ptr: int, d_ptr: int, source_ptr: int, dt):
        """One SSPRK2 step of a constituent on device arrays (cfdg_scalar_step_device)."""
        self._check(self.L.cfdg_scalar_step_device(self.h, C.c_void_p(u_ptr), C.c_void_p(c_ptr), C.c_void_p(d_ptr),
                                                   C.c_void_p(source_ptr), float(dt)))

    def set_receptors(self, weights):
        """Receptor weights for sample_receptors (cfdg_receptors_set): one list of
        (cell, weight) pairs per receptor, as receptors.receptor_weights returns them."""
        off = np.zeros(len(weights) + 1, dtype=np.int64)
        for r, w in enumerate(weights):
            off[r + 1] = off[r] + len(w)
        cells = np.array([c for w in weights for c, _ in w], dtype=np.int64)
        vals = np.array([v for w in weights for _, v in w], dtype=np.float64)
        self._check(self.L.cfdg_receptors_set(self.h, len(weights), _vp(off), _vp(cells), _vp(vals)))

    def sample_receptors(self, c_ptr: int, out_ptr: int):
        """The receptor values of the device concentration at c_ptr into out_ptr (device)."""
        self._check(self.L.cfdg_receptors_sample(self.h, C.c_void_p(c_ptr), C.c_void_p(out_ptr)))

    def momentum_update(self, u, p, dt):
        """u + dt (R(u) - grad p) with the fixed face values, before a stage's projection."""
        u = np.ascontiguousarray(u, np.float64)
        p = np.ascontiguousarray(p, np.float64)
        out = np.zeros_like(u)
        self._check(self.L.cfdg_debug_momentum_update(self.h, _vp(u), _vp(p), float(dt), _vp(out)))
        return out

    def set_cycle(self, nu_fine: int, nu_coarse: int):
        """Mixed form: V-cycle sweeps on level 0 and on the coarse levels (cfdg_grid_set_cycle)."""
        self._check(self.L.cfdg_grid_set_cycle(self.h, int(nu_fine), int(nu_coarse)))

    def set_sweep_tile(self, rows: int, stages: int):
        """Mixed form: rows per shared-memory stage (8, 16, 32) and stages in flight of the
        staged level-0 half sweeps (cfdg_grid_set_sweep_tile); results do not change."""
        self._check(self.L.cfdg_grid_set_sweep_tile(self.h, int(rows), int(stages)))

    def set_coarse_scale(self, alpha: float):
        """Mixed form: scale of the coarse corrections on aggregation hierarchies
        (cfdg_grid_set_coarse_scale; default 1.8, 1 is the reference's cycle)."""
        self._check(self.L.cfdg_grid_set_coarse_scale(self.h, float(alpha)))

    def set_coarse_layout(self, bins: bool):
        """Mixed form: the first coarse level as the 2x2x2 bin grid where the hierarchy
        allows it (True, the default) or in the aggregates' colour order (False); the same
        bits either way (cfdg_grid_set_coarse_layout)."""
        self._check(self.L.cfdg_grid_set_coarse_layout(self.h, 1 if bins else 0))

    def device_bytes(self) -> int:
        return int(self.L.cfdg_grid_device_bytes(self.h))

    def set_stream(self, stream_handle: int):
        """Enqueue on a caller's CUDA stream (an integer cudaStream_t; 0 = the grid's own)."""
        self._check(self.L.cfdg_grid_set_stream(self.h, C.c_void_p(stream_handle or None)))

    def project_device(self, u_ptr: int, p_ptr: int, dt, tol, max_iter, control=None) -> LinearInfo:
        """project() on device arrays (u: F doubles, p: N doubles) given as raw pointers."""
        info = E.Info()
        cb = self._poll_fn(control)
        rc = self.L.cfdg_project_device(self.h, C.c_void_p(u_ptr), C.c_void_p(p_ptr), float(dt), float(tol),
                                        int(max_iter), cb, None, C.byref(info))
        self._check(rc)
        return LinearInfo(info.iterations, info.relative_residual, info.as_dict())

    def time_kernel(self, which: int, reps: int = 20):
        """(ms per launch, algorithmic bytes) of one unit of work; see cfdg_debug_time_kernel."""
        ms, b = C.c_double(), C.c_double()
        self._check(self.L.cfdg_debug_time_kernel(self.h, which, reps, C.byref(ms), C.byref(b)))
        return ms.value, b.value

    def wave_stall(self, hold_tile: int = -1, spin_limit: int = 1 << 22):
        """Test hook of the bounded wavefront waits (cfdg_debug_wave_stall): tile hold_tile
        never publishes its progress and waits give up after spin_limit polls; (-1, 1 << 22)
        restores normal sweeps."""
        self._check(self.L.cfdg_debug_wave_stall(self.h, int(hold_tile), int(spin_limit)))

    def _check(self, rc):
        if rc:
            raise PressureError(rc, E.last_error())

    @staticmethod
    def _poll_fn(control):
        if control is None:
            return E.POLL(0)

        def cb(_ctx):
            c = control.check()
            return 0 if c == 0 else (2 if c == E.CFDG_WALL_TIME else 1)

        return E.POLL(cb)

    def project(self, u, p, dt, tol, max_iter, control=None) -> LinearInfo:
        assert u.dtype == np.float64 and u.flags.c_contiguous and u.size == self.grid.n_faces
        assert p.dtype == np.float64 and p.flags.c_contiguous and p.size == self.grid.count
        info = E.Info()
        cb = self._poll_fn(control)
        rc = self.L.cfdg_project(self.h, _vp(u), _vp(p), float(dt), float(tol), int(max_iter), cb, None,
                                 C.byref(info))
        self._check(rc)
        return LinearInfo(info.iterations, info.relative_residual, info.as_dict())

    def solve_scaled(self, b, scale, tol, max_iter, control=None):
        b = np.ascontiguousarray(b, np.float64)
        s = None if scale is None else np.ascontiguousarray(scale, np.float64)
        x = np.zeros(self.grid.count)
        info = E.Info()
        cb = self._poll_fn(control)
        rc = self.L.cfdg_solve_scaled(self.h, _vp(b), None if s is None else _vp(s), float(tol), int(max_iter), cb,
                                      None, _vp(x), C.byref(info))
        self._check(rc)
        return x, LinearInfo(info.iterations, info.relative_residual, info.as_dict())

    def apply(self, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.empty(self.grid.count)
        self._check(self.L.cfdg_apply(self.h, _vp(x), _vp(y)))
        return y

    def center_nullspaces(self, x):
        assert x.dtype == np.float64 and x.flags.c_contiguous
        self._check(self.L.cfdg_center_nullspaces(self.h, _vp(x)))

    def precondition(self, r):
        r = np.ascontiguousarray(r, np.float64)
        z = np.empty(self.grid.count)
        self._check(self.L.cfdg_debug_precondition(self.h, _vp(r), _vp(z)))
        return z

    def projection_rhs(self, u, dt):
        u = np.ascontiguousarray(u, np.float64)
        b = np.empty(self.grid.count)
        t = np.empty(self.grid.count)
        self._check(self.L.cfdg_debug_projection_rhs(self.h, _vp(u), float(dt), _vp(b), _vp(t)))
        return b, t

    def multigrid_stats(self):
        buf = C.create_string_buffer(1 << 16)
        rc = self.L.cfdg_multigrid_stats_json(self.h, buf, len(buf))
        if rc == E.CFDG_PENDING:
            return None
        self._check(rc)
        return json.loads(buf.value.decode())


def device_grid(grid) -> DeviceGrid:
    """The grid's engine handle, opened on first use (like Grid::pressure_factor's OnceLock)."""
    dg = getattr(grid, "_device", None)
    if dg is None:
        dg = DeviceGrid(grid)
        object.__setattr__(grid, "_device", dg)
    return dg


def project(grid, u, p, dt, tol, max_iter, control=None) -> LinearInfo:
    return device_grid(grid).project(u, p, dt, tol, max_iter, control)


def solve_scaled(grid, b, roundoff_scale, tol, max_iter, control=None):
    return device_grid(grid).solve_scaled(b, roundoff_scale, tol, max_iter, control)


def solve(grid, b, tol, max_iter, control=None):
    return device_grid(grid).solve_scaled(b, None, tol, max_iter, control)


def apply(grid, x):
    return device_grid(grid).apply(x)


def center_nullspaces(grid, x):
    device_grid(grid).center_nullspaces(x)


def multigrid_stats(grid):
    return device_grid(grid).multigrid_stats()


class Batch:
    """Several grids projected together in the mixed form (cfdg_batch).

    ``project(us, ps, dts, tol, max)`` returns one (code, LinearInfo) per case; a case
    with a nonzero code keeps its inputs unchanged."""

    def __init__(self, device_grids, ctx: Context = None):
        self.ctx = ctx or device_grids[0].ctx
        self.grids = list(device_grids)
        L = E.load()
        arr = (C.c_void_p * len(self.grids))(*[g.h for g in self.grids])
        h = C.c_void_p()
        rc = L.cfdg_batch_create(self.ctx.h, arr, len(self.grids), C.byref(h))
        if rc:
            raise PressureError(rc, E.last_error())
        self.h = h
        self.L = L
        _open_groups.add(self)

    def close(self):
        if getattr(self, "h", None):
            self.L.cfdg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle: int):
        rc = self.L.cfdg_batch_set_stream(self.h, C.c_void_p(stream_handle or None))
        if rc:
            raise PressureError(rc, E.last_error())

    def _run(self, fn, us, ps, dts, tol, max_iter, control):
        n = len(self.grids)
        ua = (C.c_void_p * n)(*us)
        pa = (C.c_void_p * n)(*ps)
        da = (C.c_double * n)(*[float(d) for d in dts])
        infos = (E.Info * n)()
        codes = (C.c_int32 * n)()
        cb = DeviceGrid._poll_fn(control)
        rc = fn(self.h, ua, pa, da, float(tol), int(max_iter), cb, None, infos, codes)
        if rc:
            raise PressureError(rc, E.last_error())
        return [(int(codes[i]), LinearInfo(infos[i].iterations, infos[i].relative_residual, infos[i].as_dict()))
                for i in range(n)]

    def project(self, us, ps, dts, tol, max_iter, control=None):
        for u, p, g in zip(us, ps, self.grids):
            assert u.dtype == np.float64 and u.flags.c_contiguous and u.size == g.grid.n_faces
            assert p.dtype == np.float64 and p.flags.c_contiguous and p.size == g.grid.count
        return self._run(self.L.cfdg_batch_project, [u.ctypes.data for u in us], [p.ctypes.data for p in ps], dts,
                         tol, max_iter, control)

    def project_device(self, u_ptrs, p_ptrs, dts, tol, max_iter, control=None):
        return self._run(self.L.cfdg_batch_project_device, u_ptrs, p_ptrs, dts, tol, max_iter, control)

    def stats(self) -> dict:
        """Per case and coarse level: rows, nonzeros, colours, ELL entries, groups, blocks."""
        import json

        n = self.L.cfdg_batch_stats_json(self.h, None, 0)
        if n < 0:
            raise PressureError(int(-n), E.last_error())
        buf = C.create_string_buffer(int(n))
        self.L.cfdg_batch_stats_json(self.h, buf, int(n))
        return json.loads(buf.value.decode())

    def time_kernel(self, which: int, reps: int = 20):
        """(ms per launch, algorithmic bytes); see cfdg_batch_time_kernel."""
        ms, b = C.c_double(), C.c_double()
        rc = self.L.cfdg_batch_time_kernel(self.h, which, reps, C.byref(ms), C.byref(b))
        if rc:
            raise PressureError(rc, E.last_error())
        return ms.value, b.value

    def debug_rhs(self, c: int, n_cells: int):
        """(b, terms) of case c's last projection (cfdg_batch_debug_rhs)."""
        b, t = np.empty(n_cells), np.empty(n_cells)
        rc = self.L.cfdg_batch_debug_rhs(self.h, int(c), _vp(b), _vp(t))
        if rc:
            raise PressureError(rc, E.last_error())
        return b, t


class Server:
    """Continuous-batching projection server over resident grids (cfdg_server)."""

    def __init__(self, device_grids, max_active: int, ctx: Context = None):
        self.ctx = ctx or device_grids[0].ctx
        self.grids = list(device_grids)
        L = E.load()
        arr = (C.c_void_p * len(self.grids))(*[g.h for g in self.grids])
        h = C.c_void_p()
        rc = L.cfdg_server_create(self.ctx.h, arr, len(self.grids), int(max_active), C.byref(h))
        if rc:
            raise PressureError(rc, E.last_error())
        self.h = h
        self.L = L
        _open_groups.add(self)

    def close(self):
        if getattr(self, "h", None):
            self.L.cfdg_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc:
            raise PressureError(rc, E.last_error())

    def set_stream(self, stream_handle: int):
        self._check(self.L.cfdg_server_set_stream(self.h, C.c_void_p(stream_handle or None)))

    def submit(self, grid_index: int, u_ptr: int, p_ptr: int, dt, tol, max_iter) -> int:
        t = C.c_uint64()
        self._check(self.L.cfdg_server_submit(self.h, int(grid_index), C.c_void_p(u_ptr), C.c_void_p(p_ptr),
                                              float(dt), float(tol), int(max_iter), C.byref(t)))
        return t.value

    def submit_host(self, grid_index: int, u_ptr: int, p_ptr: int, u_out_ptr: int, p_out_ptr: int, dt, tol,
                    max_iter) -> int:
        """Queues pressure::project of grid `grid_index` on host buffers given as raw pointers
        (cfdg_server_submit_host): u (F doubles) and p (N doubles) in, the projected fields
        (or the unchanged inputs on failure) into u_out and p_out before the ticket reports
        done. Page-locked buffers let the copies overlap the solves."""
        t = C.c_uint64()
        self._check(self.L.cfdg_server_submit_host(self.h, int(grid_index), C.c_void_p(u_ptr), C.c_void_p(p_ptr),
                                                   C.c_void_p(u_out_ptr), C.c_void_p(p_out_ptr), float(dt),
                                                   float(tol), int(max_iter), C.byref(t)))
        return t.value

    def set_chunk(self, iterations: int):
        """Iterations per graph chunk (cfdg_server_set_chunk)."""
        self._check(self.L.cfdg_server_set_chunk(self.h, int(iterations)))

    def progress(self) -> int:
        n = C.c_int32()
        self._check(self.L.cfdg_server_progress(self.h, C.byref(n)))
        return n.value

    def result(self, ticket: int):
        """(code, LinearInfo) when finished, None while pending."""
        info = E.Info()
        code = C.c_int32()
        rc = self.L.cfdg_server_result(self.h, int(ticket), C.byref(info), C.byref(code))
        if rc == E.CFDG_PENDING:
            return None
        self._check(rc)
        return int(code.value), LinearInfo(info.iterations, info.relative_residual, info.as_dict())

    def pending(self) -> int:
        return int(self.L.cfdg_server_pending(self.h))

    def stats(self) -> dict:
        """Rounds, chunks, chunk device ms, progress host ms, finished, admitted."""
        import json

        n = self.L.cfdg_server_stats_json(self.h, None, 0)
        if n < 0:
            raise PressureError(int(-n), E.last_error())
        buf = C.create_string_buffer(int(n))
        self.L.cfdg_server_stats_json(self.h, buf, int(n))
        return json.loads(buf.value.decode())


# Candidate (level-0 sweeps, coarse-level sweeps) pairs of the mixed form's V-cycle.
# (sweeps on level 0, sweeps on the coarse levels, coarse-correction scale)
CYCLE_CANDIDATES = ((1, 2, 1.85), (2, 1, 1.85), (2, 2, 1.7), (2, 2, 1.85), (2, 3, 1.85), (3, 2, 1.85))
# Tile shapes of the staged level-0 half sweeps: (rows per shared-memory stage, stages in flight).
SWEEP_TILE_CANDIDATES = ((8, 4), (16, 2), (16, 3), (16, 4), (32, 2), (32, 3))


def autotune_sweep_tile(device_grids, u_ptrs, p_ptrs, reset, dts, tol=1e-8, max_iter=10000,
                        candidates=SWEEP_TILE_CANDIDATES, stream_handle=None, reps=20):
    """Picks the tile shape of the staged level-0 half sweeps (cfdg_grid_set_sweep_tile) with
    the shortest kernel time on these grids and applies it. Taller stages halve the y-halo
    rows per stage and the copies per byte; more stages keep more bytes in flight but hold
    more shared memory, so fewer blocks fit an SM. The best shape depends on the row lengths
    of the mix, which is why it is measured: for each candidate a batch of all grids
    projects once (the inputs restored by `reset()`), then one half sweep over every case is
    timed `reps` times with CUDA events. Results do not depend on the shape, bit for bit.
    Returns {"choice": [rows, stages], "us": {...}}, or None when the mix does not take the
    staged path (non-uniform weights, or ceil(nx/2) not a multiple of 8)."""
    probe = Batch(device_grids)
    try:
        if not probe.stats()["staged_sweeps"]:
            return None
    finally:
        probe.close()
    timing = {}
    for cand in candidates:
        for d in device_grids:
            d.set_sweep_tile(*cand)
        b = Batch(device_grids)
        if stream_handle:
            b.set_stream(stream_handle)
        try:
            reset()
            if any(code != 0 for code, _ in b.project_device(u_ptrs, p_ptrs, dts, tol, max_iter)):
                continue
            timing[cand] = b.time_kernel(0, reps)[0]
        finally:
            b.close()
    if not timing:
        return None
    choice = min(timing, key=timing.get)
    for d in device_grids:
        d.set_sweep_tile(*choice)
    reset()
    return {"choice": list(choice), "us": {f"{r}x{n}": round(1e3 * t, 2) for (r, n), t in timing.items()}}


def autotune(device_grids, u_ptrs, p_ptrs, reset, dts, tol=1e-8, max_iter=10000, candidates=CYCLE_CANDIDATES,
             stream_handle=None):
    """Picks the mixed form's V-cycle sweep counts and coarse-correction scale with the
    shortest time to `tol` on these grids and applies them (cfdg_grid_set_cycle,
    cfdg_grid_set_coarse_scale; a candidate without a scale keeps the grids' own).

    For each candidate a batch of all the grids projects the device velocities u_ptrs /
    p_ptrs twice (the first call builds the batch's graph and is not timed); `reset()`
    restores the inputs before every call. More sweeps make a cycle dearer and the
    iteration count smaller; the optimum depends on the case mix (stencil anisotropy,
    buildings, the share of wide-stencil coarse levels), which is why it is measured.
    The tile shape of the staged half sweeps is picked first (autotune_sweep_tile).
    Returns {"choice": [nu_fine, nu_coarse(, scale)], "ms": {...}, "iterations": {...},
    "sweep_tile": {...} | None}."""
    import time

    tile = autotune_sweep_tile(device_grids, u_ptrs, p_ptrs, reset, dts, tol, max_iter, stream_handle=stream_handle)
    timing, iters = {}, {}
    def apply(cand):
        for d in device_grids:
            d.set_cycle(cand[0], cand[1])
            if len(cand) > 2:
                d.set_coarse_scale(cand[2])

    for cand in candidates:
        apply(cand)
        b = Batch(device_grids)
        if stream_handle:
            b.set_stream(stream_handle)
        try:
            best = None
            for rep in range(2):
                reset()
                t0 = time.perf_counter()
                res = b.project_device(u_ptrs, p_ptrs, dts, tol, max_iter)
                dt_s = time.perf_counter() - t0
                if any(code != 0 for code, _ in res):
                    best = None
                    break
                if rep:
                    best = dt_s
                    iters[cand] = sum(i.iterations for _, i in res) / len(res)
        finally:
            b.close()
        if best is not None:
            timing[cand] = best
    if not timing:
        raise PressureError(E.CFDG_ERR_INVALID, "no candidate cycle converged")
    choice = min(timing, key=timing.get)
    apply(choice)
    reset()

    def key(c):
        return ",".join(str(v) for v in c)

    return {"choice": list(choice), "ms": {key(c): round(1e3 * t, 2) for c, t in timing.items()},
            "iterations": {key(c): round(v, 2) for c, v in iters.items()}, "sweep_tile": tile}
