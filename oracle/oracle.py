"""ctypes wrapper of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference legs
use this module. It loads ``oracle/_build/libcfd_oracle.so`` (built by
``oracle/Makefile``), a plain C++ restatement of the CFD-craft pressure
projection (crates/cfd-craft/src/grid.rs, pressure.rs, multigrid.rs,
multigrid/masked.rs, multigrid/line.rs) and of the steps around it (flow.rs laminar
momentum, transport.rs scalar transport). Cases are reference-schema case dictionaries
(``cfd-craft.case/0.1``); only the fields the projection reads are used.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libcfd_oracle.so")

BOUNDARY = {"periodic": 0, "open": 1, "wall": 2, "slip": 3, "ground_open_top": 4}
FLOW = {"prescribed_uniform": 0, "laminar": 1, "neutral_rans": 2}
PRECONDITIONER = {"ic0": 0, "multigrid": 1}
# Return codes (shared with the engine's C ABI).
OK, E031, E032, E033, E034, E035, CANCELLED, WALL_TIME, UNSUPPORTED = 0, 31, 32, 33, 34, 35, 100, 101, 299


class _Case(C.Structure):
    _fields_ = [
        ("n", C.c_int32 * 3),
        ("size_m", C.c_double * 3),
        ("boundary", C.c_int32 * 3),
        ("flow_kind", C.c_int32),
        ("velocity", C.c_double * 3),
        ("speed_m_s", C.c_double),
        ("reference_height_m", C.c_double),
        ("roughness_m", C.c_double),
        ("direction_deg_from", C.c_double),
        ("n_boxes", C.c_int32),
        ("boxes", C.POINTER(C.c_double)),
        ("preconditioner", C.c_int32),
    ]


class Info(C.Structure):
    _fields_ = [
        ("iterations", C.c_uint64),
        ("relative_residual", C.c_double),
        ("work_units", C.c_uint64),
        ("operator_applications", C.c_uint64),
        ("preconditioner_applications", C.c_uint64),
        ("true_residual_checks", C.c_uint64),
        ("hierarchy_builds", C.c_uint64),
        ("hierarchy_levels", C.c_uint64),
        ("hierarchy_cells", C.c_uint64),
        ("hierarchy_nonzeros", C.c_uint64),
        ("cycles", C.c_uint64),
        ("smoothing_cell_updates", C.c_uint64),
        ("residual_cell_updates", C.c_uint64),
        ("restriction_cell_updates", C.c_uint64),
        ("prolongation_cell_updates", C.c_uint64),
        ("coarse_solves", C.c_uint64),
        ("polls", C.c_uint64),
        ("block_smoothing_cell_updates", C.c_uint64),
        ("block_solves", C.c_uint64),
        ("block_level_cell_visits", C.c_uint64),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


POLL = C.CFUNCTYPE(C.c_int, C.c_void_p)
_lock = threading.Lock()
_lib = None


def build():
    """Compiles the oracle library with its Makefile (idempotent)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                build()
            L = C.CDLL(LIB_PATH)
            P = C.c_void_p
            dp = C.POINTER(C.c_double)
            L.ora_grid_build.restype = P
            L.ora_grid_build.argtypes = [C.POINTER(_Case), C.c_char_p, C.c_size_t]
            L.ora_grid_free.argtypes = [P]
            L.ora_grid_set_preconditioner.argtypes = [P, C.c_int32]
            L.ora_grid_counts.argtypes = [P, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
            L.ora_grid_export.argtypes = [P] + [C.c_void_p] * 11
            L.ora_grid_set_faces.argtypes = [P, C.c_void_p, C.c_void_p]
            L.ora_project.restype = C.c_int32
            L.ora_project.argtypes = [P, dp, dp, C.c_double, C.c_double, C.c_uint64, POLL, C.c_void_p, C.POINTER(Info)]
            L.ora_solve_scaled.restype = C.c_int32
            L.ora_solve_scaled.argtypes = [P, dp, C.c_void_p, C.c_double, C.c_uint64, POLL, C.c_void_p, dp, C.POINTER(Info)]
            for name in ("ora_apply", "ora_operator_apply", "ora_divergence", "ora_gradient", "ora_ic0_apply"):
                getattr(L, name).argtypes = [P, dp, dp]
            L.ora_center_nullspaces.argtypes = [P, dp]
            L.ora_enforce_velocity.argtypes = [P, dp]
            L.ora_projection_rhs.argtypes = [P, dp, C.c_double, dp, dp]
            L.ora_ic0_nnz.restype = C.c_int64
            L.ora_ic0_nnz.argtypes = [P]
            L.ora_ic0_export.argtypes = [P, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
            L.ora_mg_apply.restype = C.c_int32
            L.ora_mg_apply.argtypes = [P, dp, dp, C.POINTER(Info)]
            L.ora_mg_levels.restype = C.c_int32
            L.ora_mg_levels.argtypes = [P, C.c_void_p, C.c_void_p, C.c_int32]
            L.ora_mg_dims.restype = C.c_int32
            L.ora_mg_dims.argtypes = [P, C.c_void_p, C.c_int32]
            L.ora_mg_blocks.restype = C.c_int32
            L.ora_mg_blocks.argtypes = [P, C.c_void_p, C.c_int32]
            L.ora_mg_level_dense.restype = C.c_int64
            L.ora_mg_level_dense.argtypes = [P, C.c_int32, C.c_void_p, C.c_void_p]
            L.ora_mg_transfer_dense.restype = C.c_int64
            L.ora_mg_transfer_dense.argtypes = [P, C.c_int32, C.c_void_p]
            L.ora_block_sweep.argtypes = [P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]
            L.ora_mg_masked_level.restype = C.c_int64
            L.ora_mg_masked_level.argtypes = [P, C.c_int32] + [C.c_void_p] * 6
            L.ora_grid_set_flow_terms.argtypes = [P, C.c_double, dp]
            L.ora_momentum_rhs.restype = C.c_int32
            L.ora_momentum_rhs.argtypes = [P, dp, dp]
            L.ora_scalar_step.argtypes = [P, dp, dp, dp, dp, C.c_double, C.c_void_p]
            L.ora_scalar_rates.argtypes = [P, dp, dp, dp, dp, dp, C.c_int32]
            L.ora_scalar_step_adv.argtypes = [P, dp, dp, dp, dp, C.c_double, C.c_void_p, C.c_int32]
            L.ora_step.restype = C.c_int32
            L.ora_step.argtypes = [P, dp, dp, C.c_double, C.c_double, C.c_uint64, C.POINTER(C.c_uint64)]
            _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _vp(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class OracleError(RuntimeError):
    def __init__(self, code, message=""):
        super().__init__(f"oracle error {code}: {message}")
        self.code = code


class Grid:
    """Oracle grid built from a reference-schema case dict (grid.rs:246-464)."""

    def __init__(self, case: dict):
        L = lib()
        c = _Case()
        n = case["grid"]["cells"]
        size = case["domain"]["size_m"]
        b = case["boundaries"]
        flow = case["flow"]
        for a in range(3):
            c.n[a] = int(n[a])
            c.size_m[a] = float(size[a])
            c.boundary[a] = BOUNDARY[b["xyz"[a]]]
        c.flow_kind = FLOW[flow["kind"]]
        vel = flow.get("initial_velocity_m_s", flow.get("velocity_m_s", [0.0, 0.0, 0.0]))
        for a in range(3):
            c.velocity[a] = float(vel[a])
        c.speed_m_s = float(flow.get("speed_m_s", 0.0))
        c.reference_height_m = float(flow.get("reference_height_m", 1.0))
        c.roughness_m = float(flow.get("roughness_m", 0.1))
        c.direction_deg_from = float(flow.get("direction_deg_from", 0.0))
        boxes = []
        for g in case.get("geometry", []):
            if g.get("footprint_m") is not None:
                raise ValueError("the oracle restates boxes only")
            boxes.extend([float(v) for v in g["min_m"]] + [float(v) for v in g["max_m"]])
        self._boxes = np.ascontiguousarray(boxes, dtype=np.float64)
        c.n_boxes = len(boxes) // 6
        c.boxes = _ptr(self._boxes) if len(boxes) else None
        c.preconditioner = PRECONDITIONER[case.get("numerics", {}).get("pressure_preconditioner", "ic0")]
        err = C.create_string_buffer(512)
        h = L.ora_grid_build(C.byref(c), err, 512)
        if not h:
            raise OracleError(-1, err.value.decode())
        self.h = C.c_void_p(h)
        self.n = tuple(int(v) for v in n)
        cells, faces, comps = C.c_int64(), C.c_int64(), C.c_int64()
        L.ora_grid_counts(self.h, C.byref(cells), C.byref(faces), C.byref(comps))
        self.count, self.n_faces, self.n_components = cells.value, faces.value, comps.value
        N, F = self.count, self.n_faces
        self.fluid = np.zeros(N, np.uint8)
        self.face_kind = np.zeros(F, np.uint8)
        self.face_lo = np.zeros(F, np.int64)
        self.face_hi = np.zeros(F, np.int64)
        self.face_area = np.zeros(F, np.float64)
        self.face_distance = np.zeros(F, np.float64)
        self.component = np.zeros(N, np.int32)
        self.anchored = np.zeros(max(self.n_components, 1), np.uint8)[: self.n_components]
        self.cell_faces = np.zeros((N, 6), np.int64)
        self.face_center = np.zeros((F, 3), np.float64)
        self.face_axis = np.zeros(F, np.uint8)
        L.ora_grid_export(self.h, _vp(self.fluid), _vp(self.face_kind), _vp(self.face_lo), _vp(self.face_hi),
                          _vp(self.face_area), _vp(self.face_distance), _vp(self.component), _vp(self.anchored),
                          _vp(self.cell_faces), _vp(self.face_center), _vp(self.face_axis))
        acc = np.ascontiguousarray(flow.get("acceleration_m_s2", [0.0, 0.0, 0.0]), dtype=np.float64)
        L.ora_grid_set_flow_terms(self.h, float(flow.get("viscosity_m2_s", 1.5e-5)), _ptr(acc))

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and _lib is not None:
            _lib.ora_grid_free(h)
            self.h = None

    def momentum_rhs(self, u):
        """flow::momentum_rhs for laminar flow (flow.rs:426-525), per face."""
        u = np.ascontiguousarray(u, np.float64)
        out = np.zeros(self.n_faces)
        code = lib().ora_momentum_rhs(self.h, _ptr(u), _ptr(out))
        if code:
            raise OracleError(code, "momentum_rhs")
        return out

    def step(self, u, p, dt, tol=1e-8, max_iter=10000):
        """One SSPRK2 step of laminar flow with a projection per stage (solver.rs:879-960).
        Returns (code, u, p, pressure iterations)."""
        uu = np.array(u, dtype=np.float64, copy=True)
        pp = np.array(p, dtype=np.float64, copy=True)
        it = C.c_uint64()
        code = lib().ora_step(self.h, _ptr(uu), _ptr(pp), float(dt), float(tol), int(max_iter), C.byref(it))
        return code, uu, pp, it.value

    def scalar_step(self, c, u, d, source, dt, budget=None, muscl=False):
        """advance_scalar (solver.rs:808-855): one SSPRK2 step of a constituent, linear upwind
        or (muscl) MUSCL with the monotonized-central limiter (transport.rs:502-526,670-694).
        `budget` (a float64 array of 3, optional) accumulates the emitted, inflow and outflow
        masses in kg as solver.rs:851-853 does."""
        cc = np.array(c, dtype=np.float64, copy=True)
        bp = None
        if budget is not None:
            assert budget.dtype == np.float64 and budget.shape == (3,) and budget.flags.c_contiguous
            bp = budget.ctypes.data_as(C.c_void_p)
        lib().ora_scalar_step_adv(self.h, _ptr(cc), _ptr(np.ascontiguousarray(u, np.float64)),
                                  _ptr(np.ascontiguousarray(d, np.float64)),
                                  _ptr(np.ascontiguousarray(source, np.float64)), float(dt), bp, 1 if muscl else 0)
        return cc

    def scalar_rates(self, c, u, d, source, muscl=False):
        """(emitted, inflow, outflow) in kg/s of the field c: the rates rhs_into returns
        (transport.rs:651-699)."""
        out = np.zeros(3)
        lib().ora_scalar_rates(self.h, _ptr(np.ascontiguousarray(c, np.float64)),
                               _ptr(np.ascontiguousarray(u, np.float64)), _ptr(np.ascontiguousarray(d, np.float64)),
                               _ptr(np.ascontiguousarray(source, np.float64)), _ptr(out), 1 if muscl else 0)
        return float(out[0]), float(out[1]), float(out[2])

    def set_preconditioner(self, name):
        lib().ora_grid_set_preconditioner(self.h, PRECONDITIONER[name])

    def set_faces(self, area=None, distance=None):
        if area is not None:
            self.face_area = np.ascontiguousarray(area, dtype=np.float64)
        if distance is not None:
            self.face_distance = np.ascontiguousarray(distance, dtype=np.float64)
        lib().ora_grid_set_faces(self.h, _vp(self.face_area), _vp(self.face_distance))

    def _vec(self, x, n):
        x = np.ascontiguousarray(x, dtype=np.float64)
        assert x.shape == (n,)
        return x

    def apply(self, x):
        x = self._vec(x, self.count)
        y = np.empty(self.count)
        lib().ora_apply(self.h, _ptr(x), _ptr(y))
        return y

    def operator_apply(self, x):
        x = self._vec(x, self.count)
        y = np.empty(self.count)
        lib().ora_operator_apply(self.h, _ptr(x), _ptr(y))
        return y

    def divergence(self, u):
        u = self._vec(u, self.n_faces)
        y = np.empty(self.count)
        lib().ora_divergence(self.h, _ptr(u), _ptr(y))
        return y

    def gradient(self, p):
        p = self._vec(p, self.count)
        y = np.empty(self.n_faces)
        lib().ora_gradient(self.h, _ptr(p), _ptr(y))
        return y

    def enforce_velocity(self, u):
        u = np.array(u, dtype=np.float64, copy=True)
        lib().ora_enforce_velocity(self.h, _ptr(u))
        return u

    def center_nullspaces(self, x):
        x = np.array(x, dtype=np.float64, copy=True)
        lib().ora_center_nullspaces(self.h, _ptr(x))
        return x

    def projection_rhs(self, u, dt):
        u = self._vec(u, self.n_faces)
        b = np.empty(self.count)
        t = np.empty(self.count)
        lib().ora_projection_rhs(self.h, _ptr(u), float(dt), _ptr(b), _ptr(t))
        return b, t

    def ic0_apply(self, r):
        r = self._vec(r, self.count)
        z = np.zeros(self.count)
        lib().ora_ic0_apply(self.h, _ptr(r), _ptr(z))
        return z

    def ic0_factor(self):
        L = lib()
        nnz = L.ora_ic0_nnz(self.h)
        ro = np.zeros(self.count + 1, np.int64)
        cols = np.zeros(nnz, np.int64)
        lower = np.zeros(nnz)
        diag = np.zeros(self.count)
        L.ora_ic0_export(self.h, _vp(ro), _vp(cols), _vp(lower), _vp(diag))
        return ro, cols, lower, diag

    def mg_apply(self, r):
        r = self._vec(r, self.count)
        z = np.zeros(self.count)
        info = Info()
        code = lib().ora_mg_apply(self.h, _ptr(r), _ptr(z), C.byref(info))
        if code:
            raise OracleError(code)
        return z, info.as_dict()

    def mg_level_dense(self, level):
        """(dims, dense matrix) of an unmasked hierarchy level (after a build)."""
        dims = np.zeros(3, np.int64)
        n = lib().ora_mg_level_dense(self.h, int(level), _vp(dims), None)
        if n < 0:
            raise OracleError(-1)
        a = np.zeros((n, n))
        lib().ora_mg_level_dense(self.h, int(level), _vp(dims), _vp(a))
        return tuple(int(v) for v in dims), a

    def mg_transfer_dense(self, level):
        """The prolongation of an unmasked level to the next one, dense (n x nc)."""
        nc = lib().ora_mg_transfer_dense(self.h, int(level), None)
        if nc < 0:
            raise OracleError(-1)
        n = self.mg_level_dense(level)[1].shape[0]
        p = np.zeros((n, nc))
        lib().ora_mg_transfer_dense(self.h, int(level), _vp(p))
        return p

    def block_sweep(self, level, axes, periodic, backward, rhs, x):
        """One block Gauss-Seidel sweep (multigrid/line.rs) over `axes` on a level's matrix."""
        rhs = np.ascontiguousarray(rhs, np.float64)
        xx = np.array(x, dtype=np.float64, copy=True)
        mask = sum(1 << a for a in axes)
        pmask = sum(1 << a for a in range(3) if periodic[a])
        code = lib().ora_block_sweep(self.h, int(level), mask, pmask, int(bool(backward)), _vp(rhs), _vp(xx))
        if code:
            raise OracleError(code)
        return xx

    def block_bandwidth(self, level, axes, periodic):
        """Half-bandwidth of the block factor a block smoother over `axes` gets on a level."""
        mask = sum(1 << a for a in axes)
        pmask = sum(1 << a for a in range(3) if periodic[a])
        code = lib().ora_block_sweep(self.h, int(level), mask, pmask, 0, None, None)
        if code > -1000:
            raise OracleError(code)
        return -code - 1000

    def mg_levels(self):
        cells = np.zeros(64, np.uint64)
        nz = np.zeros(64, np.uint64)
        L = lib().ora_mg_levels(self.h, _vp(cells), _vp(nz), 64)
        return [int(v) for v in cells[:L]], [int(v) for v in nz[:L]]

    def mg_stats(self):
        """MultigridStats (multigrid.rs:55-72) of the current hierarchy without the storage
        bytes: level_cells, level_nonzeros, level_dimensions (unmasked hierarchies; empty
        for masked ones) and block_smoothers (level, axes, block_unknowns, block_count,
        half_bandwidth)."""
        cells, nz = self.mg_levels()
        dims = np.zeros(3 * 64, np.int64)
        nd = lib().ora_mg_dims(self.h, _vp(dims), 64)
        blk = np.zeros(5 * 256, np.int64)
        nb = lib().ora_mg_blocks(self.h, _vp(blk), 256)
        smoothers = []
        for s_ in range(min(nb, 256)):
            lv, mask, unk, cnt, bw = (int(v) for v in blk[5 * s_:5 * s_ + 5])
            smoothers.append({"level": lv, "axes": [a for a in range(3) if mask >> a & 1], "block_unknowns": unk,
                              "block_count": cnt, "half_bandwidth": bw})
        return {"level_cells": cells, "level_nonzeros": nz,
                "level_dimensions": [[int(v) for v in dims[3 * i:3 * i + 3]] for i in range(nd)],
                "block_smoothers": smoothers}

    def mg_masked_level(self, level):
        L = lib()
        nnz = C.c_int64()
        n = L.ora_mg_masked_level(self.h, level, None, None, None, None, None, C.byref(nnz))
        if n < 0:
            return None
        parent = np.zeros(n, np.int64)
        off = np.zeros(n + 1, np.int64)
        cols = np.zeros(nnz.value, np.int64)
        vals = np.zeros(nnz.value)
        diag = np.zeros(n)
        L.ora_mg_masked_level(self.h, level, _vp(parent), _vp(off), _vp(cols), _vp(vals), _vp(diag), None)
        return dict(parent=parent, offsets=off, columns=cols, values=vals, diagonal=diag)

    def solve_scaled(self, b, terms=None, tol=1e-8, max_iter=10000, poll=None):
        b = self._vec(b, self.count)
        if terms is not None:
            terms = self._vec(terms, self.count)
        x = np.zeros(self.count)
        info = Info()
        cb = POLL(poll) if poll else POLL(0)
        code = lib().ora_solve_scaled(self.h, _ptr(b), _vp(terms), tol, int(max_iter), cb, None, _ptr(x),
                                      C.byref(info))
        return code, x, info.as_dict()

    def solve(self, b, tol=1e-8, max_iter=10000, poll=None):
        return self.solve_scaled(b, None, tol, max_iter, poll)

    def project(self, u, p, dt, tol=1e-8, max_iter=10000, poll=None):
        """Returns (code, u', p', info); inputs are not modified."""
        u = np.array(u, dtype=np.float64, copy=True)
        p = np.array(p, dtype=np.float64, copy=True)
        assert u.shape == (self.n_faces,) and p.shape == (self.count,)
        info = Info()
        cb = POLL(poll) if poll else POLL(0)
        code = lib().ora_project(self.h, _ptr(u), _ptr(p), float(dt), tol, int(max_iter), cb, None, C.byref(info))
        return code, u, p, info.as_dict()

    def centers(self):
        """Cell centres (N, 3) in metres: (q + 0.5) * dx."""
        nx, ny, nz = self.n
        idx = np.arange(self.count)
        q = np.stack([idx % nx, idx // nx % ny, idx // (nx * ny)], axis=1).astype(np.float64)
        return q


def manufactured_rhs(grid: Grid, case: dict):
    """performance_probe.rs:83-95: exact = sin(2 pi x/Lx) + 0.3 cos(4 pi z/Lz) on fluid cells,
    gauge-centred, and its operator image. Returns (exact, rhs)."""
    nx, ny, nz = grid.n
    size = case["domain"]["size_m"]
    dx = [size[a] / grid.n[a] for a in range(3)]
    idx = np.arange(grid.count)
    x = ((idx % nx).astype(np.float64) + 0.5) * dx[0]
    z = ((idx // (nx * ny)).astype(np.float64) + 0.5) * dx[2]
    # math.sin/cos are the C library's (the functions Rust's f64::sin/cos call on Linux).
    exact = np.array([math.sin(2.0 * math.pi * xv / size[0]) + 0.3 * math.cos(4.0 * math.pi * zv / size[2])
                      for xv, zv in zip(x.tolist(), z.tolist())])
    exact[grid.fluid == 0] = 0.0
    exact = grid.center_nullspaces(exact)
    return exact, grid.apply(exact)
