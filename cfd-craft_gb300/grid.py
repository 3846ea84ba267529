"""The staggered grid of a case, restated with numpy (crates/cfd-craft/src/grid.rs).

``Grid.build(case)`` turns a reference-schema case dictionary into the arrays the
engine's C ABI takes (cfdg_grid_desc): the solid mask, the face list (x-faces, then
y, then z, each x fastest), face kinds, cells and coefficients, and the fluid
components with their anchoring. It follows ``Grid::build`` (grid.rs:246-464),
``Flow::vector`` (case.rs:345-365) and the box raster of geometry.rs:118-150.
Polygon-prism footprints are outside the projection engine's scope and rejected.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

BOUNDARY = ("periodic", "open", "wall", "slip", "ground_open_top")
INTERIOR, WALL, SLIP, INLET, OUTLET, BLOCKED = range(6)


def flow_vector(flow: dict, z: float):
    """Flow::vector (case.rs:345-365): the case flow at height z."""
    kind = flow["kind"]
    if kind == "prescribed_uniform":
        return tuple(float(v) for v in flow["velocity_m_s"])
    if kind == "laminar":
        return tuple(float(v) for v in flow["initial_velocity_m_s"])
    if kind == "neutral_rans":
        s = float(flow["speed_m_s"])
        h = float(flow["reference_height_m"])
        z0 = float(flow["roughness_m"])
        u = s * math.log((max(z, 0.0) + z0) / z0) / math.log((h + z0) / z0)
        t = float(flow["direction_deg_from"]) * (math.pi / 180.0)
        return (-u * math.sin(t), -u * math.cos(t), 0.0)
    raise ValueError(f"unknown flow kind {kind}")


@dataclass
class Grid:
    n: tuple
    dx: tuple
    volume: float
    periodic: tuple
    boundaries: tuple
    flow: dict
    fluid: np.ndarray            # u8[N]
    face_kind: np.ndarray        # u8[F]
    face_lo: np.ndarray          # i64[F], -1 for none
    face_hi: np.ndarray          # i64[F]
    face_area: np.ndarray        # f64[F]
    face_distance: np.ndarray    # f64[F]
    face_axis: np.ndarray        # u8[F]
    face_z: np.ndarray           # f64[F] face centre height
    component: np.ndarray        # i32[N], -1 solid
    anchored: np.ndarray         # u8[n_components]
    face_offsets: tuple = field(default=(0, 0, 0))
    face_dims: tuple = field(default=())
    preconditioner: str = "ic0"

    @property
    def count(self):
        return int(self.fluid.size)

    @property
    def n_faces(self):
        return int(self.face_kind.size)

    @property
    def n_components(self):
        return int(self.anchored.size)

    # ------------------------------------------------------------ construction
    @staticmethod
    def build(case: dict) -> "Grid":
        n = tuple(int(v) for v in case["grid"]["cells"])
        size = tuple(float(v) for v in case["domain"]["size_m"])
        dx = tuple(size[a] / n[a] for a in range(3))
        volume = ((1.0 * dx[0]) * dx[1]) * dx[2]
        bnd = tuple(case["boundaries"][k] for k in "xyz")
        for b in bnd:
            if b not in BOUNDARY:
                raise ValueError(f"unknown boundary {b}")
        periodic = tuple(b == "periodic" for b in bnd)
        flow = case["flow"]
        nx, ny, nz = n
        solid = np.zeros((nz, ny, nx), dtype=bool)
        for bi, blk in enumerate(case.get("geometry", [])):
            if blk.get("footprint_m") is not None:
                raise ValueError("polygon-prism footprints are not supported by the projection engine")
            rng = []
            for a in range(3):
                centres = (np.arange(n[a], dtype=np.float64) + 0.5) * dx[a]
                lo, hi = float(blk["min_m"][a]), float(blk["max_m"][a])
                first = n[a] if math.isnan(lo) else int(np.count_nonzero(centres < lo))
                end = int(np.count_nonzero(centres < hi))
                rng.append((first, max(end, first)))
            (i0, i1), (j0, j1), (k0, k1) = rng
            if i1 <= i0 or j1 <= j0 or k1 <= k0:
                raise ValueError(f"CFD-E028: geometry[{bi}] (box {blk.get('id', '')}) contains no cell center, "
                                 "so the grid does not represent it; enlarge it or refine the grid")
            solid[k0:k1, j0:j1, i0:i1] = True
        fluid3 = ~solid
        if not fluid3.any():
            raise ValueError("CFD-E030: geometry contains no fluid cells")
        fluid = fluid3.reshape(-1)
        N = fluid.size
        kinds, los, his, areas, dists, axes, zs = [], [], [], [], [], [], []
        offsets, dims = [], []
        offset = 0
        for a in range(3):
            fd = list(n)
            if not periodic[a]:
                fd[a] += 1
            offsets.append(offset)
            dims.append(tuple(fd))
            kk, jj, ii = np.meshgrid(np.arange(fd[2]), np.arange(fd[1]), np.arange(fd[0]), indexing="ij")
            q = [ii.reshape(-1), jj.reshape(-1), kk.reshape(-1)]
            t = q[a]
            cnt = t.size
            p_lo = [v.copy() for v in q]
            p_lo[a] = np.where(t > 0, t - 1, n[a] - 1)
            lo0 = (p_lo[2] * ny + p_lo[1]) * nx + p_lo[0]
            lo0 = np.where((t > 0) | periodic[a], lo0, -1)
            hi0 = np.where(t < n[a], (q[2] * ny + q[1]) * nx + q[0], -1)
            lo = np.where(lo0 >= 0, np.where(fluid[np.maximum(lo0, 0)], lo0, -1), -1)
            hi = np.where(hi0 >= 0, np.where(fluid[np.maximum(hi0, 0)], hi0, -1), -1)
            zc = (q[2].astype(np.float64) + (0.0 if a == 2 else 0.5)) * dx[2]
            kind = np.full(cnt, BLOCKED, dtype=np.uint8)
            interior = (lo >= 0) & (hi >= 0)
            blocked = (lo < 0) & (hi < 0)
            wall_between = ~interior & ~blocked & (lo0 >= 0) & (hi0 >= 0)
            boundary = ~interior & ~blocked & ~wall_between
            kind[interior] = INTERIOR
            kind[wall_between] = WALL
            b = bnd[a]
            if b == "wall":
                kind[boundary] = WALL
            elif b == "slip":
                kind[boundary] = SLIP
            elif b == "ground_open_top":
                kind[boundary & (t == 0)] = WALL
                kind[boundary & (t != 0)] = SLIP
            elif b == "open":
                sel = np.nonzero(boundary)[0]
                if sel.size:
                    # Only a few distinct face heights: evaluate Flow::vector per height with libm.
                    uz, inv = np.unique(zc[sel], return_inverse=True)
                    comp = np.array([flow_vector(flow, float(z))[a] for z in uz])[inv]
                    normal = np.where(t[sel] == 0, -1.0, 1.0)
                    v = comp * normal
                    kind[sel] = np.where(v < -1e-12, INLET, np.where(v > 1e-12, OUTLET, SLIP)).astype(np.uint8)
            kinds.append(kind)
            los.append(lo)
            his.append(hi)
            areas.append(np.full(cnt, volume / dx[a]))
            dists.append(np.where(kind == INTERIOR, dx[a], 0.5 * dx[a]))
            axes.append(np.full(cnt, a, dtype=np.uint8))
            zs.append(zc)
            offset += cnt
        face_kind = np.concatenate(kinds)
        face_lo = np.concatenate(los).astype(np.int64)
        face_hi = np.concatenate(his).astype(np.int64)
        component, anchored = _components(N, fluid, face_kind, face_lo, face_hi)
        pre = case.get("numerics", {}).get("pressure_preconditioner", "ic0")
        return Grid(n=n, dx=dx, volume=volume, periodic=periodic, boundaries=bnd, flow=flow,
                    fluid=fluid.astype(np.uint8), face_kind=face_kind, face_lo=face_lo, face_hi=face_hi,
                    face_area=np.concatenate(areas), face_distance=np.concatenate(dists),
                    face_axis=np.concatenate(axes), face_z=np.concatenate(zs), component=component,
                    anchored=anchored, face_offsets=tuple(offsets), face_dims=tuple(dims), preconditioner=pre)

    # ------------------------------------------------------------ face helpers
    def cell_face_indices(self):
        """(N, 3, 2) lower/upper face index per cell and axis (Grid::cell_faces, grid.rs:125-128)."""
        nx, ny, nz = self.n
        idx = np.arange(self.count)
        q = [idx % nx, idx // nx % ny, idx // (nx * ny)]
        out = np.empty((self.count, 3, 2), dtype=np.int64)
        for a in range(3):
            fd = self.face_dims[a]
            lo = self.face_offsets[a] + (q[2] * fd[1] + q[1]) * fd[0] + q[0]
            up = [v.copy() for v in q]
            up[a] = np.where(self.periodic[a] & (q[a] == self.n[a] - 1), 0, q[a] + 1)
            hi = self.face_offsets[a] + (up[2] * fd[1] + up[1]) * fd[0] + up[0]
            out[:, a, 0] = lo
            out[:, a, 1] = hi
        return out

    def divergence(self, u):
        """Grid::divergence (grid.rs:612-627); zero on solid cells."""
        cf = self.cell_face_indices()
        s = np.full(self.count, -0.0)
        for a in range(3):
            s = s + (u[cf[:, a, 1]] - u[cf[:, a, 0]]) / self.dx[a]
        return np.where(self.fluid == 1, s, 0.0)

    def gradient(self, p):
        """Grid::gradient (grid.rs:650-665)."""
        g = np.zeros(self.n_faces)
        lo, hi, k, d = self.face_lo, self.face_hi, self.face_kind, self.face_distance
        it = k == INTERIOR
        g[it] = (p[hi[it]] - p[lo[it]]) / d[it]
        ol = (k == OUTLET) & (lo >= 0)
        oh = (k == OUTLET) & (lo < 0)
        g[ol] = -p[lo[ol]] / d[ol]
        g[oh] = p[hi[oh]] / d[oh]
        return g

    def inlet_velocity(self):
        """The case flow's normal component at every inlet face (Flow::vector at the face centre)."""
        vals = np.zeros(self.n_faces)
        sel = np.nonzero(self.face_kind == INLET)[0]
        if sel.size:
            uz, inv = np.unique(self.face_z[sel], return_inverse=True)
            for a in range(3):
                m = self.face_axis[sel] == a
                if m.any():
                    comp = np.array([flow_vector(self.flow, float(z))[a] for z in uz])
                    vals[sel[m]] = comp[inv[m]]
        return vals

    def enforce_velocity(self, u):
        """Grid::enforce_velocity (grid.rs:683-691), in place."""
        k = self.face_kind
        u[(k == WALL) | (k == SLIP) | (k == BLOCKED)] = 0.0
        inlet = k == INLET
        if inlet.any():
            u[inlet] = self.inlet_velocity()[inlet]
        return u

    def initial_velocity(self):
        """Grid::initial_velocity (grid.rs:668-679)."""
        u = np.zeros(self.n_faces)
        k = self.face_kind
        live = ~((k == WALL) | (k == SLIP) | (k == BLOCKED))
        sel = np.nonzero(live)[0]
        if sel.size:
            uz, inv = np.unique(self.face_z[sel], return_inverse=True)
            for a in range(3):
                m = self.face_axis[sel] == a
                if m.any():
                    comp = np.array([flow_vector(self.flow, float(z))[a] for z in uz])
                    u[sel[m]] = comp[inv[m]]
        return u

    def weights(self):
        """Pressure face weights area / (distance * volume) (pressure.rs:257)."""
        return self.face_area / (self.face_distance * self.volume)


def _components(N, fluid, kind, lo, hi):
    """Fluid components through interior faces, numbered by their lowest cell
    (the breadth-first scan of grid.rs:430-462), and whether each touches an outlet."""
    from scipy.sparse import coo_matrix
    from scipy.sparse.csgraph import connected_components

    it = (kind == INTERIOR) & (lo != hi)
    a = coo_matrix((np.ones(int(it.sum()), dtype=np.int8), (lo[it], hi[it])), shape=(N, N))
    _, labels = connected_components(a, directed=False)
    comp = np.full(N, -1, dtype=np.int32)
    f = fluid.astype(bool)
    cells = np.nonzero(f)[0]
    lab = labels[cells]
    # Order components by their lowest fluid cell.
    first = {}
    for c, l in zip(cells[np.unique(lab, return_index=True)[1]].tolist(), np.unique(lab).tolist()):
        first[l] = c
    order = sorted(first, key=lambda l: first[l])
    remap = np.full(labels.max() + 1, -1, dtype=np.int64)
    for new, l in enumerate(order):
        remap[l] = new
    comp[cells] = remap[lab].astype(np.int32)
    anchored = np.zeros(len(order), dtype=np.uint8)
    out = kind == OUTLET
    cell = np.where(lo[out] >= 0, lo[out], hi[out])
    anchored[np.unique(comp[cell])] = 1
    return comp, anchored
