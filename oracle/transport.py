"""CPU restatement of CFD-craft's scalar transport and receptor sampling (test infrastructure).

Used only by tests/ to state the mixed-precision form's error on receptor
concentrations: the same constituent release is transported on the flow projected by
the FP64 oracle and on the flow projected by the engine's mixed form, and the receptor
concentrations are compared. Nothing in the engine imports this module.

Follows crates/cfd-craft/src/transport.rs:
  * rhs_into (transport.rs:651-699), linear upwind (Advection::LinearUpwind, case.rs:835):
    per transporting face (Interior, Inlet, Outlet) the donor value is the upwind cell's
    concentration (the inlet value where that side has no cell), the diffusive flux is
    d_face (c_lo - c_hi) / distance with d_face the mean of the two cells' diffusivities
    (one cell's on a boundary face, none on outlets), flux = (u donor + diff) area, and
    flux / volume is subtracted from the lo cell and added to the hi cell;
  * MUSCL (Advection::Muscl, transport.rs:502-526, 670-694): the donor value of a face is
    the upwind cell's value plus (flow towards hi) or minus half its slope along the face's
    axis, slope = minmod((c_hi - c_lo) / 2, minmod(2 (c - c_lo), 2 (c_hi - c))) with a
    neighbour counted only through an interior face (the cell's own value otherwise);
  * receptor_weights for a point receptor (transport.rs:374-399, :428-436): trilinear
    weights between cell centres, clamped at the domain boundary, weights below 1e-14
    dropped, normalised to sum 1.
The grid arrays are cfd-craft_gb300/grid.py's (the reference's face order).
"""
from __future__ import annotations

import math

import numpy as np

INTERIOR, INLET, OUTLET = 0, 3, 4


def _minmod(a, b):
    """minmod (transport.rs:510-516): 0 where a b <= 0, else sign(a) min(|a|, |b|)."""
    return np.where(a * b <= 0.0, 0.0, np.sign(a) * np.minimum(np.abs(a), np.abs(b)))


class Transport:
    """Linear-upwind transport operator of one grid, vectorised over faces."""

    def __init__(self, g, diffusivity):
        self.g = g
        kind = np.asarray(g.face_kind)
        sel = (kind == INTERIOR) | (kind == INLET) | (kind == OUTLET)
        self.faces = np.nonzero(sel)[0]
        self.lo = np.asarray(g.face_lo)[self.faces].astype(np.int64)
        self.hi = np.asarray(g.face_hi)[self.faces].astype(np.int64)
        self.kind = kind[self.faces]
        self.area = np.asarray(g.face_area)[self.faces]
        self.dist = np.asarray(g.face_distance)[self.faces]
        d = np.full(g.count, float(diffusivity)) if np.isscalar(diffusivity) else np.asarray(diffusivity)
        dl = np.where(self.lo >= 0, d[np.maximum(self.lo, 0)], 0.0)
        dh = np.where(self.hi >= 0, d[np.maximum(self.hi, 0)], 0.0)
        both = (self.lo >= 0) & (self.hi >= 0)
        self.dface = np.where(both, 0.5 * (dl + dh), np.where(self.lo >= 0, dl, dh))
        self.volume = float(g.volume)

    def slopes(self, c):
        """(N, 3) monotonized-central limited slopes of c per cell and axis (MUSCL)."""
        g = self.g
        cf = g.cell_face_indices()
        kind = np.asarray(g.face_kind)
        flo, fhi = np.asarray(g.face_lo), np.asarray(g.face_hi)
        out = np.zeros((g.count, 3))
        for a in range(3):
            fl, fh = cf[:, a, 0], cf[:, a, 1]
            lo = np.where(kind[fl] == INTERIOR, c[np.maximum(flo[fl], 0)], c)
            hi = np.where(kind[fh] == INTERIOR, c[np.maximum(fhi[fh], 0)], c)
            out[:, a] = _minmod(0.5 * (hi - lo), _minmod(2.0 * (c - lo), 2.0 * (hi - c)))
        return out

    def rhs(self, c, u, source, inlet_value=0.0, muscl=False):
        """dc/dt (kg/m3/s) for concentrations c and face velocities u (transport.rs:651-699),
        linear upwind or (muscl) MUSCL donors."""
        lo, hi = self.lo, self.hi
        cl = np.where(lo >= 0, c[np.maximum(lo, 0)], inlet_value)
        cr = np.where(hi >= 0, c[np.maximum(hi, 0)], inlet_value)
        uf = u[self.faces]
        if muscl:
            sl = self.slopes(c)
            axis = np.asarray(self.g.face_axis)[self.faces].astype(np.int64)
            dl = np.where(lo >= 0, cl + 0.5 * sl[np.maximum(lo, 0), axis], cl)
            dh = np.where(hi >= 0, cr - 0.5 * sl[np.maximum(hi, 0), axis], cr)
            donor = np.where(uf >= 0.0, dl, dh)
        else:
            donor = np.where(uf >= 0.0, cl, cr)
        diff = np.where(self.kind == OUTLET, 0.0, self.dface * (cl - cr) / self.dist)
        per_volume = (uf * donor + diff) * self.area / self.volume
        v = np.array(source, dtype=np.float64, copy=True)
        np.subtract.at(v, lo[lo >= 0], per_volume[lo >= 0])
        np.add.at(v, hi[hi >= 0], per_volume[hi >= 0])
        return v

    def stable_dt(self, u, cfl=0.4):
        """A forward-Euler step within the advective and diffusive limits of this flow."""
        g = self.g
        umax = float(np.max(np.abs(u[self.faces]))) if self.faces.size else 0.0
        dmin = min(g.dx)
        dt_adv = cfl * dmin / max(umax, 1e-30)
        dmax = float(np.max(self.dface)) if self.dface.size else 0.0
        dt_diff = 0.1 * dmin * dmin / max(dmax, 1e-30)
        return min(dt_adv, dt_diff)

    def run(self, u, source, steps, dt, inlet_value=0.0):
        c = np.zeros(self.g.count)
        fluid = np.asarray(self.g.fluid, dtype=bool)
        for _ in range(steps):
            c = c + dt * self.rhs(c, u, source, inlet_value)
            c[~fluid] = 0.0
        return c


def point_weights(g, point_m):
    """Normalised trilinear weights of a point receptor (transport.rs:374-399, :428-436)."""
    n = [int(v) for v in g.n]
    base = [math.floor(point_m[a] / g.dx[a] - 0.5) for a in range(3)]
    frac = [point_m[a] / g.dx[a] - 0.5 - base[a] for a in range(3)]
    out = []
    for k in range(2):
        for j in range(2):
            for i in range(2):
                b = (i, j, k)
                q = [min(max(base[a] + b[a], 0), n[a] - 1) for a in range(3)]
                w = 1.0
                for a in range(3):
                    w *= (1.0 - frac[a]) if b[a] == 0 else frac[a]
                if w > 1e-14:
                    out.append(((q[2] * n[1] + q[1]) * n[0] + q[0], w))
    total = sum(w for _, w in out)
    return [(i, w / total) for i, w in out]


def sample(c, weights):
    return sum(c[i] * w for i, w in weights)
