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
  * receptor_weights for a point receptor (transport.rs:374-399, :428-436): trilinear
    weights between cell centres, clamped at the domain boundary, weights below 1e-14
    dropped, normalised to sum 1.
The grid arrays are cfd-craft_gb300/grid.py's (the reference's face order).
"""
from __future__ import annotations

import math

import numpy as np

INTERIOR, INLET, OUTLET = 0, 3, 4


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

    def rhs(self, c, u, source, inlet_value=0.0):
        """dc/dt (kg/m3/s) for concentrations c and face velocities u (transport.rs:651-699)."""
        lo, hi = self.lo, self.hi
        cl = np.where(lo >= 0, c[np.maximum(lo, 0)], inlet_value)
        cr = np.where(hi >= 0, c[np.maximum(hi, 0)], inlet_value)
        uf = u[self.faces]
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
