"""Source density fields of a case's emissions (crates/cfd-craft/src/transport.rs:90-178
source_fields), for the device transport step (cfdg_scalar_step_device's d_source).

Per source, cell weights: a point source puts weight 1 on the cell holding the point; a
line source splits its segment at the cell faces it crosses and gives each piece's cell
its parameter length (crossings closer than 1e-14 merged); a volume source gives each
cell its exact overlap with the box. A positive weight on a solid cell is CFD-E040, no
support CFD-E041; in steady mode a gas source whose support touches a sealed component is
CFD-E043 (particle constituents in steady mode need the deposition sinks, which are not
restated). The field receives rate * w / sum(w) / volume, the rate being rate_kg_s,
rate_kg_s_m times the line length, or rate_kg_s_m3 times the box volume (case.rs:684-705).
The arithmetic follows the reference's order, so the fields are the same bits.
"""
from __future__ import annotations

import math

import numpy as np


class SourceError(ValueError):
    """A CFD-E040/E041/E043/E044 source error."""


def rate(source: dict) -> float:
    """case.rs:684-705."""
    kind = source["kind"]
    if kind == "point":
        return float(source["rate_kg_s"])
    if kind == "line":
        s = -0.0
        for a in range(3):
            d = source["to_m"][a] - source["from_m"][a]
            s = s + d * d
        return source["rate_kg_s_m"] * math.sqrt(s)
    p = 1.0
    for a in range(3):
        p = p * (source["max_m"][a] - source["min_m"][a])
    return source["rate_kg_s_m3"] * p


def _cell_at(g, p):
    """transport.rs:24-29."""
    n = [int(v) for v in g.n]
    q = [min(int(math.floor(p[a] / g.dx[a])), n[a] - 1) for a in range(3)]
    return (q[2] * n[1] + q[1]) * n[0] + q[0]


def _weights(g, s):
    n = [int(v) for v in g.n]
    count = n[0] * n[1] * n[2]
    w = [0.0] * count
    kind = s["kind"]
    if kind == "point":
        w[_cell_at(g, s["point_m"])] = 1.0
    elif kind == "line":
        a0, a1 = s["from_m"], s["to_m"]
        ts = [0.0, 1.0]
        for a in range(3):
            d = a1[a] - a0[a]
            if abs(d) > 1e-14:
                for j in range(1, n[a]):
                    t = (float(j) * g.dx[a] - a0[a]) / d
                    if 0.0 < t < 1.0:
                        ts.append(t)
        ts.sort()
        kept = []
        for t in ts:  # Vec::dedup_by: drop an entry within 1e-14 of the last kept one
            if kept and abs(t - kept[-1]) < 1e-14:
                continue
            kept.append(t)
        for t0, t1 in zip(kept[:-1], kept[1:]):
            t = 0.5 * (t0 + t1)
            centre = [a0[a] + t * (a1[a] - a0[a]) for a in range(3)]
            c = _cell_at(g, centre)
            w[c] = w[c] + (t1 - t0)
    elif kind == "volume":
        lo, hi = s["min_m"], s["max_m"]
        for c in range(count):
            q = (c % n[0], (c // n[0]) % n[1], c // (n[0] * n[1]))
            v = 1.0
            for a in range(3):
                p = (q[a] + 0.5) * g.dx[a]
                v = v * max(min(hi[a], p + 0.5 * g.dx[a]) - max(lo[a], p - 0.5 * g.dx[a]), 0.0)
            w[c] = v
    else:
        raise ValueError(f"source kind {kind!r}")
    return w


def source_fields(case: dict, g) -> list:
    """One source density field (kg/m3/s per cell, numpy) per constituent, in case order."""
    constituents = [c["id"] for c in case.get("constituents", [])]
    fields = [[0.0] * int(g.count) for _ in constituents]
    steady = case.get("run", {}).get("mode") == "steady"
    fluid = np.asarray(g.fluid).astype(bool)
    comp = np.asarray(g.component)
    for s in case.get("sources", []):
        if s["constituent"] not in constituents:
            raise SourceError("unknown source constituent")
        si = constituents.index(s["constituent"])
        w = _weights(g, s)
        if any(wi > 1e-14 and not fluid[i] for i, wi in enumerate(w)):
            raise SourceError(f"CFD-E040: source {s['id']} intersects masked solid; no implicit redistribution")
        r = rate(s)
        if steady and r > 0.0:
            if case["constituents"][si].get("particle") is not None:
                raise NotImplementedError("steady particle sources need the deposition sinks")
            if any(wi > 1e-14 and not g.anchored[comp[i]] for i, wi in enumerate(w)):
                raise SourceError(f"CFD-E043: steady source {s['id']} has no outlet or represented particle "
                                  "deposition sink in its fluid component")
        norm = -0.0
        for wi in w:
            norm = norm + wi
        if norm <= 0.0:
            raise SourceError(f"CFD-E041: source {s['id']} has no support")
        dst = fields[si]
        for i, wi in enumerate(w):
            dst[i] = dst[i] + r * wi / norm / g.volume
    out = [np.array(f) for f in fields]
    if any(not np.all(np.isfinite(f)) for f in out):
        raise SourceError("CFD-E044: represented source density is nonfinite")
    return out


def diffusivity(case: dict, constituent: int, nut=None, cells: int = None) -> np.ndarray:
    """solver.rs:585-597: per cell the constituent's molecular diffusivity plus nu_t / Sc
    (Sc the case's turbulent Schmidt number with neutral_rans, else 1); `nut` the eddy
    viscosity per cell (zeros for laminar flow, then `cells` gives the count)."""
    flow = case["flow"]
    sc = flow["turbulent_schmidt"] if flow.get("kind") == "neutral_rans" else 1.0
    d0 = case["constituents"][constituent]["diffusivity_m2_s"]
    nut = np.zeros(int(cells)) if nut is None else np.asarray(nut, dtype=np.float64)
    return np.array([d0 + n / sc for n in nut.tolist()])

