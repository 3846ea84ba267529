"""Receptor weights of a grid (crates/cfd-craft/src/transport.rs:366-436 receptor_weights),
for DeviceGrid.set_receptors / cfdg_receptors_set.

A point receptor takes trilinear weights between cell centres, clamped at the domain
boundary, dropping weights <= 1e-14 (transport.rs:376-397); a volume average takes each
cell's exact overlap with the box (:398-411). Weights are then normalised by their sum in
order (:428-434). A receptor with no weight or a positive weight on a solid cell is
CFD-E042 (:422-427). Path receptors (transport.rs:412-420, receptor_path_weights) are not
restated. The arithmetic follows the reference's order so the weights are the same bits.
"""
from __future__ import annotations

import math


class ReceptorError(ValueError):
    """CFD-E042: the receptor is empty or samples through a solid."""


def _point(g, point_m):
    n = [int(v) for v in g.n]
    base = [math.floor(point_m[a] / g.dx[a] - 0.5) for a in range(3)]
    frac = [point_m[a] / g.dx[a] - 0.5 - base[a] for a in range(3)]
    out = []
    for k in range(2):
        for j in range(2):
            for i in range(2):
                b = (i, j, k)
                q = [min(max(base[a] + b[a], 0), n[a] - 1) for a in range(3)]
                w = 1.0  # Iterator::product starts from 1.0
                for a in range(3):
                    w = w * ((1.0 - frac[a]) if b[a] == 0 else frac[a])
                if w > 1e-14:
                    out.append(((q[2] * n[1] + q[1]) * n[0] + q[0], w))
    return out


def _volume(g, min_m, max_m):
    n = [int(v) for v in g.n]
    out = []
    for c in range(n[0] * n[1] * n[2]):
        q = (c % n[0], (c // n[0]) % n[1], c // (n[0] * n[1]))
        w = 1.0
        for a in range(3):
            p = (q[a] + 0.5) * g.dx[a]  # Grid::center
            w = w * max(min(max_m[a], p + 0.5 * g.dx[a]) - max(min_m[a], p - 0.5 * g.dx[a]), 0.0)
        if w > 1e-14:
            out.append((c, w))
    return out


def receptor_weights(g, receptor: dict):
    """Normalised (cell, weight) pairs of a receptor given as the case schema's object:
    {"kind": "point", "point_m": [...]} or {"kind": "volume_average", "min_m": [...], "max_m": [...]}."""
    kind = receptor.get("kind", "point")
    if kind == "point":
        w = _point(g, receptor["point_m"])
    elif kind == "volume_average":
        w = _volume(g, receptor["min_m"], receptor["max_m"])
    else:
        raise ValueError(f"receptor kind {kind!r} is not restated")
    fluid = g.fluid
    if not w or any(not fluid[c] for c, _ in w):
        raise ReceptorError(f"CFD-E042: receptor {receptor.get('id', '?')} is empty or samples through a solid")
    norm = -0.0  # Iterator::sum
    for _, v in w:
        norm = norm + v
    return [(c, v / norm) for c, v in w]
