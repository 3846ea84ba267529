"""Receptor weights of a grid (crates/cfd-craft/src/transport.rs:366-436 receptor_weights),
for DeviceGrid.set_receptors / cfdg_receptors_set.

A point receptor takes trilinear weights between cell centres, clamped at the domain
boundary, dropping weights <= 1e-14 (transport.rs:376-397); a volume average takes each
cell's exact overlap with the box (:398-411); a path receptor combines the point weights
of its samples with their trapezoidal coefficients (:412-420), the samples equally spaced
in arc length along the polyline at a constant height (path_samples, :202-281; sample
count case.rs:795-820), after every segment was checked against the domain and against
represented solid cells (check_path_segments, :282-336; CFD-E086/E087/E088). Weights are
then normalised by their sum in order (:428-434). A receptor with no weight or a positive
weight on a solid cell is CFD-E042 (:422-427). The arithmetic follows the reference's
order (hypot from the C library, as Rust's f64::hypot) so the weights are the same bits.
"""
from __future__ import annotations

import ctypes
import ctypes.util
import math

try:  # the C library's hypot, which Rust's f64::hypot calls
    _libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
    _libm.hypot.restype = ctypes.c_double
    _libm.hypot.argtypes = [ctypes.c_double, ctypes.c_double]
    _hypot = _libm.hypot
except OSError:  # pragma: no cover
    _hypot = math.hypot

PATH_SAMPLES_MAX = 20001  # case.rs:789


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


def path_sample_count(receptor: dict) -> int:
    """case.rs:795-820: ceil(length / spacing) intervals (at least 1), plus one."""
    pts = receptor["polyline_m"]
    length = -0.0
    for a, b in zip(pts[:-1], pts[1:]):
        length = length + _hypot(b[0] - a[0], b[1] - a[1])
    spacing = receptor["sample_spacing_m"]
    if not math.isfinite(length) or length <= 0.0 or not math.isfinite(spacing) or spacing <= 0.0:
        return PATH_SAMPLES_MAX + 1
    return max(int(math.ceil(length / spacing)), 1) + 1


def path_samples(receptor: dict):
    """transport.rs:202-281: (points, distances, trapezoidal coefficients) of a path."""
    rid = receptor.get("id", "?")
    count = path_sample_count(receptor)
    if count > PATH_SAMPLES_MAX:
        raise ReceptorError(f"CFD-E088: receptor {rid} exceeds 20001 path samples")
    pts, height = receptor["polyline_m"], receptor["height_m"]
    if not 2 <= len(pts) <= 4097 or not math.isfinite(height) or not all(math.isfinite(v) for p in pts for v in p):
        raise ReceptorError(f"CFD-E086: receptor {rid} has invalid path vertices/height")
    cumulative = [0.0]
    for a, b in zip(pts[:-1], pts[1:]):
        seg = _hypot(b[0] - a[0], b[1] - a[1])
        if seg <= 0.0:
            raise ReceptorError(f"CFD-E086: receptor {rid} has a zero-length segment")
        cumulative.append(cumulative[-1] + seg)
    length = cumulative[-1]
    intervals = count - 1
    points, distances, coeffs = [], [], []
    segment = 0
    for sample in range(count):
        distance = length if sample == intervals else length * float(sample) / float(intervals)
        while segment + 2 < len(cumulative) and cumulative[segment + 1] < distance:
            segment += 1
        t = min(max((distance - cumulative[segment]) / (cumulative[segment + 1] - cumulative[segment]), 0.0), 1.0)
        if sample == intervals:
            point = [pts[-1][0], pts[-1][1], height]
        else:
            a, b = pts[segment], pts[segment + 1]
            point = [a[0] + t * (b[0] - a[0]), a[1] + t * (b[1] - a[1]), height]
        points.append(point)
        distances.append(distance)
        coeffs.append(0.5 / intervals if sample in (0, intervals) else 1.0 / intervals)
    return points, distances, coeffs


def _cell_at(g, p):
    """transport.rs:24-29."""
    n = [int(v) for v in g.n]
    q = [min(int(math.floor(p[a] / g.dx[a])), n[a] - 1) for a in range(3)]
    return (q[2] * n[1] + q[1]) * n[0] + q[0]


def _check_path_segments(g, receptor: dict):
    """transport.rs:282-336: the path inside the domain and no segment through a solid cell."""
    rid = receptor.get("id", "?")
    pts, height = receptor["polyline_m"], receptor["height_m"]
    n = [int(v) for v in g.n]
    if any(p[0] < 0.0 or p[1] < 0.0 or p[0] >= n[0] * g.dx[0] or p[1] >= n[1] * g.dx[1] for p in pts) \
            or height < 0.0 or height >= n[2] * g.dx[2]:
        raise ReceptorError(f"CFD-E086: receptor {rid} path is outside the domain")
    fluid = g.fluid
    for index, (a, b) in enumerate(zip(pts[:-1], pts[1:])):
        crossings = [0.0, 1.0]
        for axis in range(2):
            delta = b[axis] - a[axis]
            if delta == 0.0:
                continue
            for k in range(1, n[axis]):
                t = (float(k) * g.dx[axis] - a[axis]) / delta
                if 0.0 < t < 1.0:
                    crossings.append(t)
        crossings.sort()
        for lo, hi in zip(crossings[:-1], crossings[1:]):
            if hi <= lo:
                continue
            t = 0.5 * (lo + hi)
            point = [a[0] + t * (b[0] - a[0]), a[1] + t * (b[1] - a[1]), height]
            if not fluid[_cell_at(g, point)]:
                raise ReceptorError(f"CFD-E087: receptor {rid} path segment {index} crosses a represented solid cell")


def _path(g, receptor: dict):
    points, _, coeffs = path_samples(receptor)
    _check_path_segments(g, receptor)
    combined = {}
    for point, coefficient in zip(points, coeffs):
        try:
            sample = receptor_weights(g, {"kind": "point", "id": receptor.get("id", "?"), "point_m": point})
        except ReceptorError as e:
            raise ReceptorError(f"CFD-E087: receptor {receptor.get('id', '?')} path sample has invalid "
                                f"interpolation support: {e}") from None
        for cell, value in sample:  # BTreeMap entry += coefficient * value
            combined[cell] = (combined[cell] if cell in combined else 0.0) + coefficient * value
    return sorted(combined.items())


def receptor_weights(g, receptor: dict):
    """Normalised (cell, weight) pairs of a receptor given as the case schema's object:
    {"kind": "point", "point_m": [...]}, {"kind": "volume_average", "min_m": [...], "max_m": [...]}
    or {"kind": "path", "polyline_m": [[x, y], ...], "height_m": h, "sample_spacing_m": s}."""
    kind = receptor.get("kind", "point")
    if kind == "point":
        w = _point(g, receptor["point_m"])
    elif kind == "volume_average":
        w = _volume(g, receptor["min_m"], receptor["max_m"])
    elif kind == "path":
        w = _path(g, receptor)
    else:
        raise ValueError(f"receptor kind {kind!r} is not restated")
    fluid = g.fluid
    if not w or any(not fluid[c] for c, _ in w):
        raise ReceptorError(f"CFD-E042: receptor {receptor.get('id', '?')} is empty or samples through a solid")
    norm = -0.0  # Iterator::sum
    for _, v in w:
        norm = norm + v
    return [(c, v / norm) for c, v in w]
