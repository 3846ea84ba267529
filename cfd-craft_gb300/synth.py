"""Seeded synthetic cases in the reference's case schema (cfd-craft.case/0.1).

The benchmark configurations name grid shapes, building counts and velocity
distributions but no dataset; these generators draw them from numpy's PCG64
(default_rng(seed)) so the engine and the oracle see identical inputs.
"""
from __future__ import annotations

import copy

import numpy as np

_BASE = {
    "schema_version": "cfd-craft.case/0.1",
    "name": "synthetic",
    "domain": {"size_m": [1.0, 1.0, 1.0]},
    "grid": {"cells": [2, 2, 2]},
    "boundaries": {"x": "open", "y": "wall", "z": "wall"},
    "flow": {"kind": "laminar", "initial_velocity_m_s": [1.0, 0.0, 0.0], "viscosity_m2_s": 1.5e-5,
             "acceleration_m_s2": [0.0, 0.0, 0.0]},
    "geometry": [],
    "constituents": [],
    "initial_conditions": [],
    "sources": [],
    "receptors": [],
    "numerics": {"transport": "linear_upwind", "max_time_step_s": 0.1, "advective_cfl_max": 0.4,
                 "pressure_relative_tolerance": 1e-8, "pressure_max_iterations": 10000,
                 "steady_residual_tolerance": 1e-5, "steady_monitor_tolerance": 1e-3, "monitor_window": 10},
    "run": {"mode": "transient", "end_time_s": 20.0, "max_steps": 200, "wall_time_limit_s": 3600.0,
            "threads": 1, "memory_limit_mib": 65536},
    "output": {"fields": False, "checkpoint": False, "max_total_mib": 64},
}


def case(cells, dx=1.0, boundaries=("open", "wall", "wall"), inflow=1.0, boxes=(), preconditioner="ic0",
         name="synthetic"):
    """A laminar case with open-x inflow `inflow` m/s on a uniform grid of spacing dx."""
    c = copy.deepcopy(_BASE)
    c["name"] = name
    c["grid"]["cells"] = [int(v) for v in cells]
    c["domain"]["size_m"] = [float(v) * dx for v in cells]
    c["boundaries"] = dict(zip("xyz", boundaries))
    c["flow"]["initial_velocity_m_s"] = [float(inflow), 0.0, 0.0]
    c["numerics"]["pressure_preconditioner"] = preconditioner
    c["geometry"] = [dict(id=f"b{i}", min_m=list(map(float, lo)), max_m=list(map(float, hi)))
                     for i, (lo, hi) in enumerate(boxes)]
    return c


def random_boxes(rng, count, size_m, side=(10.0, 30.0), height=(10.0, 60.0), dx=1.0):
    """`count` ground-based boxes: footprint sides U[side], heights U[height] clipped below
    the domain top, origins uniform inside the domain; each contains at least one cell centre."""
    boxes = []
    lx, ly, lz = size_m
    for _ in range(count):
        sx, sy = rng.uniform(*side), rng.uniform(*side)
        h = min(rng.uniform(*height), lz - dx)
        x0 = rng.uniform(0.0, max(lx - sx, dx))
        y0 = rng.uniform(0.0, max(ly - sy, dx))
        boxes.append(((x0, y0, 0.0), (min(x0 + sx, lx), min(y0 + sy, ly), max(h, dx))))
    return boxes


def config1():
    """64x64x32 uniform grid, dx = 1 m, no buildings, open x / wall y,z; IC(0)."""
    return case((64, 64, 32), 1.0, preconditioner="ic0", name="c1-64x64x32")


def config2(seed=1):
    """128x128x64 grid, dx = 2 m, 12 box buildings, inflow 5 m/s; multigrid."""
    rng = np.random.default_rng(seed)
    cells = (128, 128, 64)
    size = [v * 2.0 for v in cells]
    return case(cells, 2.0, inflow=5.0, boxes=random_boxes(rng, 12, size, dx=2.0), preconditioner="multigrid",
                name="c2-128x128x64-12b")


def config3(seed=2, preconditioner="multigrid"):
    """256x256x128 grid (8.4 M cells), dx = 2 m, 40 box buildings."""
    rng = np.random.default_rng(seed)
    cells = (256, 256, 128)
    size = [v * 2.0 for v in cells]
    return case(cells, 2.0, inflow=5.0, boxes=random_boxes(rng, 40, size, dx=2.0), preconditioner=preconditioner,
                name="c3-256x256x128-40b")


SHAPES4 = ((48, 48, 48), (64, 64, 32), (96, 96, 48), (128, 128, 64), (160, 160, 80))


def config4(count=64, seed=100, preconditioner="multigrid"):
    """`count` uneven cases: shapes uniform over SHAPES4, 0-20 boxes each, dx = 2 m."""
    out = []
    for i in range(count):
        rng = np.random.default_rng(seed + i)
        cells = SHAPES4[int(rng.integers(len(SHAPES4)))]
        size = [v * 2.0 for v in cells]
        nb = int(rng.integers(0, 21))
        out.append(case(cells, 2.0, inflow=5.0, boxes=random_boxes(rng, nb, size, dx=2.0),
                        preconditioner=preconditioner, name=f"c4-{i}"))
    return out


def config5(seed=4, preconditioner="multigrid"):
    """36 wind directions (10 degree steps) over a 128x128x64 grid with 30 buildings
    (open x/y, ground_open_top z, neutral_rans), plus 16 cases at 96x96x48."""
    out = []
    rng = np.random.default_rng(seed)
    cells = (128, 128, 64)
    size = [v * 2.0 for v in cells]
    boxes = random_boxes(rng, 30, size, dx=2.0)
    for d in range(36):
        c = case(cells, 2.0, boundaries=("open", "open", "ground_open_top"), boxes=boxes,
                 preconditioner=preconditioner, name=f"c5-dir{10 * d}")
        c["flow"] = {"kind": "neutral_rans", "speed_m_s": 5.0, "reference_height_m": 10.0, "roughness_m": 0.1,
                     "direction_deg_from": float(10 * d), "viscosity_m2_s": 1.5e-5, "turbulent_schmidt": 0.7}
        out.append(c)
    for i in range(16):
        r2 = np.random.default_rng(seed * 1000 + i)
        cells2 = (96, 96, 48)
        size2 = [v * 2.0 for v in cells2]
        out.append(case(cells2, 2.0, inflow=5.0, boxes=random_boxes(r2, int(r2.integers(0, 21)), size2, dx=2.0),
                        preconditioner=preconditioner, name=f"c5-small{i}"))
    return out


def random_velocity(grid, seed=0, lo=-1.0, hi=1.0):
    """Face velocities i.i.d. U[lo, hi], then the fixed boundary values (enforce_velocity)."""
    rng = np.random.default_rng(seed)
    u = rng.uniform(lo, hi, size=grid.n_faces)
    grid.enforce_velocity(u)
    return u
