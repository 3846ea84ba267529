"""Small cases shared by the tests: the reference's unit-test grids, restated.

The reference tests mutate committed cases (cases/verification/periodic-tracer.json,
lid-cavity.json) in place; the fields the projection reads are reproduced here so
nothing reads the reference checkout at run time.
"""
import copy

LID_CAVITY = {
    "schema_version": "cfd-craft.case/0.1",
    "name": "lid-cavity-re100",
    "domain": {"size_m": [1.0, 1.0, 1.0]},
    "grid": {"cells": [24, 2, 24]},
    "boundaries": {"x": "wall", "y": "periodic", "z": "wall"},
    "flow": {"kind": "laminar", "initial_velocity_m_s": [0.0, 0.0, 0.0], "viscosity_m2_s": 0.01,
             "acceleration_m_s2": [0.0, 0.0, 0.0]},
    "geometry": [],
    "numerics": {"pressure_relative_tolerance": 1e-10, "pressure_max_iterations": 1200},
}

# cases/performance/canyon-93k.json: the fields the pressure path reads.
CANYON_93K = {
    "schema_version": "cfd-craft.case/0.1",
    "name": "performance-canyon-93k",
    "domain": {"size_m": [18.0, 16.0, 6.0]},
    "grid": {"cells": [54, 48, 36]},
    "boundaries": {"x": "open", "y": "open", "z": "ground_open_top"},
    "flow": {"kind": "neutral_rans", "speed_m_s": 2.0, "reference_height_m": 1.0, "roughness_m": 0.01,
             "direction_deg_from": 270, "viscosity_m2_s": 1.5e-05, "turbulent_schmidt": 0.7},
    "geometry": [
        {"id": "west", "min_m": [5.0, 3.0, 0.0], "max_m": [6.0, 13.0, 1.0]},
        {"id": "east", "min_m": [7.0, 3.0, 0.0], "max_m": [8.0, 13.0, 1.0]},
    ],
    "numerics": {"pressure_relative_tolerance": 1e-10, "pressure_max_iterations": 1200},
}

# The reference's periodic-tracer unit-test grid (pressure.rs:509-526): periodic
# axes, cell size 1 m, laminar flow at rest.
PERIODIC = {
    "schema_version": "cfd-craft.case/0.1",
    "name": "periodic",
    "domain": {"size_m": [3.0, 3.0, 3.0]},
    "grid": {"cells": [3, 3, 3]},
    "boundaries": {"x": "periodic", "y": "periodic", "z": "periodic"},
    "flow": {"kind": "laminar", "initial_velocity_m_s": [0.0, 0.0, 0.0], "viscosity_m2_s": 0.01,
             "acceleration_m_s2": [0.0, 0.0, 0.0]},
    "geometry": [],
    "numerics": {},
}

KERNELS = {
    "cavity24": [24, 2, 24],
    "cavity48": [48, 2, 48],
    "cavity96": [96, 2, 96],
    "cube24": [24, 24, 24],
    "cube48": [48, 48, 48],
}
# docs/evidence/pressure-multigrid.md:32-38 (IC(0) / multigrid iterations, tol 1e-11).
KERNEL_ITERATIONS = {
    "cavity24": (53, 6), "cavity48": (102, 6), "cavity96": (193, 6), "cube24": (61, 7), "cube48": (113, 7),
}


def kernel_case(name, pre):
    c = copy.deepcopy(LID_CAVITY)
    c["grid"]["cells"] = list(KERNELS[name])
    c["numerics"]["pressure_preconditioner"] = pre
    return c


def periodic_case(n, boundary_x="periodic", open_flow=False, barrier=False):
    """pressure.rs:509-526 `case(n)` with the mutations of its tests."""
    c = copy.deepcopy(PERIODIC)
    c["grid"]["cells"] = list(n)
    c["domain"]["size_m"] = [float(v) for v in n]
    c["boundaries"]["x"] = boundary_x
    if open_flow:
        c["flow"]["initial_velocity_m_s"] = [1.0, 0.0, 0.0]
    if barrier:
        c["geometry"] = [{"id": "barrier", "min_m": [2.0, 0.0, 0.0], "max_m": [3.0, 3.0, 2.0]}]
    return c


def sin_field(n, k=0.73):
    """(k * i).sin() per cell, with the C library's sin (what Rust's f64::sin calls)."""
    import math

    import numpy as np

    return np.array([math.sin(k * float(i)) for i in range(n)])
