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


# docs/evidence/anisotropic-pressure.md:122-141 (shapes) and :41-60 (iterations IC(0) /
# point MG / candidate MG): the rough manufactured pressure sin(0.73 i) + 0.3 cos(0.17 i),
# centred, its operator image as the RHS (examples/pressure_probe.rs:60-68), tol 1e-14,
# at most 1200 iterations. The oracle's multigrid is the candidate (line/plane block
# smoothing with semicoarsening on anisotropic grids, multigrid/line.rs); on the three
# shapes below the anisotropy threshold it is the point cycle, whose counts equal the
# candidate's there.
ANISOTROPIC = {
    "isotropic": ([24, 2, 24], [1.0, 1.0, 1.0], "wall", 60, 8),
    "near-isotropic": ([96, 2, 24], [4.0, 0.1, 1.0], "wall", 122, 13),
    "threshold25": ([64, 2, 64], [1.0, 0.1, 0.2], "wall", 108, 24),
    "thin100": ([64, 2, 64], [1.0, 0.1, 0.1], "wall", 92, 5),
    "thin400": ([64, 2, 64], [1.0, 0.1, 0.05], "wall", 86, 5),
    "cube100": ([48, 48, 48], [1.0, 1.0, 0.1], "wall", 147, 5),
    "slab100": ([32, 32, 16], [1.0, 1.0, 0.05], "wall", 118, 6),
    "plate64": ([64, 8, 64], [1.0, 1.0, 1.0], "wall", 126, 11),
    "plate256": ([64, 16, 64], [1.0, 4.0, 1.0], "wall", 199, 12),
    "thin1600": ([64, 8, 64], [1.0, 1.0, 0.2], "wall", 152, 19),
    "thin6400": ([64, 8, 64], [1.0, 1.0, 0.1], "wall", 162, 18),
    "review-stretched": ([64, 8, 64], [1.0, 1.0, 0.02], "wall", 161, 17),
    "odd": ([33, 5, 17], [1.0, 1.0, 0.1], "wall", 87, 14),
    "periodic": ([31, 5, 17], [0.05, 1.0, 1.0], "periodic", 145, 7),
    "outlet": ([33, 5, 17], [1.0, 1.0, 0.1], "open", 92, 13),
    "stiff-two-cell": ([32, 2, 32], [1.0, 0.001, 1.0], "wall", 95, 9),
    "long-domain": ([128, 2, 16], [100.0, 1.0, 1.0], "wall", 220, 23),
    "short-stiff-axis": ([64, 64, 8], [1.0, 1.0, 0.01], "wall", 204, 6),
}


def anisotropic_case(name, pre):
    n, size, bx, _, _ = ANISOTROPIC[name]
    c = copy.deepcopy(LID_CAVITY)
    c["grid"]["cells"] = list(n)
    c["domain"]["size_m"] = list(size)
    c["boundaries"]["x"] = bx
    if bx == "open":
        c["flow"]["initial_velocity_m_s"] = [1.0, 0.0, 0.0]
    c["numerics"]["pressure_preconditioner"] = pre
    return c


def rough_rhs(g):
    """pressure_probe.rs:60-68: the rough exact pressure, centred, and its operator image."""
    import math

    import numpy as np

    exact = np.array([math.sin(0.73 * v) + 0.3 * math.cos(0.17 * v) for v in range(g.count)])
    exact = g.center_nullspaces(exact)
    return exact, g.apply(exact)


def urban_case(n, open_x, blocks):
    """tests/urban_pressure_reference.rs:15-31 `base(n, open)` with its blocks: the lid
    cavity re-gridded to n cells of 1 m, walls in y and z, x open (inflow 1 m/s) or wall,
    multigrid preconditioner."""
    c = copy.deepcopy(LID_CAVITY)
    c["grid"]["cells"] = list(n)
    c["domain"]["size_m"] = [float(v) for v in n]
    c["boundaries"] = {"x": "open" if open_x else "wall", "y": "wall", "z": "wall"}
    c["flow"]["initial_velocity_m_s"] = [1.0, 0.0, 0.0]
    c["numerics"]["pressure_preconditioner"] = "multigrid"
    c["geometry"] = [{"id": name, "min_m": list(lo), "max_m": list(hi)} for name, lo, hi in blocks]
    return c


# urban_pressure_reference.rs:138-147 and :150-169
URBAN_BARRIER = ((9, 2, 5), True, [("full-barrier", (3.0, 0.0, 0.0), (4.0, 2.0, 5.0))])
URBAN_SINGLETON = ((7, 3, 5), True, [("left", (2.0, 1.0, 2.0), (3.0, 2.0, 3.0)), ("right", (4.0, 1.0, 2.0), (5.0, 2.0, 3.0)),
                                     ("front", (3.0, 0.0, 2.0), (4.0, 1.0, 3.0)), ("back", (3.0, 2.0, 2.0), (4.0, 3.0, 3.0)),
                                     ("floor", (3.0, 1.0, 1.0), (4.0, 2.0, 2.0)), ("roof", (3.0, 1.0, 3.0), (4.0, 2.0, 4.0))])


def dense_reference(g):
    """urban_pressure_reference.rs:52-136: the matrix assembled directly from the face
    energies, the manufactured field sin(0.19 i) on fluid cells (centred per sealed
    component), its image b, and an independent pivoted dense solve with one gauge cell
    per sealed component removed, centred. Returns (exact, b, reference)."""
    import numpy as np

    n = g.count
    a = np.zeros((n, n))
    kind, lo, hi = np.asarray(g.face_kind), np.asarray(g.face_lo), np.asarray(g.face_hi)
    w = np.asarray(g.face_area) / np.asarray(g.face_distance) / g.volume
    for f in range(g.n_faces):
        if kind[f] == 0:
            i, j = lo[f], hi[f]
            a[i, i] += w[f]
            a[j, j] += w[f]
            a[i, j] -= w[f]
            a[j, i] -= w[f]
        elif kind[f] == 4:
            i = lo[f] if lo[f] >= 0 else hi[f]
            a[i, i] += w[f]
    comp = np.asarray(g.component)
    sealed = [cid for cid in range(g.n_components) if not g.anchored[cid]]

    def center(x):
        x = x.copy()
        for cid in sealed:
            m = comp == cid
            x[m] -= x[m].mean()
        return x

    fluid = np.asarray(g.fluid).astype(bool)
    exact = center(np.where(fluid, np.sin(0.19 * np.arange(n)), 0.0))
    b = a @ exact
    gauges = [int(np.nonzero(comp == cid)[0][0]) for cid in sealed]
    active = [i for i in range(n) if fluid[i] and i not in gauges]
    sol = np.linalg.solve(a[np.ix_(active, active)], b[active])
    ref = np.zeros(n)
    ref[active] = sol
    return exact, b, center(ref)


def lid_case(n, boundary_x):
    """tests/multigrid.rs:12-27 `case(n, boundary)`: the lid cavity (1 m cube, periodic y,
    wall z) re-gridded to n cells, x boundary as given, inflow 1 m/s, multigrid."""
    c = copy.deepcopy(LID_CAVITY)
    c["grid"]["cells"] = list(n)
    c["boundaries"]["x"] = boundary_x
    c["flow"]["initial_velocity_m_s"] = [1.0, 0.0, 0.0]
    c["numerics"]["pressure_preconditioner"] = "multigrid"
    return c


MANUFACTURED_SHAPES = [(9, 2, 7), (8, 5, 6), (2, 2, 2), (9, 1, 7)]


def topology_case(cells, boundaries, solid):
    """multigrid/masked.rs:468-510 `topology`: the lid cavity re-gridded to `cells` 1 m
    cells with the given boundaries and one 1 m block per solid cell."""
    c = copy.deepcopy(LID_CAVITY)
    c["grid"]["cells"] = list(cells)
    c["domain"]["size_m"] = [float(v) for v in cells]
    c["boundaries"] = dict(zip("xyz", boundaries))
    c["flow"]["initial_velocity_m_s"] = [1.0, 0.0, 0.0]
    c["numerics"]["pressure_preconditioner"] = "multigrid"
    c["geometry"] = []
    for z in range(cells[2]):
        for y in range(cells[1]):
            for x in range(cells[0]):
                if solid((x, y, z)):
                    c["geometry"].append({"id": f"s{x}-{y}-{z}", "min_m": [float(x), float(y), float(z)],
                                          "max_m": [float(x + 1), float(y + 1), float(z + 1)]})
    return c


def porous_mask():
    """multigrid/masked.rs:551-559: a fixed pseudo-random 45 % solid mask of 8 x 6 x 6 cells
    from a 64-bit linear congruential generator."""
    state, mask = 12345, []
    for _ in range(8 * 6 * 6):
        state = (state * 6364136223846793005 + 1442695040888963407) % (1 << 64)
        mask.append((state >> 33) % 100 < 45)
    return mask
