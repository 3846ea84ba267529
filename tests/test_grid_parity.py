"""The package's numpy Grid.build against the oracle's restatement of grid.rs, bit for bit."""
import copy

import numpy as np
import pytest

from cases import CANYON_93K, LID_CAVITY, periodic_case

FIELDS = ["fluid", "face_kind", "face_lo", "face_hi", "face_area", "face_distance", "component", "anchored"]


def _cases(pkg):
    out = [LID_CAVITY, CANYON_93K, periodic_case([3, 1, 4]), periodic_case([1, 3, 1]),
           periodic_case([6, 3, 2], "open", True, True), periodic_case([6, 3, 2], "wall", False, True),
           pkg.synth.config1(), pkg.synth.case((40, 36, 20), 2.0, boxes=[((10, 10, 0), (30, 16, 20)),
                                                                          ((0, 30, 0), (20, 40, 40))])]
    for d in (0, 45, 90, 200, 270, 315):
        c = copy.deepcopy(CANYON_93K)
        c["flow"]["direction_deg_from"] = d
        out.append(c)
    # A sealed pocket: a closed component inside buildings.
    out.append(pkg.synth.case((12, 12, 6), 1.0, boxes=[((3, 3, 0), (9, 4, 4)), ((3, 8, 0), (9, 9, 4)),
                                                       ((3, 3, 0), (4, 9, 4)), ((8, 3, 0), (9, 9, 4)),
                                                       ((3, 3, 3), (9, 9, 4))]))
    return out


def test_grid_build_matches_oracle(pkg, O):
    for case in _cases(pkg):
        g = pkg.grid.Grid.build(case)
        og = O.Grid(case)
        for k in FIELDS:
            a, b = getattr(g, k), getattr(og, k)
            assert a.shape == b.shape, k
            if a.dtype == np.float64:
                assert np.array_equal(a.view(np.uint64), b.view(np.uint64)), (case["name"], k)
            else:
                assert np.array_equal(a, b), (case["name"], k)
        cf = g.cell_face_indices()
        f = g.fluid == 1
        assert np.array_equal(cf[f].reshape(-1, 6), og.cell_faces[f])


def test_sealed_pocket_is_a_closed_component(pkg):
    c = _cases(pkg)[-1]
    g = pkg.grid.Grid.build(c)
    assert g.n_components == 2 and list(g.anchored) == [1, 0]


def test_divergence_gradient_enforce_match_oracle(pkg, O):
    for case in _cases(pkg)[:8]:
        g = pkg.grid.Grid.build(case)
        og = O.Grid(case)
        rng = np.random.default_rng(1)
        u = rng.uniform(-1, 1, g.n_faces)
        p = rng.uniform(-1, 1, g.count)
        assert np.array_equal(g.divergence(u), og.divergence(u))
        assert np.array_equal(g.gradient(p), og.gradient(p))
        assert np.array_equal(g.enforce_velocity(u.copy()), og.enforce_velocity(u))
