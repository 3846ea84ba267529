"""Writes tests/golden/path_receptors.json: receptor weights of point, volume-average and
path receptors on a small grid with a building, computed by the reference's own
independent checker (validation/check_fields.py receptor_weights / path_weights, pure
Python), as golden vectors for the package's restatement (cfd-craft_gb300/receptors.py).

    python tests/golden/make_path_receptors.py REFERENCE_CHECKOUT

The argument is the CFD-craft checkout (its validation/check_fields.py is imported).
"""
import importlib.util
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

CASE = {"cells": [24, 16, 8], "dx": 2.0, "boxes": [[[20.0, 10.0, 0.0], [30.0, 20.0, 10.0]]]}
RECEPTORS = [
    {"kind": "point", "id": "pt", "point_m": [7.3, 5.1, 3.9]},
    {"kind": "volume_average", "id": "vol", "min_m": [1.0, 2.5, 0.5], "max_m": [9.0, 6.0, 4.0]},
    {"kind": "path", "id": "p1", "polyline_m": [[2.5, 3.0], [15.0, 3.3], [16.0, 25.0]], "height_m": 3.2,
     "sample_spacing_m": 1.7},
    {"kind": "path", "id": "p2", "polyline_m": [[1.0, 30.0], [44.0, 29.5]], "height_m": 9.0,
     "sample_spacing_m": 0.9},
]


def main(reference):
    spec = importlib.util.spec_from_file_location("check_fields", os.path.join(reference, "validation",
                                                                               "check_fields.py"))
    cf = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(cf)
    import __graft_entry__ as entry

    pkg = entry.package()
    case = pkg.synth.case(tuple(CASE["cells"]), CASE["dx"], boxes=[tuple(map(tuple, b)) for b in CASE["boxes"]])
    g = pkg.grid.Grid.build(case)
    nx, ny, nz = CASE["cells"]
    index = lambda i, j, k: (k * ny + j) * nx + i  # noqa: E731
    fluid = [bool(v) for v in g.fluid]
    out = {"case": CASE, "receptors": []}
    for r in RECEPTORS:
        w = cf.receptor_weights(r, [CASE["dx"]] * 3, CASE["cells"], fluid, index)
        out["receptors"].append({"receptor": r, "weights": [[int(c), float(v)] for c, v in sorted(w.items())]})
    with open(os.path.join(HERE, "path_receptors.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1])
