"""Writes tests/golden/*.npz: small regression fixtures of the oracle.

The reference (Rust) cannot run here; its published known answers are pinned in
tests/test_oracle_pins.py. These fixtures freeze the oracle's outputs on small seeded
cases (grid arrays, projection results, iteration counts) so that both the oracle and the
engine are checked against stored numbers, not only against each other. Regenerate with
    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))


def cases(pkg):
    from cases import LID_CAVITY, kernel_case, periodic_case

    return {
        "buildings_12x10x8": pkg.synth.case((12, 10, 8), 1.0, boxes=[((4.0, 3.0, 0.0), (7.0, 6.0, 4.0))]),
        "pocket_12x12x6": pkg.synth.case((12, 12, 6), 1.0, boxes=[((3, 3, 0), (9, 4, 4)), ((3, 8, 0), (9, 9, 4)),
                                                                  ((3, 3, 0), (4, 9, 4)), ((8, 3, 0), (9, 9, 4)),
                                                                  ((3, 3, 3), (9, 9, 4))]),
        "cavity_24x2x24": kernel_case("cavity24", "ic0"),
        "periodic_masked_6x3x2": periodic_case([6, 3, 2], "wall", False, True),
    }


def main():
    import __graft_entry__ as entry
    from oracle import oracle as O

    pkg = entry.package()
    for name, case in cases(pkg).items():
        og = O.Grid(case)
        g = pkg.grid.Grid.build(case)
        u = pkg.synth.random_velocity(g, 42)
        p = np.zeros(g.count)
        out = dict(fluid=og.fluid, face_kind=og.face_kind, face_lo=og.face_lo, face_hi=og.face_hi,
                   face_area=og.face_area, face_distance=og.face_distance, component=og.component,
                   anchored=og.anchored, u=u)
        for pre in ("ic0", "multigrid"):
            og.set_preconditioner(pre)
            code, uu, pp, info = og.project(u, p, 0.25, 1e-10, 10000)
            out[f"{pre}_code"] = np.int64(code)
            out[f"{pre}_u"] = uu
            out[f"{pre}_p"] = pp
            out[f"{pre}_iterations"] = np.int64(info["iterations"])
            out[f"{pre}_relative_residual"] = np.float64(info["relative_residual"])
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        print(name, g.count, out["ic0_code"], out["ic0_iterations"], out["multigrid_iterations"])


if __name__ == "__main__":
    main()
