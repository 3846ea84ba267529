"""The oracle and the grid builder against the stored fixtures of tests/golden/."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def fixtures(pkg):
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.cases(pkg)


def test_oracle_reproduces_golden(pkg, O):
    for name, case in fixtures(pkg).items():
        ref = np.load(os.path.join(GOLDEN, f"{name}.npz"))
        og = O.Grid(case)
        g = pkg.grid.Grid.build(case)
        for k in ("fluid", "face_kind", "face_lo", "face_hi", "face_area", "face_distance", "component", "anchored"):
            assert np.array_equal(getattr(og, k), ref[k]), (name, k)
            assert np.array_equal(getattr(g, k), ref[k]), (name, k)
        for pre in ("ic0", "multigrid"):
            og.set_preconditioner(pre)
            code, uu, pp, info = og.project(ref["u"], np.zeros(og.count), 0.25, 1e-10, 10000)
            assert code == int(ref[f"{pre}_code"])
            assert info["iterations"] == int(ref[f"{pre}_iterations"])
            assert np.array_equal(uu.view(np.uint64), ref[f"{pre}_u"].view(np.uint64))
            assert np.array_equal(pp.view(np.uint64), ref[f"{pre}_p"].view(np.uint64))


@pytest.mark.gpu
def test_engine_matches_golden(pkg):
    for name, case in fixtures(pkg).items():
        ref = np.load(os.path.join(GOLDEN, f"{name}.npz"))
        g = pkg.grid.Grid.build(case)
        for pre in ("ic0", "multigrid"):
            dg = pkg.pressure.DeviceGrid(g, preconditioner=pre)
            u, p = ref["u"].copy(), np.zeros(g.count)
            code = int(ref[f"{pre}_code"])
            if code:
                with pytest.raises(pkg.pressure.PressureError) as e:
                    dg.project(u, p, 0.25, 1e-10, 10000)
                assert e.value.code == code
            else:
                info = dg.project(u, p, 0.25, 1e-10, 10000)
                assert abs(info.iterations - int(ref[f"{pre}_iterations"])) <= 1
                for got, want in ((u, ref[f"{pre}_u"]), (p, ref[f"{pre}_p"])):
                    assert np.max(np.abs(got - want)) <= 1e-10 * max(1.0, np.max(np.abs(want))), (name, pre)
            dg.close()


def test_receptor_weights_against_reference_checker_vectors(pkg):
    """cfd-craft_gb300/receptors.py (point, volume-average and path receptors,
    transport.rs:202-436) against weights computed by the reference's independent archive
    checker (validation/check_fields.py), stored by tests/golden/make_path_receptors.py.
    The checker sums with math.fsum and math.dist, so the bar is 1e-13 relative, same cells."""
    import json
    import os
    from importlib import import_module

    R = import_module(pkg.__name__ + ".receptors")
    with open(os.path.join(os.path.dirname(__file__), "golden", "path_receptors.json")) as f:
        gold = json.load(f)
    spec = gold["case"]
    case = pkg.synth.case(tuple(spec["cells"]), spec["dx"], boxes=[tuple(map(tuple, b)) for b in spec["boxes"]])
    g = pkg.grid.Grid.build(case)
    for item in gold["receptors"]:
        ours = R.receptor_weights(g, item["receptor"])
        ref = item["weights"]
        assert [c for c, _ in ours] == [c for c, _ in ref], item["receptor"]["id"]
        for (_, a), (_, b) in zip(ours, ref):
            assert abs(a - b) <= 1e-13 * max(abs(b), 1e-300), (item["receptor"]["id"], a, b)
    # A path through the building is refused (CFD-E087), one leaving the domain too (E086).
    for bad, code in (({"kind": "path", "id": "x", "polyline_m": [[2.0, 15.0], [46.0, 15.0]], "height_m": 3.0,
                        "sample_spacing_m": 1.0}, "CFD-E087"),
                      ({"kind": "path", "id": "y", "polyline_m": [[2.0, 5.0], [60.0, 5.0]], "height_m": 3.0,
                        "sample_spacing_m": 1.0}, "CFD-E086")):
        try:
            R.receptor_weights(g, bad)
            raise AssertionError("accepted " + bad["id"])
        except R.ReceptorError as e:
            assert str(e).startswith(code), str(e)
