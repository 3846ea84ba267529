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
