"""Run archives with a constituent (output.rs:162-242 format with the solver state's
concentrations and budgets, solver.rs:190-260, and the summary's ScalarEvidence): the
package's writer on laminar steps and linear-upwind transport computed by the oracle,
with the budgets advance_scalar keeps (solver.rs:851-853) and the current rates rhs_into
returns. The restated checks of validation/check_fields.py (mass accounting, emission x
time, current boundary rates, receptor values) pass, and so does the reference's own
checker when a CFD-craft checkout is present."""
import importlib.util
import json
import os

import numpy as np
import pytest

REFERENCE = os.environ.get("CFD_CRAFT_REFERENCE", "/root/reference")


def constituent_case(pkg, name="archive-gas-16x12x8"):
    case = pkg.synth.case((16, 12, 8), 2.0, inflow=3.0, boxes=[((10.0, 6.0, 0.0), (16.0, 14.0, 8.0))], name=name)
    case["output"]["fields"] = True
    case["constituents"] = [{"id": "gas", "diffusivity_m2_s": 0.05}]
    case["sources"] = [
        {"id": "stack", "kind": "point", "constituent": "gas", "point_m": [5.0, 5.0, 3.0], "rate_kg_s": 2e-3},
        {"id": "area", "kind": "volume", "constituent": "gas", "min_m": [2.0, 16.0, 0.0], "max_m": [6.0, 22.0, 2.0],
         "rate_kg_s_m3": 1e-5},
    ]
    case["receptors"] = [
        {"id": "R1", "kind": "point", "point_m": [21.0, 9.0, 3.0]},
        {"id": "R2", "kind": "volume_average", "min_m": [24.0, 2.0, 0.0], "max_m": [30.0, 8.0, 4.0]},
    ]
    return case


def receptor_values(R, g, case, c):
    """solver.rs:1035-1037: Σ c w over each receptor's weights in order, from -0.0."""
    out = {}
    for r in case["receptors"]:
        acc = -0.0
        for cell, w in R.receptor_weights(g, r):
            acc = acc + c[cell] * w
        out[r["id"]] = acc
    return out


def test_archive_with_constituent_passes_checkers(pkg, O, tmp_path):
    from importlib import import_module

    from archive_check import check_archive

    A = import_module(pkg.__name__ + ".archive")
    S = import_module(pkg.__name__ + ".sources")
    R = import_module(pkg.__name__ + ".receptors")
    case = constituent_case(pkg)
    g = pkg.grid.Grid.build(case)
    og = O.Grid(case)
    code, u, p, info = og.project(g.initial_velocity(), np.zeros(g.count), 1.0, 1e-10, 10000)
    assert code == 0
    p[:] = 0.0
    its = info["iterations"]
    source = S.source_fields(case, g)[0]
    d = S.diffusivity(case, 0, cells=g.count)
    c = np.zeros(g.count)
    budget = np.zeros(3)
    steps, dt = 4, 0.1
    for _ in range(steps):
        code, u, p, it = og.step(u, p, dt, 1e-10, 10000)
        assert code == 0
        its += it
        c = og.scalar_step(c, u, d, source, dt, budget)
    rates = og.scalar_rates(c, u, d, source)
    entry = {"concentration": c, "rates": rates, "receptors": receptor_values(R, g, case, c),
             "budget": {"initial_kg": 0.0, "emitted_kg": budget[0], "inflow_kg": budget[1], "outflow_kg": budget[2]}}
    out = tmp_path / "run"
    A.write_run(str(out), case, g, u, p, steps=steps, time_s=dt * steps, pressure_iterations=its,
                constituents=[entry])
    weights = lambda c_, r: R.receptor_weights(pkg.grid.Grid.build(c_), r)
    check_archive(out, lambda c_: pkg.grid.Grid.build(c_).fluid.astype(bool), receptor_weights=weights)
    summary = json.loads((out / "summary.json").read_text())
    rec = summary["constituents"][0]
    assert rec["mass_kg"] > 0 and rec["relative_budget_defect"] < 1e-12
    assert (out / "probes.csv").read_text().count("\n") == 3
    checker = os.path.join(REFERENCE, "validation", "check_fields.py")
    if os.path.exists(checker):
        spec = importlib.util.spec_from_file_location("cfd_craft_check_fields", checker)
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        result = mod.check(str(out))
        assert result["passed"] and result["scalars"][0]["relative_defect"] < 1e-9, result


def test_archive_refuses_missing_or_unsupported_constituents(pkg, O, tmp_path):
    from importlib import import_module

    A = import_module(pkg.__name__ + ".archive")
    case = constituent_case(pkg)
    g = pkg.grid.Grid.build(case)
    u, p = g.initial_velocity(), np.zeros(g.count)
    with pytest.raises(ValueError):  # no entry for the case's constituent
        A.write_run(str(tmp_path / "a"), case, g, u, p, steps=0, time_s=0.0)
    entry = {"concentration": np.full(g.count, np.nan), "rates": (0.0, 0.0, 0.0), "receptors": {},
             "budget": {"initial_kg": 0.0, "emitted_kg": 0.0, "inflow_kg": 0.0, "outflow_kg": 0.0}}
    with pytest.raises(ValueError):  # non-finite concentration
        A.write_run(str(tmp_path / "b"), case, g, u, p, steps=0, time_s=0.0, constituents=[entry])
    particle = dict(case, constituents=[dict(case["constituents"][0], particle={"diameter_m": 1e-6})])
    with pytest.raises(ValueError):  # deposition is not written
        A.write_run(str(tmp_path / "c"), particle, g, u, p, steps=0, time_s=0.0, constituents=[entry])
