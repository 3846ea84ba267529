"""Run archives written from device fields, audited by the reference's own checker.

tests/golden/device_archive_{plain,mixed} hold archives of three laminar SSPRK2 steps
that cfdg_step_device computed on a GB300 (plain FP64 and mixed FP32/FP64 projections),
written by the package's archive writer; device_archive_gas adds a gas constituent whose
transport steps, mass budget (cfdg_scalar_step_budget), current rates and receptor values
were computed on the device too, and device_archive_gas_muscl the same with MUSCL
advection; tests/golden/make_device_archive.py made them.
The unmodified validation/check_fields.py of a CFD-craft checkout (its independent
archive checker: hashes, mask, finiteness and the independent local continuity,
validation/check_fields.py:299-530) must pass on them; it runs when a checkout is
present (CFD_CRAFT_REFERENCE, default /root/reference) and is skipped otherwise. The
restated checks (tests/archive_check.py) run always.
"""
import importlib.util
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
REFERENCE = os.environ.get("CFD_CRAFT_REFERENCE", "/root/reference")
FORMS = ("plain", "mixed", "gas", "gas_muscl")


def archive(form):
    path = os.path.join(GOLDEN, f"device_archive_{form}")
    assert os.path.isdir(path), f"{path} missing: run tests/golden/make_device_archive.py on a GPU"
    return path


@pytest.mark.parametrize("form", FORMS)
def test_device_archive_passes_restated_checks(pkg, form):
    from archive_check import check_archive

    path = archive(form)
    manifest = json.load(open(os.path.join(path, "manifest.json")))
    assert manifest["engine"] == "cfd-craft_gb300" and manifest["executable_sha256"]
    from importlib import import_module

    R = import_module(pkg.__name__ + ".receptors")
    weights = lambda c, r: R.receptor_weights(pkg.grid.Grid.build(c), r)
    max_div = check_archive(path, lambda c: pkg.grid.Grid.build(c).fluid.astype(bool), receptor_weights=weights)
    assert max_div < 1e-7


@pytest.mark.parametrize("form", FORMS)
def test_device_archive_passes_reference_checker(form):
    checker = os.path.join(REFERENCE, "validation", "check_fields.py")
    if not os.path.exists(checker):
        pytest.skip("no CFD-craft checkout with validation/check_fields.py")
    spec = importlib.util.spec_from_file_location("cfd_craft_check_fields", checker)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    result = mod.check(archive(form))
    print(form, json.dumps(result))
    assert result["passed"] is True
    assert result["max_divergence_s_inv"] < 1e-7
    if form.startswith("gas"):  # the independent mass accounting of the device budget
        assert len(result["scalars"]) == 1 and result["scalars"][0]["relative_defect"] < 1e-9


def test_archive_writer_refuses_non_finite_fields(pkg, tmp_path):
    from importlib import import_module

    A = import_module(pkg.__name__ + ".archive")
    case = pkg.synth.case((4, 3, 2), 1.0)
    g = pkg.grid.Grid.build(case)
    u = np.zeros(g.n_faces)
    u[3] = np.nan
    with pytest.raises(ValueError, match="non-finite velocity"):
        A.write_run(str(tmp_path / "run"), case, g, u, np.zeros(g.count), steps=1, time_s=0.1)
