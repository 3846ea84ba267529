"""Run archives of device runs in CFD-craft's archive format, so that the reference's
independent checker (validation/check_fields.py) audits fields the engine produced.

Follows crates/cfd-craft/src/output.rs:162-242 (write_run): the artifacts case.json,
summary.json, geometry.json, probes.csv and fields.json, each hashed (SHA-256) into
manifest.json (schema cfd-craft.manifest/0.1, with the byte count before the manifest),
then complete.json holding the manifest's hash. fields.json is the solver State
(solver.rs:211-260: steps, time_s, velocity, pressure, k, epsilon, concentrations,
budgets, floor_events, pressure_iterations, monitor_history) as compact JSON;
geometry.json carries the fluid mask's hash (grid.rs:550, mask_sha256) and counts.

Scope: laminar runs on the device, with or without constituents. A constituent carries
its concentration field, its mass budget (solver.rs:190-202: initial, emitted, inflow and
outflow kg, the increments kept by cfdg_scalar_step_budget), its current rates
(cfdg_scalar_rates) and its receptor values (cfdg_receptors_sample); the writer adds the
summary's evidence record (solver.rs ScalarEvidence: mass, budget defect, extrema,
negative mass, rates, receptors) and the probes.csv rows. Gases only (no deposition) and
point or volume receptors (path receptors are refused). The summary holds the fields the
checker and a reader need (schema, name, termination, assessment, model scope, steps,
time, constituents), not the reference's full run summary (timings, profile, checks;
the constituent records omit steady_residual). The manifest carries the reference's keys
(output.rs:218-226); source_sha256 and executable_sha256 identify this engine's sources
and built library rather than the reference's CLI binary.
"""
from __future__ import annotations

import hashlib
import json
import os
import platform

import numpy as np

MANIFEST_SCHEMA = "cfd-craft.manifest/0.1"  # output.rs:229
RESULT_SCHEMA = "cfd-craft.result/0.1"      # solver.rs:374
ENGINE_VERSION = "0.2.0"


def _sha(data: bytes) -> str:
    return hashlib.sha256(data).hexdigest()


def _write(path: str, data: bytes):
    """Atomic write (output.rs atomic_write): a temporary file renamed into place."""
    tmp = path + ".tmp"
    with open(tmp, "wb") as f:
        f.write(data)
        f.flush()
        os.fsync(f.fileno())
    os.replace(tmp, path)


def _rust_e17(v: float) -> str:
    """A float as Rust formats it with {:.17e}: 17 digits after the point and the exponent
    without sign padding or leading zeros (1.00000000000000000e0, 2.5...e-5)."""
    mant, exp = f"{v:.17e}".split("e")
    return f"{mant}e{int(exp)}"


def _floats(a):
    return [float(v) for v in np.asarray(a, dtype=np.float64).ravel()]


def _engine_identity():
    """(source_sha256, executable_sha256) of the engine: the hash of its CUDA/C++ sources in
    name order and of the built library, the build identity output.rs records."""
    here = os.path.dirname(os.path.abspath(__file__))
    src = os.path.join(here, "csrc")
    h = hashlib.sha256()
    if os.path.isdir(src):
        for name in sorted(os.listdir(src)):
            with open(os.path.join(src, name), "rb") as fh:
                h.update(name.encode() + b"\0" + fh.read())
    lib = os.path.join(here, "_build", "libcfdgpu.so")
    exe = None
    if os.path.exists(lib):
        with open(lib, "rb") as fh:
            exe = _sha(fh.read())
    return h.hexdigest(), exe


def constituent_record(sp: dict, grid, c, budget: dict, rates, receptors: dict) -> dict:
    """The summary's evidence for one constituent (solver.rs ScalarEvidence) from its
    archived field, budget, current rates (emitted, inflow, outflow in kg/s) and receptor
    values: mass = Σ c over fluid cells × volume (an exact sum, math.fsum), the budget
    defect mass - initial - emitted - inflow + outflow and its ratio to their sum, the
    extrema (minimum over fluid cells, maximum over all cells and at least 0) and the mass
    of negative concentrations."""
    import math

    fluid = np.asarray(grid.fluid).astype(bool)
    c = np.asarray(c, dtype=np.float64)
    volume = float(grid.volume)
    mass = math.fsum(c[fluid].tolist()) * volume
    defect = mass - budget["initial_kg"] - budget["emitted_kg"] - budget["inflow_kg"] + budget["outflow_kg"]
    scale = max(budget["initial_kg"] + budget["emitted_kg"] + budget["inflow_kg"] + budget["outflow_kg"], 1e-30)
    negative = -math.fsum(np.minimum(c[fluid], 0.0).tolist()) * volume
    return {
        "id": sp["id"],
        "mass_kg": mass,
        "emitted_kg": float(budget["emitted_kg"]),
        "inflow_kg": float(budget["inflow_kg"]),
        "outflow_kg": float(budget["outflow_kg"]),
        "budget_defect_kg": defect,
        "relative_budget_defect": abs(defect) / scale,
        "minimum_kg_m3": float(c[fluid].min()) if fluid.any() else 0.0,
        "maximum_kg_m3": max(float(c.max()), 0.0),
        "negative_mass_kg": negative,
        "source_rate_kg_s": float(rates[0]),
        "boundary_inflow_rate_kg_s": float(rates[1]),
        "boundary_outflow_rate_kg_s": float(rates[2]),
        "receptors_kg_m3": {str(k): float(v) for k, v in sorted(receptors.items())},
    }


def write_run(out: str, case: dict, grid, velocity, pressure, *, steps: int, time_s: float,
              pressure_iterations: int = 0, k=None, epsilon=None, constituents=None, input_sha256: str = None,
              initial_state_sha256: str = None, engine: str = "cfd-craft_gb300") -> list:
    """Writes the archive of a run into the new directory `out`.

    velocity (F) and pressure (N) are host arrays (for example the device fields after
    cfdg_step_device, copied back). k and epsilon default to zeros (laminar).
    constituents: one dict per case constituent, in case order, with "concentration" (N),
    "budget" (initial_kg, emitted_kg, inflow_kg, outflow_kg), "rates" (the current
    emitted, inflow and outflow rates) and "receptors" ({receptor id: value}). Every value
    must be finite: the reference serialises the state with serde_json, which cannot write
    NaN or infinity, and its checker rejects non-finite fields (ValueError here). Returns
    the names of the files written, manifest.json and complete.json last."""
    species = case.get("constituents") or []
    constituents = constituents or []
    if len(constituents) != len(species):
        raise ValueError("one constituent entry per case constituent, in case order")
    if any(r.get("kind") == "path" for r in case.get("receptors", [])) and species:
        raise ValueError("path receptors are not written by this archive writer")
    if any(sp.get("particle") is not None for sp in species):
        raise ValueError("particle constituents (deposition) are not written by this archive writer")
    n, f = int(grid.count), int(grid.n_faces)
    velocity = np.asarray(velocity, dtype=np.float64)
    pressure = np.asarray(pressure, dtype=np.float64)
    if velocity.shape != (f,) or pressure.shape != (n,):
        raise ValueError("velocity must have one value per face and pressure one per cell")
    k = np.zeros(n) if k is None else np.asarray(k, dtype=np.float64)
    epsilon = np.zeros(n) if epsilon is None else np.asarray(epsilon, dtype=np.float64)
    for name, a in (("velocity", velocity), ("pressure", pressure), ("k", k), ("epsilon", epsilon)):
        if not np.all(np.isfinite(a)):
            raise ValueError(f"non-finite {name}: a run archive holds finite fields only")
    records = []
    for sp, entry in zip(species, constituents):
        conc = np.asarray(entry["concentration"], dtype=np.float64)
        if conc.shape != (n,) or not np.all(np.isfinite(conc)):
            raise ValueError(f"constituent {sp['id']}: one finite concentration per cell")
        records.append(constituent_record(sp, grid, conc, entry["budget"], entry["rates"], entry["receptors"]))
    source_sha256, executable_sha256 = _engine_identity()
    os.makedirs(out, exist_ok=False)
    files = {}
    written = []
    total = 0

    def put(name, data: bytes):
        nonlocal total
        _write(os.path.join(out, name), data)
        files[name] = _sha(data)
        written.append(name)
        total += len(data)

    case_bytes = json.dumps(case, indent=2).encode()
    put("case.json", case_bytes)
    summary = {
        "schema_version": RESULT_SCHEMA,
        "name": case.get("name", ""),
        "case_sha256": _sha(json.dumps(case, separators=(",", ":")).encode()),
        "termination": "completed",
        "assessment": "transient_interval_completed",
        "error": None,
        "model_scope": "incompressible_laminar",
        "steps": int(steps),
        "time_s": float(time_s),
        "pressure_iterations": int(pressure_iterations),
        "constituents": records,
        "engine": engine,
        "source_sha256": source_sha256,
        "build_version": f"{engine} {ENGINE_VERSION}",
        "initial_state_sha256": initial_state_sha256,
    }
    put("summary.json", json.dumps(summary, indent=2).encode())
    fluid = np.asarray(grid.fluid, dtype=np.uint8)
    geometry = {
        "mask_sha256": _sha(fluid.tobytes()),
        "cells": [int(v) for v in grid.n],
        "fluid_cells": int(fluid.sum()),
        "solid_cells": int(n - fluid.sum()),
        "components": int(grid.n_components),
    }
    put("geometry.json", json.dumps(geometry, indent=2).encode())
    probes = "constituent,receptor,concentration_kg_m3\n"
    for rec in records:  # output.rs:195-201: quoted fields, the value as Rust's {:.17e}
        for rid, value in rec["receptors_kg_m3"].items():
            probes += '"{}","{}",{}\n'.format(rec["id"].replace('"', '""'), rid.replace('"', '""'), _rust_e17(value))
    put("probes.csv", probes.encode())
    fields = {
        "steps": int(steps),
        "time_s": float(time_s),
        "velocity": _floats(velocity),
        "pressure": _floats(pressure),
        "k": _floats(k),
        "epsilon": _floats(epsilon),
        "concentrations": [_floats(e["concentration"]) for e in constituents],
        "budgets": [{k2: float(e["budget"][k2]) for k2 in ("initial_kg", "emitted_kg", "inflow_kg", "outflow_kg")}
                    for e in constituents],
        "floor_events": 0,
        "pressure_iterations": int(pressure_iterations),
        "monitor_history": [],
    }
    put("fields.json", json.dumps(fields, separators=(",", ":"), allow_nan=False).encode())
    manifest = {
        "schema_version": MANIFEST_SCHEMA,
        "files": files,
        "omitted": {},
        "input_case_sha256": input_sha256 or _sha(case_bytes),
        "source_sha256": source_sha256,
        "version": f"{engine} {ENGINE_VERSION}",
        "initial_state_sha256": initial_state_sha256,
        "executable_sha256": executable_sha256,
        "bytes_before_manifest": total,
        "threads": int(case.get("run", {}).get("threads", 1)),
        "engine": engine,
        "architecture": platform.machine(),
        "os": platform.system().lower(),
    }
    manifest_bytes = json.dumps(manifest, indent=2).encode()
    _write(os.path.join(out, "manifest.json"), manifest_bytes)
    _write(os.path.join(out, "complete.json"), json.dumps({"manifest_sha256": _sha(manifest_bytes)}).encode())
    return written + ["manifest.json", "complete.json"]
