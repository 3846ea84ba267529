"""Restated checks of validation/check_fields.py (the reference's independent archive
checker) that an archive must pass: the completion marker's manifest hash (:301-302), the
manifest schema (:304-307), every artifact's hash and no unlisted entries (:308-317), the
fluid mask hash against geometry.json (:329-346), finite fields with one value per cell
(:433-438), the face count of the velocity (:450-460), the independent local continuity
max |div u| <= 1e-7 max(1, max|u|) / min(dx) (:500-518), and per gas constituent
(:519-840): counts and order, finite values, zero in solid cells, receptor values from
their weights (1e-12), the archived mass against the record (1e-11 of the budget scale)
and the independent mass accounting mass - initial - emitted - inflow + outflow (1e-9),
no negative concentration, the emission against rate x time (1e-9), and the current
source and boundary rates recomputed from the fields of a laminar flow (1e-9). Test
helper."""
import hashlib
import json
import math
from pathlib import Path


def sha(p):
    return hashlib.sha256(p.read_bytes()).hexdigest()


def check_archive(path, fluid_of_case, receptor_weights=None):
    """receptor_weights(case, receptor) -> [(cell, weight)]: checks the recorded receptor values."""
    path = Path(path)
    marker = json.loads((path / "complete.json").read_text())
    assert sha(path / "manifest.json") == marker["manifest_sha256"], "manifest hash"
    manifest = json.loads((path / "manifest.json").read_text())
    assert manifest["schema_version"] == "cfd-craft.manifest/0.1"
    for name, digest in manifest["files"].items():
        assert sha(path / name) == digest, f"artifact hash: {name}"
    unlisted = {e.name for e in path.iterdir()} - set(manifest["files"]) - {"manifest.json", "complete.json"}
    assert not unlisted, unlisted
    c = json.loads((path / "case.json").read_text())
    geometry = json.loads((path / "geometry.json").read_text())
    s = json.loads((path / "fields.json").read_text())
    nx, ny, nz = c["grid"]["cells"]
    n = nx * ny * nz
    dx = [L / N for L, N in zip(c["domain"]["size_m"], [nx, ny, nz])]
    fluid = fluid_of_case(c)
    assert hashlib.sha256(bytes(int(f) for f in fluid)).hexdigest() == geometry["mask_sha256"], "mask"
    assert all(math.isfinite(v) for v in s["velocity"])
    for name in ("pressure", "k", "epsilon"):
        assert len(s[name]) == n and all(math.isfinite(v) for v in s[name]), name
    comps, off = [], 0
    for a in range(3):
        dims = [nx, ny, nz]
        periodic = c["boundaries"]["xyz"[a]] == "periodic"
        if not periodic:
            dims[a] += 1
        cnt = dims[0] * dims[1] * dims[2]
        comps.append((dims, s["velocity"][off:off + cnt]))
        off += cnt
    assert off == len(s["velocity"]), "face count"
    max_div = 0.0
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                cell = (k * ny + j) * nx + i
                if not fluid[cell]:
                    continue
                div = 0.0
                for a, (dims, v) in enumerate(comps):
                    p = [i, j, k]
                    lo = (p[2] * dims[1] + p[1]) * dims[0] + p[0]
                    p[a] += 1
                    if c["boundaries"]["xyz"[a]] == "periodic":
                        p[a] %= [nx, ny, nz][a]
                    hi = (p[2] * dims[1] + p[1]) * dims[0] + p[0]
                    div += (v[hi] - v[lo]) / dx[a]
                max_div = max(max_div, abs(div))
    speed = max((abs(v) for v in s["velocity"]), default=0.0)
    assert max_div <= 1e-7 * max(1.0, speed) / min(dx), ("independent local continuity", max_div)
    summary = json.loads((path / "summary.json").read_text())
    assert len(c["constituents"]) == len(s["concentrations"]) == len(s["budgets"]) == len(summary["constituents"])
    volume = dx[0] * dx[1] * dx[2]
    for sp, values, budget, record in zip(c["constituents"], s["concentrations"], s["budgets"],
                                          summary["constituents"]):
        assert record["id"] == sp["id"]
        assert len(values) == n and all(math.isfinite(v) for v in values)
        assert all(v == 0.0 for v, f in zip(values, fluid) if not f), "solid cell concentration"
        if receptor_weights is not None:
            for r in c["receptors"]:
                w = receptor_weights(c, r)
                value = math.fsum(values[cell] * wi for cell, wi in w)
                assert abs(record["receptors_kg_m3"][r["id"]] - value) <= 1e-12 * max(abs(value), 1e-300) + 1e-300
        mass = math.fsum(v for v, f in zip(values, fluid) if f) * volume
        scale = max(budget["initial_kg"] + budget["emitted_kg"] + budget["inflow_kg"] + budget["outflow_kg"], 1e-30)
        defect = mass - budget["initial_kg"] - budget["emitted_kg"] - budget["inflow_kg"] + budget["outflow_kg"]
        assert abs(mass - record["mass_kg"]) < 1e-11 * scale, "reported mass"
        assert abs(defect) < 1e-9 * scale, ("independent mass accounting", defect / scale)
        assert min(values) >= -1e-10 * max(max(values), 1e-30), "negative concentration"
        rate = 0.0
        for src in c["sources"]:
            if src["constituent"] != sp["id"]:
                continue
            if src["kind"] == "point":
                rate += src["rate_kg_s"]
            elif src["kind"] == "line":
                rate += src["rate_kg_s_m"] * math.dist(src["from_m"], src["to_m"])
            else:
                rate += src["rate_kg_s_m3"] * math.prod(b - a for a, b in zip(src["min_m"], src["max_m"]))
        assert abs(budget["emitted_kg"] - rate * s["time_s"]) < 1e-9 * scale, "emission x time"
        incoming = outgoing = 0.0
        nominal_u = c["flow"].get("velocity_m_s", c["flow"].get("initial_velocity_m_s"))
        for a, (dims, v) in enumerate(comps):
            if c["boundaries"]["xyz"[a]] != "open":
                continue
            for k in range(nz):
                for j in range(ny):
                    for i in range(nx):
                        q = [i, j, k]
                        for side in (-1, 1):
                            if q[a] != (0 if side < 0 else [nx, ny, nz][a] - 1):
                                continue
                            cell = (k * ny + j) * nx + i
                            if not fluid[cell]:
                                continue
                            face = list(q)
                            if side > 0:
                                face[a] += 1
                            normal_u = side * v[(face[2] * dims[1] + face[1]) * dims[0] + face[0]]
                            flux = max(normal_u, 0.0) * values[cell] * volume / dx[a]
                            if side * nominal_u[a] < -1e-12:
                                flux += sp["diffusivity_m2_s"] * values[cell] / (0.5 * dx[a]) * volume / dx[a]
                            outgoing += max(flux, 0.0)
                            incoming += max(-flux, 0.0)
        flux_scale = max(rate + outgoing + incoming, 1e-30)
        assert abs(record["source_rate_kg_s"] - rate) < 1e-9 * flux_scale, "current source rate"
        assert abs(record["boundary_outflow_rate_kg_s"] - outgoing) < 1e-9 * flux_scale, "current outflow"
        assert abs(record["boundary_inflow_rate_kg_s"] - incoming) < 1e-9 * flux_scale, "current inflow"
    return max_div
