"""Restated checks of validation/check_fields.py (the reference's independent archive
checker) that a flow-only archive must pass: the completion marker's manifest hash
(:301-302), the manifest schema (:304-307), every artifact's hash and no unlisted entries
(:308-317), the fluid mask hash against geometry.json (:329-346), finite fields with one
value per cell (:433-438), the face count of the velocity (:450-460) and the independent
local continuity max |div u| <= 1e-7 max(1, max|u|) / min(dx) (:500-518). Test helper."""
import hashlib
import json
import math
from pathlib import Path


def sha(p):
    return hashlib.sha256(p.read_bytes()).hexdigest()


def check_archive(path, fluid_of_case):
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
    assert len(c["constituents"]) == len(s["concentrations"]) == len(s["budgets"]) == 0
    return max_div
