"""Writes run archives of laminar steps computed on the device, as fixtures for the
reference's own archive checker (validation/check_fields.py), which the CPU tests run
on them (tests/test_device_archive.py).

    python tests/golden/make_device_archive.py [OUT_DIR]

Needs a CUDA device and the built engine. For each arithmetic form (plain FP64, mixed
FP32/FP64) it projects the initial state of a 16x10x8 laminar case with one building
(dt = 1, like the solver's start, solver.rs:1436-1445), runs three SSPRK2 steps of
dt = 0.1 s with cfdg_step_device (a projection per stage), copies the fields back and
writes the archive with the package's writer (output.rs:162-242 format) into
OUT_DIR/device_archive_<form> (default: this directory). device_archive_gas adds a gas
constituent (a point and a volume source, a point and a volume receptor) on a 16x12x8
case, and device_archive_gas_muscl the same case with MUSCL advection: each of four steps of dt = 0.1 s is a flow step (mixed form) and a transport step
with its budget (cfdg_scalar_step_budget), then the current rates (cfdg_scalar_rates)
and the receptor values (cfdg_receptors_sample), all computed on the device.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def archive_case(pkg):
    c = pkg.synth.case((16, 10, 8), 2.0, inflow=5.0, preconditioner="multigrid",
                       boxes=[((12.0, 6.0, 0.0), (20.0, 14.0, 10.0))], name="device-archive-16x10x8")
    c["output"]["fields"] = True
    return c


def main(out_dir=HERE):
    sys.path.insert(0, ROOT)
    import torch
    from importlib import import_module

    import __graft_entry__ as entry

    pkg = entry.package()
    A = import_module(pkg.__name__ + ".archive")
    case = archive_case(pkg)
    g = pkg.grid.Grid.build(case)
    dev = torch.device("cuda", 0)
    for form in ("plain", "mixed"):
        dg = pkg.pressure.DeviceGrid(g, preconditioner="multigrid", precision=form)
        dg.set_flow(case)
        u, p = g.initial_velocity(), np.zeros(g.count)
        its = dg.project(u, p, 1.0, 1e-8, 10000).iterations
        p[:] = 0.0  # the solver zeroes the pressure after the initial projection (solver.rs:1448)
        d_u, d_p = torch.from_numpy(u).to(dev), torch.from_numpy(p).to(dev)
        steps = 3
        for _ in range(steps):
            its += dg.step_device(d_u.data_ptr(), d_p.data_ptr(), 0.1, 1e-8, 10000).iterations
        torch.cuda.synchronize()
        dg.close()
        out = os.path.join(out_dir, f"device_archive_{form}")
        if os.path.exists(out):
            import shutil

            shutil.rmtree(out)
        A.write_run(out, case, g, d_u.cpu().numpy(), d_p.cpu().numpy(), steps=steps, time_s=0.1 * steps,
                    pressure_iterations=int(its))
        print(out)


def gas_case(pkg, advection="linear_upwind"):
    suffix = "" if advection == "linear_upwind" else "-" + advection
    case = pkg.synth.case((16, 12, 8), 2.0, inflow=3.0, boxes=[((10.0, 6.0, 0.0), (16.0, 14.0, 8.0))],
                          name="device-archive-gas-16x12x8" + suffix)
    case["output"]["fields"] = True
    case["numerics"]["transport"] = advection
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


def gas_archive(pkg, out_dir, advection="linear_upwind"):
    import torch
    from importlib import import_module

    A = import_module(pkg.__name__ + ".archive")
    S = import_module(pkg.__name__ + ".sources")
    R = import_module(pkg.__name__ + ".receptors")
    case = gas_case(pkg, advection)
    g = pkg.grid.Grid.build(case)
    dev = torch.device("cuda", 0)
    dg = pkg.pressure.DeviceGrid(g, preconditioner="multigrid", precision="mixed")
    dg.set_flow(case)
    dg.set_advection(case["numerics"]["transport"])
    u, p = g.initial_velocity(), np.zeros(g.count)
    its = dg.project(u, p, 1.0, 1e-8, 10000).iterations
    p[:] = 0.0
    d_u, d_p = torch.from_numpy(u).to(dev), torch.from_numpy(p).to(dev)
    d_s = torch.from_numpy(S.source_fields(case, g)[0]).to(dev)
    d_d = torch.from_numpy(S.diffusivity(case, 0, cells=g.count)).to(dev)
    d_c = torch.zeros(g.count, dtype=torch.float64, device=dev)
    d_b = torch.zeros(3, dtype=torch.float64, device=dev)
    steps, dt = 4, 0.1
    for _ in range(steps):
        its += dg.step_device(d_u.data_ptr(), d_p.data_ptr(), dt, 1e-8, 10000).iterations
        dg.scalar_step_budget(d_u.data_ptr(), d_c.data_ptr(), d_d.data_ptr(), d_s.data_ptr(), dt, d_b.data_ptr())
    rates = dg.scalar_rates(d_u.data_ptr(), d_c.data_ptr(), d_d.data_ptr(), d_s.data_ptr())
    dg.set_receptors([R.receptor_weights(g, r) for r in case["receptors"]])
    d_r = torch.zeros(len(case["receptors"]), dtype=torch.float64, device=dev)
    dg.sample_receptors(d_c.data_ptr(), d_r.data_ptr())
    torch.cuda.synchronize()
    b = d_b.cpu().numpy()
    entry = {"concentration": d_c.cpu().numpy(), "rates": rates,
             "receptors": {r["id"]: float(v) for r, v in zip(case["receptors"], d_r.cpu().numpy())},
             "budget": {"initial_kg": 0.0, "emitted_kg": float(b[0]), "inflow_kg": float(b[1]),
                        "outflow_kg": float(b[2])}}
    dg.close()
    out = os.path.join(out_dir, "device_archive_gas" + ("" if advection == "linear_upwind" else "_" + advection))
    if os.path.exists(out):
        import shutil

        shutil.rmtree(out)
    A.write_run(out, case, g, d_u.cpu().numpy(), d_p.cpu().numpy(), steps=steps, time_s=dt * steps,
                pressure_iterations=int(its), constituents=[entry])
    print(out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
    sys.path.insert(0, ROOT)
    import __graft_entry__ as entry

    for scheme in ("linear_upwind", "muscl"):
        gas_archive(entry.package(), sys.argv[1] if len(sys.argv) > 1 else HERE, scheme)
