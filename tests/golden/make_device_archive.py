"""Writes run archives of laminar steps computed on the device, as fixtures for the
reference's own archive checker (validation/check_fields.py), which the CPU tests run
on them (tests/test_device_archive.py).

    python tests/golden/make_device_archive.py [OUT_DIR]

Needs a CUDA device and the built engine. For each arithmetic form (plain FP64, mixed
FP32/FP64) it projects the initial state of a 16x10x8 laminar case with one building
(dt = 1, like the solver's start, solver.rs:1436-1445), runs three SSPRK2 steps of
dt = 0.1 s with cfdg_step_device (a projection per stage), copies the fields back and
writes the archive with the package's writer (output.rs:162-242 format) into
OUT_DIR/device_archive_<form> (default: this directory).
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


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
