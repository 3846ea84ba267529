"""The mixed form's error against the FP64 oracle on pressure, divergence and receptor
concentrations.

One seeded flow step of a 64x64x32 grid with buildings (inflow 5 m/s plus noise) is
projected by the FP64 oracle and by the engine's mixed form; a constituent released near
the inflow is then transported with the same linear-upwind restatement of the
reference (oracle/transport.py) on each projected flow, and the concentrations at point
receptors downstream are compared. Stated bounds: pressure and velocities 1e-7 relative
(as the mixed-form tests), receptor concentrations 1e-6 relative; the measured values are
printed.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_receptor_concentrations_mixed_vs_fp64(pkg, O):
    from oracle import transport as T

    rng = np.random.default_rng(31)
    case = pkg.synth.case((64, 64, 32), 2.0, inflow=5.0, preconditioner="multigrid",
                          boxes=pkg.synth.random_boxes(rng, 6, (128.0, 128.0, 64.0), side=(10.0, 24.0),
                                                       height=(10.0, 40.0), dx=2.0))
    g = pkg.grid.Grid.build(case)
    og = O.Grid(case)
    # u*: the inflow speed along x on the free faces plus 10 % noise, boundary values enforced.
    free = (g.face_kind == pkg.grid.INTERIOR) | (g.face_kind == pkg.grid.OUTLET)
    u = np.where(free & (g.face_axis == 0), 5.0, 0.0) + np.where(free, rng.uniform(-0.5, 0.5, g.n_faces), 0.0)
    g.enforce_velocity(u)
    dt, tol = 0.1, 1e-8
    code, ou, op, _ = og.project(u, np.zeros(g.count), dt, tol, 10000)
    assert code == 0
    dg = pkg.pressure.DeviceGrid(g, preconditioner="multigrid", precision="mixed")
    mu, mp = u.copy(), np.zeros(g.count)
    info = dg.project(mu, mp, dt, tol, 10000)
    dg.close()
    assert info.relative_residual <= tol
    ep = np.max(np.abs(mp - op)) / np.max(np.abs(op))
    eu = np.max(np.abs(mu - ou)) / np.max(np.abs(ou))
    div_ref = np.max(np.abs(og.divergence(ou)))
    div_mix = np.max(np.abs(og.divergence(mu)))
    div0 = np.max(np.abs(og.divergence(u)))
    # The release: 1e-3 kg/m3/s in one fluid cell near the inflow at 5 m height.
    fluid = g.fluid.astype(bool)
    src = np.zeros(g.count)
    nx, ny = g.n[0], g.n[1]
    for i in range(2, nx):
        c = (2 * ny + ny // 2) * nx + i
        if fluid[c]:
            src[c] = 1e-3
            break
    assert src.sum() > 0
    tr = T.Transport(g, diffusivity=0.05)
    dts = min(tr.stable_dt(ou), tr.stable_dt(mu))
    steps = int(np.ceil(20.0 / dts))  # 20 s of transport: the plume crosses most of the domain
    c_ref = tr.run(ou, src, steps, dts)
    c_mix = tr.run(mu, src, steps, dts)
    errs = []
    for x in (40.0, 70.0, 100.0):
        for y in (48.0, 64.0, 80.0):
            p = (x, y, 5.0)
            w = T.point_weights(g, p)
            if any(not fluid[i] for i, _ in w):
                continue  # receptor inside a building
            r = T.sample(c_ref, w)
            if r <= 1e-12:
                continue  # not reached by the plume
            errs.append(abs(T.sample(c_mix, w) - r) / r)
    assert len(errs) >= 3
    print(f"mixed vs FP64: pressure {ep:.2e}, velocity {eu:.2e}, max|div| {div_mix:.2e} (FP64 {div_ref:.2e}, "
          f"before {div0:.2e}), receptors max {max(errs):.2e} over {len(errs)} receptors, {steps} transport steps")
    assert ep <= 1e-7 and eu <= 1e-7
    assert div_mix <= 1e-6 * div0
    assert max(errs) <= 1e-6
