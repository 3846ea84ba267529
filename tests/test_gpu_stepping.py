"""Laminar time stepping on the device (cfdg_step_device): the momentum right-hand side
and stage update bit-identical to the reference algorithm (the oracle's restatement of
flow.rs:426-525 and solver.rs:671-732), and SSPRK2 steps with a projection per stage
matching the oracle's steps (plain form: 1e-10 relative, the parity bar of a projection;
mixed form: 1e-7)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float64).view(np.uint64)


def cases(pkg):
    return {
        "building-open-wall": pkg.synth.case((24, 16, 12), 2.0, inflow=5.0, preconditioner="multigrid",
                                             boxes=[((16.0, 10.0, 0.0), (26.0, 20.0, 10.0))]),
        "slip-channel-ic0": pkg.synth.case((20, 12, 10), 1.0, boundaries=("open", "slip", "wall"), inflow=2.0,
                                           preconditioner="ic0", boxes=[((6.0, 0.0, 0.0), (9.0, 5.0, 4.0))]),
    }


@pytest.mark.parametrize("name", ["building-open-wall", "slip-channel-ic0"])
def test_momentum_update_bit_identical(pkg, O, name):
    case = cases(pkg)[name]
    case["flow"]["acceleration_m_s2"] = [0.01, 0.0, -0.002]
    g = pkg.grid.Grid.build(case)
    og = O.Grid(case)
    rng = np.random.default_rng(5)
    u = g.initial_velocity() + np.where(g.face_kind == pkg.grid.INTERIOR, rng.uniform(-1, 1, g.n_faces), 0.0)
    g.enforce_velocity(u)
    p = rng.uniform(-3, 3, g.count) * g.fluid
    dt = 0.05
    ref = u + dt * (og.momentum_rhs(u) - og.gradient(p))
    ref = og.enforce_velocity(ref)
    dg = pkg.pressure.DeviceGrid(g, preconditioner=case["numerics"]["pressure_preconditioner"])
    dg.set_flow(case)
    out = dg.momentum_update(u, p, dt)
    dg.close()
    assert np.array_equal(bits(out), bits(ref))


@pytest.mark.parametrize("name,precision,bound", [("building-open-wall", "plain", 1e-10),
                                                  ("slip-channel-ic0", "plain", 1e-10),
                                                  ("building-open-wall", "mixed", 1e-7)])
def test_ssprk2_steps_against_oracle(pkg, O, name, precision, bound):
    torch = pytest.importorskip("torch")
    case = cases(pkg)[name]
    g = pkg.grid.Grid.build(case)
    og = O.Grid(case)
    dt, tol = 0.1, 1e-8
    u, p = g.initial_velocity(), np.zeros(g.count)
    code, u, p, _ = og.project(u, p, dt, tol, 10000)  # the initial projection (solver.rs:1437)
    assert code == 0
    dg = pkg.pressure.DeviceGrid(g, preconditioner=case["numerics"]["pressure_preconditioner"], precision=precision)
    dg.set_flow(case)
    dev = torch.device("cuda", 0)
    d_u, d_p = torch.from_numpy(u.copy()).to(dev), torch.from_numpy(p.copy()).to(dev)
    torch.cuda.synchronize()
    ou, op = u, p
    for s in range(4):
        code, ou, op, oit = og.step(ou, op, dt, tol, 10000)
        assert code == 0
        info = dg.step_device(d_u.data_ptr(), d_p.data_ptr(), dt, tol, 10000)
        gu, gp = d_u.cpu().numpy(), d_p.cpu().numpy()
        eu = np.max(np.abs(gu - ou)) / np.max(np.abs(ou))
        ep = np.max(np.abs(gp - op)) / max(np.max(np.abs(op)), 1e-300)
        assert eu <= bound and ep <= bound, (s, eu, ep)
        if precision == "plain":
            assert abs(int(info.iterations) - int(oit)) <= 2, (info.iterations, oit)
    # The stepped flow stays divergence-free.
    assert np.max(np.abs(og.divergence(d_u.cpu().numpy()))) <= 1e-6 * 5.0 / min(g.dx)
    dg.close()


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_archive_of_device_steps(pkg, O, precision, tmp_path):
    """Laminar steps on the device archived in CFD-craft's run-archive format (the package's
    archive writer, output.rs:162-242): the restated checks of validation/check_fields.py
    pass on the device fields (hashes, mask, finiteness, independent local continuity)."""
    torch = pytest.importorskip("torch")
    from importlib import import_module

    from archive_check import check_archive

    A = import_module(pkg.__name__ + ".archive")
    case = cases(pkg)["building-open-wall"]
    g = pkg.grid.Grid.build(case)
    dg = pkg.pressure.DeviceGrid(g, preconditioner=case["numerics"]["pressure_preconditioner"], precision=precision)
    dg.set_flow(case)
    u, p = g.initial_velocity(), np.zeros(g.count)
    its = dg.project(u, p, 0.1, 1e-8, 10000).iterations
    dev = torch.device("cuda", 0)
    d_u, d_p = torch.from_numpy(u).to(dev), torch.from_numpy(p).to(dev)
    for _ in range(3):
        its += dg.step_device(d_u.data_ptr(), d_p.data_ptr(), 0.1, 1e-8, 10000).iterations
    torch.cuda.synchronize()
    dg.close()
    out = tmp_path / f"run-{precision}"
    A.write_run(str(out), case, g, d_u.cpu().numpy(), d_p.cpu().numpy(), steps=3, time_s=0.3,
                pressure_iterations=int(its))
    max_div = check_archive(out, lambda c: pkg.grid.Grid.build(c).fluid.astype(bool))
    print(f"{precision}: archived after 3 device steps, independent max |div u| {max_div:.2e} 1/s")
