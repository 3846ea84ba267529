"""Scalar transport on the device (cfdg_scalar_step_device): SSPRK2 steps of a constituent
with linear upwind advection, bit-identical to the oracle's sequential restatement of
advance_scalar (solver.rs:808-855) and rhs_into (transport.rs:651-699), and mass
conservation in a closed box at a larger size."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float64).view(np.uint64)


def flow_case(pkg, name):
    if name == "buildings-open-wall":
        return pkg.synth.case((24, 20, 12), 2.0, inflow=5.0, preconditioner="multigrid",
                              boxes=[((16.0, 10.0, 0.0), (26.0, 22.0, 10.0)), ((30.0, 4.0, 0.0), (36.0, 10.0, 16.0))])
    if name == "spacing-1.5m":  # face areas, distances and the volume not powers of two
        return pkg.synth.case((40, 14, 9), 1.5, inflow=4.0, preconditioner="multigrid",
                              boxes=[((15.0, 6.0, 0.0), (24.0, 15.0, 7.5))])
    if name == "wide-tiles":  # several x and y tiles, ragged in every axis
        return pkg.synth.case((70, 19, 11), 1.0, inflow=3.0, preconditioner="multigrid",
                              boxes=[((20.0, 5.0, 0.0), (31.0, 12.0, 6.0)), ((50.0, 0.0, 0.0), (64.0, 4.0, 9.0))])
    return pkg.synth.case((20, 12, 10), 1.0, boundaries=("open", "slip", "wall"), inflow=2.0,
                          preconditioner="ic0", boxes=[((6.0, 0.0, 0.0), (9.0, 5.0, 4.0))])


@pytest.mark.parametrize("name,perturb", [("buildings-open-wall", False), ("slip-channel", False),
                                          ("wide-tiles", False), ("spacing-1.5m", False),
                                          ("buildings-open-wall", True), ("wide-tiles", True)])
def test_scalar_steps_bit_identical(pkg, O, name, perturb):
    """perturb: face areas and distances scaled per face (the general gather that reads
    each face's lo, hi, area and distance); otherwise the structured fast path."""
    torch = pytest.importorskip("torch")
    case = flow_case(pkg, name)
    g = pkg.grid.Grid.build(case)
    og = O.Grid(case)
    rng = np.random.default_rng(11)
    # A projected flow with noise on the interior faces (backflow through the outlet included).
    code, u, _, _ = og.project(g.initial_velocity(), np.zeros(g.count), 0.1, 1e-8, 10000)
    assert code == 0
    u = u + np.where(g.face_kind == pkg.grid.INTERIOR, rng.uniform(-1.0, 1.0, g.n_faces), 0.0)
    u[g.face_kind == pkg.grid.OUTLET] *= rng.choice([1.0, -0.5], int((g.face_kind == pkg.grid.OUTLET).sum()))
    fluid = g.fluid.astype(bool)
    d = np.where(fluid, rng.uniform(0.01, 0.5, g.count), 0.0)
    source = np.zeros(g.count)
    src_cells = rng.choice(np.nonzero(fluid)[0], 5, replace=False)
    source[src_cells] = rng.uniform(1e-4, 1e-2, 5)
    c = np.where(fluid, rng.uniform(0.0, 1e-3, g.count), 0.0)
    dt = 0.02
    dg = pkg.pressure.DeviceGrid(g, preconditioner=case["numerics"]["pressure_preconditioner"])
    if perturb:
        area = np.asarray(g.face_area) * rng.uniform(0.8, 1.2, g.n_faces)
        dist = np.asarray(g.face_distance) * rng.uniform(0.9, 1.1, g.n_faces)
        og.set_faces(area, dist)
        dg.update_faces(area, dist)
    dev = torch.device("cuda", 0)
    d_u, d_c = torch.from_numpy(u.copy()).to(dev), torch.from_numpy(c.copy()).to(dev)
    d_d, d_s = torch.from_numpy(d).to(dev), torch.from_numpy(source).to(dev)
    ref = c.copy()
    for step in range(6):
        ref = og.scalar_step(ref, u, d, source, dt)
        dg.scalar_step_device(d_u.data_ptr(), d_c.data_ptr(), d_d.data_ptr(), d_s.data_ptr(), dt)
        torch.cuda.synchronize()
        got = d_c.cpu().numpy()
        assert np.array_equal(bits(got), bits(ref)), f"step {step}: max diff {np.max(np.abs(got - ref)):.3e}"
    dg.close()


@pytest.mark.parametrize("muscl", [False, True])
@pytest.mark.parametrize("name,perturb", [("wide-tiles", False), ("buildings-open-wall", False),
                                          ("spacing-1.5m", False), ("wide-tiles", True)])
def test_scalar_steps_extreme_values_bit_identical(pkg, O, name, perturb, muscl):
    """Signed zeros, subnormals and values near the top of the range in the concentration,
    diffusivity and source: the exponent-field products and the `+ 0.0` on bits must give
    the FP64 operations' bits there too; with MUSCL also the limiter's products by 0.5 and
    2, its minimum on the bits and its products a b that underflow to zero."""
    torch = pytest.importorskip("torch")
    case = flow_case(pkg, name)
    g = pkg.grid.Grid.build(case)
    og = O.Grid(case)
    rng = np.random.default_rng(5)
    u = np.where(np.isin(g.face_kind, (pkg.grid.INTERIOR, pkg.grid.INLET, pkg.grid.OUTLET)),
                 rng.uniform(-3.0, 3.0, g.n_faces), 0.0)
    pool = np.array([0.0, -0.0, 5e-324, -5e-324, 3e-310, -2.2e-308, 1e-300, 1.0, -7.5, 1e300, -3e299, 2.5e-16])
    c = rng.choice(pool, g.count)
    d = rng.choice(np.array([0.0, 1e-310, 0.1, 2.0, 1e-300]), g.count)
    source = rng.choice(np.array([0.0, -0.0, 1e-320, 1e-3, -1e290]), g.count)
    dt = 0.01
    dg = pkg.pressure.DeviceGrid(g, preconditioner="multigrid")
    if perturb:
        area = np.asarray(g.face_area) * rng.uniform(0.8, 1.2, g.n_faces)
        dist = np.asarray(g.face_distance) * rng.uniform(0.9, 1.1, g.n_faces)
        og.set_faces(area, dist)
        dg.update_faces(area, dist)
    dg.set_advection("muscl" if muscl else "linear_upwind")
    dev = torch.device("cuda", 0)
    d_u, d_c = torch.from_numpy(u).to(dev), torch.from_numpy(c.copy()).to(dev)
    d_d, d_s = torch.from_numpy(d).to(dev), torch.from_numpy(source).to(dev)
    ref = c.copy()
    for step in range(3):
        ref = og.scalar_step(ref, u, d, source, dt, muscl=muscl)
        dg.scalar_step_device(d_u.data_ptr(), d_c.data_ptr(), d_d.data_ptr(), d_s.data_ptr(), dt)
        torch.cuda.synchronize()
        got = d_c.cpu().numpy()
        assert np.all(np.isfinite(ref))
        bad = np.nonzero(bits(got) != bits(ref))[0]
        assert bad.size == 0, f"step {step}: {bad.size} cells differ, first {bad[:4]}: {got[bad[:4]]} vs {ref[bad[:4]]}"
    dg.close()


def test_scalar_mass_conserved_in_closed_box(pkg):
    """Walls on every side: no face leaves, so the mass grows by dt * emission per step."""
    torch = pytest.importorskip("torch")
    case = pkg.synth.case((96, 80, 48), 2.0, boundaries=("wall", "wall", "wall"), inflow=0.0,
                          preconditioner="multigrid", boxes=[((60.0, 40.0, 0.0), (90.0, 100.0, 50.0))])
    g = pkg.grid.Grid.build(case)
    rng = np.random.default_rng(3)
    interior = g.face_kind == pkg.grid.INTERIOR
    u = np.where(interior, rng.uniform(-2.0, 2.0, g.n_faces), 0.0)
    fluid = g.fluid.astype(bool)
    c = np.where(fluid, rng.uniform(0.0, 1.0, g.count), 0.0)
    source = np.where(fluid, rng.uniform(0.0, 1e-3, g.count), 0.0)
    d = np.where(fluid, 0.1, 0.0)
    dt = 0.01
    dg = pkg.pressure.DeviceGrid(g, preconditioner="multigrid")
    dev = torch.device("cuda", 0)
    d_u, d_c = torch.from_numpy(u).to(dev), torch.from_numpy(c.copy()).to(dev)
    d_d, d_s = torch.from_numpy(d).to(dev), torch.from_numpy(source).to(dev)
    steps = 20
    for _ in range(steps):
        dg.scalar_step_device(d_u.data_ptr(), d_c.data_ptr(), d_d.data_ptr(), d_s.data_ptr(), dt)
    torch.cuda.synchronize()
    dg.close()
    got = d_c.cpu().numpy()
    m0, m1 = c.sum() * g.volume, got.sum() * g.volume
    emitted = steps * dt * source.sum() * g.volume
    assert abs(m1 - (m0 + emitted)) <= 1e-11 * m1
    assert np.all(got[~fluid] == 0.0)


def test_receptor_values_bit_identical(pkg, O):
    """cfdg_receptors_sample after device transport steps: each receptor's value is the
    sum of c[cell] w in weight order (solver.rs:1035-1037), bit for bit."""
    torch = pytest.importorskip("torch")
    from importlib import import_module

    R = import_module(pkg.__name__ + ".receptors")
    case = flow_case(pkg, "wide-tiles")
    g = pkg.grid.Grid.build(case)
    og = O.Grid(case)
    code, u, _, _ = og.project(g.initial_velocity(), np.zeros(g.count), 0.1, 1e-8, 10000)
    assert code == 0
    fluid = g.fluid.astype(bool)
    rng = np.random.default_rng(9)
    d = np.where(fluid, 0.05, 0.0)
    source = np.zeros(g.count)
    source[np.nonzero(fluid)[0][:40]] = 1e-3
    receptors = [{"kind": "point", "point_m": [x, y, 3.3]} for x in (12.2, 40.0, 66.6) for y in (3.1, 9.5, 16.0)]
    receptors += [{"kind": "volume_average", "min_m": [35.2, 2.0, 0.5], "max_m": [48.7, 17.5, 6.0]},
                  {"kind": "point", "point_m": [0.2, 0.3, 10.8]}]
    weights = []
    for r in receptors:
        try:
            weights.append(R.receptor_weights(g, r))
        except R.ReceptorError:
            pass  # inside a building
    assert len(weights) >= 6
    dg = pkg.pressure.DeviceGrid(g, preconditioner="multigrid")
    dg.set_receptors(weights)
    dev = torch.device("cuda", 0)
    d_u, d_c = torch.from_numpy(u).to(dev), torch.zeros(g.count, dtype=torch.float64, device=dev)
    d_d, d_s = torch.from_numpy(d).to(dev), torch.from_numpy(source).to(dev)
    out = torch.empty(len(weights), dtype=torch.float64, device=dev)
    for _ in range(30):
        dg.scalar_step_device(d_u.data_ptr(), d_c.data_ptr(), d_d.data_ptr(), d_s.data_ptr(), 0.05)
    dg.sample_receptors(d_c.data_ptr(), out.data_ptr())
    torch.cuda.synchronize()
    c = d_c.cpu().numpy()
    ref = []
    for w in weights:
        acc = -0.0
        for cell, v in w:
            acc = acc + c[cell] * v
        ref.append(acc)
    got = out.cpu().numpy()
    dg.close()
    assert np.array_equal(bits(got), bits(np.array(ref))), (got, ref)
    assert np.count_nonzero(got) >= 3


@pytest.mark.parametrize("name", ["buildings-open-wall", "spacing-1.5m", "slip-channel"])
def test_scalar_budget_and_rates_match_oracle(pkg, O, name):
    """cfdg_scalar_step_budget: the concentration bit-identical to the step without budget,
    and the budget increments (emitted, inflow, outflow; solver.rs:851-853) over several
    steps within 1e-12 of the oracle's sequential sums; cfdg_scalar_rates: the current
    rates of rhs_into (transport.rs:651-699) within 1e-12."""
    torch = pytest.importorskip("torch")
    case = flow_case(pkg, name)
    g = pkg.grid.Grid.build(case)
    og = O.Grid(case)
    rng = np.random.default_rng(5)
    code, u, _, _ = og.project(g.initial_velocity(), np.zeros(g.count), 0.1, 1e-8, 10000)
    assert code == 0
    u = u + np.where(g.face_kind == pkg.grid.INTERIOR, rng.uniform(-0.5, 0.5, g.n_faces), 0.0)
    fluid = g.fluid.astype(bool)
    d = np.where(fluid, rng.uniform(0.01, 0.3, g.count), 0.0)
    source = np.zeros(g.count)
    source[rng.choice(np.nonzero(fluid)[0], 4, replace=False)] = rng.uniform(1e-4, 1e-2, 4)
    c = np.where(fluid, rng.uniform(0.0, 1e-3, g.count), 0.0)
    dt = 0.02
    dg = pkg.pressure.DeviceGrid(g, preconditioner=case["numerics"]["pressure_preconditioner"])
    dev = torch.device("cuda", 0)
    d_u, d_d, d_s = (torch.from_numpy(a.copy()).to(dev) for a in (u, d, source))
    d_c, d_c2 = torch.from_numpy(c.copy()).to(dev), torch.from_numpy(c.copy()).to(dev)
    d_b = torch.zeros(3, dtype=torch.float64, device=dev)
    budget = np.zeros(3)
    oc = c.copy()
    for _ in range(5):
        dg.scalar_step_budget(d_u.data_ptr(), d_c.data_ptr(), d_d.data_ptr(), d_s.data_ptr(), dt, d_b.data_ptr())
        dg.scalar_step_device(d_u.data_ptr(), d_c2.data_ptr(), d_d.data_ptr(), d_s.data_ptr(), dt)
        oc = og.scalar_step(oc, u, d, source, dt, budget)
    torch.cuda.synchronize()
    got_c = d_c.cpu().numpy()
    assert np.array_equal(bits(got_c), bits(d_c2.cpu().numpy()))
    assert np.array_equal(bits(got_c), bits(oc))
    got_b = d_b.cpu().numpy()
    scale = max(float(np.abs(budget).max()), 1e-300)
    assert np.all(np.abs(got_b - budget) <= 1e-12 * scale), (got_b, budget)
    rates = dg.scalar_rates(d_u.data_ptr(), d_c.data_ptr(), d_d.data_ptr(), d_s.data_ptr())
    orates = og.scalar_rates(oc, u, d, source)
    rscale = max(max(abs(v) for v in orates), 1e-300)
    assert all(abs(a - b) <= 1e-12 * rscale for a, b in zip(rates, orates)), (rates, orates)
    dg.close()


@pytest.mark.parametrize("name,perturb", [("buildings-open-wall", False), ("spacing-1.5m", False),
                                          ("wide-tiles", False), ("slip-channel", False), ("wide-tiles", True)])
def test_muscl_steps_budget_and_rates_bit_identical(pkg, O, name, perturb):
    """cfdg_grid_set_advection(1): SSPRK2 steps with MUSCL donors (transport.rs:502-526,
    670-694) bit-identical to the oracle's MUSCL step for several steps, the budget within
    1e-12 of the oracle's sequential sums, the rates of rhs_into within 1e-12; setting the
    advection back to linear upwind gives the linear-upwind bits; an unknown scheme is
    refused."""
    torch = pytest.importorskip("torch")
    case = flow_case(pkg, name)
    g = pkg.grid.Grid.build(case)
    og = O.Grid(case)
    rng = np.random.default_rng(21)
    code, u, _, _ = og.project(g.initial_velocity(), np.zeros(g.count), 0.1, 1e-8, 10000)
    assert code == 0
    u = u + np.where(g.face_kind == pkg.grid.INTERIOR, rng.uniform(-1.0, 1.0, g.n_faces), 0.0)
    u[g.face_kind == pkg.grid.OUTLET] *= rng.choice([1.0, -0.5], int((g.face_kind == pkg.grid.OUTLET).sum()))
    fluid = g.fluid.astype(bool)
    d = np.where(fluid, rng.uniform(0.01, 0.5, g.count), 0.0)
    source = np.zeros(g.count)
    source[rng.choice(np.nonzero(fluid)[0], 5, replace=False)] = rng.uniform(1e-4, 1e-2, 5)
    # Smooth and rough parts, so that limited, clipped and zero slopes all occur.
    x = np.arange(g.count) % g.n[0]
    c = np.where(fluid, 1e-3 * np.sin(0.3 * x) ** 2 + rng.uniform(0.0, 2e-4, g.count), 0.0)
    dt = 0.02
    dg = pkg.pressure.DeviceGrid(g, preconditioner=case["numerics"]["pressure_preconditioner"])
    if perturb:
        area = np.asarray(g.face_area) * rng.uniform(0.8, 1.2, g.n_faces)
        dist = np.asarray(g.face_distance) * rng.uniform(0.9, 1.1, g.n_faces)
        og.set_faces(area, dist)
        dg.update_faces(area, dist)
    with pytest.raises(ValueError):
        dg.set_advection("quick")
    assert dg.L.cfdg_grid_set_advection(dg.h, 2) == pkg.engine.CFDG_ERR_INVALID
    dg.set_advection("muscl")
    dev = torch.device("cuda", 0)
    d_u, d_d, d_s = (torch.from_numpy(a.copy()).to(dev) for a in (u, d, source))
    d_c = torch.from_numpy(c.copy()).to(dev)
    d_b = torch.zeros(3, dtype=torch.float64, device=dev)
    budget = np.zeros(3)
    ref = c.copy()
    for step in range(5):
        if step % 2:
            dg.scalar_step_budget(d_u.data_ptr(), d_c.data_ptr(), d_d.data_ptr(), d_s.data_ptr(), dt, d_b.data_ptr())
            ref = og.scalar_step(ref, u, d, source, dt, budget, muscl=True)
        else:
            dg.scalar_step_device(d_u.data_ptr(), d_c.data_ptr(), d_d.data_ptr(), d_s.data_ptr(), dt)
            ref = og.scalar_step(ref, u, d, source, dt, muscl=True)
        torch.cuda.synchronize()
        got = d_c.cpu().numpy()
        assert np.array_equal(bits(got), bits(ref)), f"step {step}: max diff {np.max(np.abs(got - ref)):.3e}"
    assert not np.array_equal(ref, og.scalar_step(c, u, d, source, dt))
    got_b = d_b.cpu().numpy()
    scale = max(float(np.abs(budget).max()), 1e-300)
    assert np.all(np.abs(got_b - budget) <= 1e-12 * scale), (got_b, budget)
    rates = dg.scalar_rates(d_u.data_ptr(), d_c.data_ptr(), d_d.data_ptr(), d_s.data_ptr())
    orates = og.scalar_rates(ref, u, d, source, muscl=True)
    rscale = max(max(abs(v) for v in orates), 1e-300)
    assert all(abs(a - b) <= 1e-12 * rscale for a, b in zip(rates, orates)), (rates, orates)
    dg.set_advection("linear_upwind")
    dg.scalar_step_device(d_u.data_ptr(), d_c.data_ptr(), d_d.data_ptr(), d_s.data_ptr(), dt)
    torch.cuda.synchronize()
    assert np.array_equal(bits(d_c.cpu().numpy()), bits(og.scalar_step(ref, u, d, source, dt)))
    dg.close()


@pytest.mark.parametrize("muscl", [False, True])
def test_transport_bench_workload_bit_identical(pkg, O, muscl):
    """The transport workload at its full size (128x128x64, 12 buildings, dx = 2 m: 1,024
    blocks of 4 slices on 152 SMs, the split the smaller grids above never take): two
    SSPRK2 steps on a flow with noise on the interior faces, bit-identical to the oracle's
    sequential step, linear upwind and MUSCL."""
    torch = pytest.importorskip("torch")
    case = pkg.synth.config2(seed=1)
    g = pkg.grid.Grid.build(case)
    og = O.Grid(case)
    rng = np.random.default_rng(31)
    u = g.initial_velocity()
    u = u + np.where(g.face_kind == pkg.grid.INTERIOR, rng.uniform(-1.0, 1.0, g.n_faces), 0.0)
    fluid = g.fluid.astype(bool)
    d = np.where(fluid, rng.uniform(0.05, 0.15, g.count), 0.0)
    source = np.zeros(g.count)
    source[rng.choice(np.nonzero(fluid)[0], 64, replace=False)] = 1e-3
    x = np.arange(g.count) % g.n[0]
    c = np.where(fluid, 1e-3 * np.cos(0.2 * x) ** 2 + rng.uniform(0.0, 1e-4, g.count), 0.0)
    dt = 0.05
    dg = pkg.pressure.DeviceGrid(g, preconditioner="multigrid")
    dg.set_advection("muscl" if muscl else "linear_upwind")
    dev = torch.device("cuda", 0)
    d_u, d_d, d_s = (torch.from_numpy(a.copy()).to(dev) for a in (u, d, source))
    d_c = torch.from_numpy(c.copy()).to(dev)
    ref = c.copy()
    for step in range(2):
        ref = og.scalar_step(ref, u, d, source, dt, muscl=muscl)
        dg.scalar_step_device(d_u.data_ptr(), d_c.data_ptr(), d_d.data_ptr(), d_s.data_ptr(), dt)
        torch.cuda.synchronize()
        got = d_c.cpu().numpy()
        bad = np.nonzero(bits(got) != bits(ref))[0]
        assert bad.size == 0, f"step {step}: {bad.size} cells differ, first {bad[:4]}"
    dg.close()
