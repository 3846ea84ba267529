"""Failure paths of the projection on the device, made on the host (no GPU fault).

* CFD-E032, lost positive definiteness (pressure.rs:394-395): a NaN face velocity seeded
  on the host makes p.Ap non-finite in the first iteration. The reference and the oracle
  return E032; the engine must return 32 in the plain form (IC(0) and multigrid), the
  mixed form and inside a server, with the caller's u and p unchanged
  (pressure.rs:468; tests/urban_pressure_reference.rs:225-262), while the other
  requests of the server complete.
* CFDG_ERR_TIMEOUT, a bounded device wait that gives up: one wavefront tile is told never
  to publish its progress (cfdg_debug_wave_stall), so the tiles that wait for it give up
  after a short, bounded number of polls. The call returns CFDG_ERR_TIMEOUT with u and
  p unchanged, and the same grid solves normally once the hook is cleared.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
DT, TOL = 0.1, 1e-8


def bits(a):
    return np.ascontiguousarray(a, np.float64).view(np.uint64)


def nan_case(pkg):
    return pkg.synth.case((24, 20, 16), 2.0, inflow=5.0, preconditioner="multigrid",
                          boxes=[((10.0, 8.0, 0.0), (22.0, 20.0, 12.0))])


def nan_inputs(pkg, g):
    u = pkg.synth.random_velocity(g, seed=9)
    interior = np.flatnonzero(g.face_kind == pkg.grid.INTERIOR)
    u[interior[len(interior) // 3]] = np.nan
    p = np.random.default_rng(2).uniform(-1, 1, g.count) * (g.fluid == 1)
    return u, p


@pytest.mark.parametrize("pre,precision", [("ic0", "plain"), ("multigrid", "plain"), ("multigrid", "mixed")])
def test_nan_right_hand_side_is_e032_and_leaves_fields(pkg, O, pre, precision):
    case = nan_case(pkg)
    g = pkg.grid.Grid.build(case)
    assert all(g.anchored)  # the compatibility check (E031) does not apply
    u, p = nan_inputs(pkg, g)
    og = O.Grid(case)
    og.set_preconditioner(pre)
    code, _, _, _ = og.project(u, p, DT, TOL, 1000)
    assert code == 32
    dg = pkg.pressure.DeviceGrid(g, preconditioner=pre, precision=precision)
    uu, pp = u.copy(), p.copy()
    with pytest.raises(pkg.pressure.PressureError) as e:
        dg.project(uu, pp, DT, TOL, 1000)
    assert e.value.code == 32 and str(e.value).startswith("CFD-E032"), (e.value.code, str(e.value))
    assert np.array_equal(bits(uu), bits(u)) and np.array_equal(bits(pp), bits(p))
    # The grid is still usable: a finite request projects like the oracle.
    uf = pkg.synth.random_velocity(g, seed=10)
    _, ou, op, _ = og.project(uf, p, DT, TOL, 1000)
    uu, pp = uf.copy(), p.copy()
    dg.project(uu, pp, DT, TOL, 1000)
    bar = 1e-10 if precision == "plain" else 1e-7
    assert np.max(np.abs(uu - ou)) <= bar * np.max(np.abs(ou))
    dg.close()


def test_nan_request_in_server_is_e032_and_others_complete(pkg):
    import torch

    dev = torch.device("cuda", 0)
    cases = [nan_case(pkg), pkg.synth.case((20, 16, 12), 2.0, inflow=5.0, preconditioner="multigrid")]
    grids = [pkg.grid.Grid.build(c) for c in cases]
    u_bad, p_bad = nan_inputs(pkg, grids[0])
    u_ok = pkg.synth.random_velocity(grids[1], seed=12)
    p_ok = np.zeros(grids[1].count)
    # The good request alone, for comparison.
    alone = pkg.pressure.DeviceGrid(grids[1], preconditioner="multigrid", precision="mixed")
    ua, pa = u_ok.copy(), p_ok.copy()
    alone.project(ua, pa, DT, TOL, 1000)
    alone.close()
    dgs = [pkg.pressure.DeviceGrid(g, preconditioner="multigrid", precision="mixed") for g in grids]
    server = pkg.pressure.Server(dgs, max_active=2)
    d_u = [torch.from_numpy(u_bad.copy()).to(dev), torch.from_numpy(u_ok.copy()).to(dev)]
    d_p = [torch.from_numpy(p_bad.copy()).to(dev), torch.from_numpy(p_ok.copy()).to(dev)]
    torch.cuda.synchronize()
    tickets = [server.submit(i, d_u[i].data_ptr(), d_p[i].data_ptr(), DT, TOL, 1000) for i in range(2)]
    done = {}
    for _ in range(100000):
        server.progress()
        for i, t in enumerate(tickets):
            if i not in done and (r := server.result(t)) is not None:
                done[i] = r
        if len(done) == 2:
            break
    assert done[0][0] == 32 and done[1][0] == 0, (done[0][0], done[1][0])
    assert np.array_equal(bits(d_u[0].cpu().numpy()), bits(u_bad))
    assert np.array_equal(bits(d_p[0].cpu().numpy()), bits(p_bad))
    assert np.array_equal(bits(d_u[1].cpu().numpy()), bits(ua))
    assert np.array_equal(bits(d_p[1].cpu().numpy()), bits(pa))
    server.close()
    for d in dgs:
        d.close()


def test_wavefront_wait_that_gives_up_is_a_timeout(pkg, O):
    """IC(0) on a structured grid runs the pipelined wavefront sweeps (8 x 8 pencils per
    tile: 3 x 2 tiles here). Tile 0 holds back its progress; tiles 1 and 3 wait for it,
    give up after 4096 polls and raise the sweep's abort flag."""
    case = pkg.synth.case((24, 20, 16), 1.0, preconditioner="ic0")
    g = pkg.grid.Grid.build(case)
    og = O.Grid(case)
    dg = pkg.pressure.DeviceGrid(g, preconditioner="ic0")
    u = pkg.synth.random_velocity(g, seed=4)
    p = np.zeros(g.count)
    dg.wave_stall(0, 4096)
    r = np.where(g.fluid == 1, np.sin(0.3 * np.arange(g.count)), 0.0)
    with pytest.raises(pkg.pressure.PressureError) as e:
        dg.precondition(r)
    assert e.value.code == 202
    uu, pp = u.copy(), p.copy()
    with pytest.raises(pkg.pressure.PressureError) as e:
        dg.project(uu, pp, DT, TOL, 40)
    assert e.value.code == 202
    assert np.array_equal(bits(uu), bits(u)) and np.array_equal(bits(pp), bits(p))
    # Out-of-range settings are refused.
    with pytest.raises(pkg.pressure.PressureError) as e:
        dg.wave_stall(6, 4096)
    assert e.value.code == 203
    # Cleared: the same grid and context project like the oracle again.
    dg.wave_stall(-1, 1 << 22)
    assert np.array_equal(bits(dg.precondition(r)), bits(og.ic0_apply(r)))
    code, ou, op, oinfo = og.project(u, p, DT, TOL, 10000)
    info = dg.project(uu, pp, DT, TOL, 10000)
    assert abs(info.iterations - oinfo["iterations"]) <= 1
    assert np.max(np.abs(uu - ou)) <= 1e-10 * max(1.0, np.max(np.abs(ou)))
    dg.close()
