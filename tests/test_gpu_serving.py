"""Continuous batching (cfdg_server): requests arriving while others run are admitted at
chunk boundaries, and every result equals the same request solved alone, bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float64).view(np.uint64)


def test_server_results_equal_alone(pkg):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(7)
    shapes = [(32, 32, 16), (40, 24, 16), (24, 24, 24), (48, 32, 16), (32, 32, 16)]
    cases = [pkg.synth.case(sh, 2.0, inflow=5.0, preconditioner="multigrid",
                            boxes=pkg.synth.random_boxes(rng, 3, [v * 2.0 for v in sh], side=(6.0, 14.0),
                                                         height=(6.0, 20.0), dx=2.0)) for sh in shapes]
    grids = [pkg.grid.Grid.build(c) for c in cases]
    dev = torch.device("cuda", 0)
    # Three time steps per grid, perturbing the velocity between steps.
    steps = 3
    u0 = [pkg.synth.random_velocity(g, 30 + i) for i, g in enumerate(grids)]
    noise = [[np.where((g.face_kind == pkg.grid.INTERIOR) | (g.face_kind == pkg.grid.OUTLET),
                       np.random.default_rng(100 * i + s).uniform(-0.05, 0.05, g.n_faces), 0.0)
              for s in range(steps)] for i, g in enumerate(grids)]
    # Alone: one mixed-form solve per step, sequentially.
    alone_u, alone_p = [], []
    for i, g in enumerate(grids):
        dg = pkg.pressure.DeviceGrid(g, preconditioner="multigrid", precision="mixed")
        u, p = u0[i].copy(), np.zeros(g.count)
        us, ps = [], []
        for s in range(steps):
            u = u + noise[i][s]
            dg.project(u, p, 0.1, 1e-8, 10000)
            us.append(u.copy())
            ps.append(p.copy())
        alone_u.append(us)
        alone_p.append(ps)
        dg.close()
    # Served: all grids resident, at most 3 running at once, requests interleaved.
    dgs = [pkg.pressure.DeviceGrid(g, preconditioner="multigrid", precision="mixed") for g in grids]
    server = pkg.pressure.Server(dgs, max_active=3)
    d_u = [torch.from_numpy(u0[i]).to(dev) for i in range(len(grids))]
    d_p = [torch.zeros(g.count, dtype=torch.float64, device=dev) for g in grids]
    torch.cuda.synchronize()
    step_of = [0] * len(grids)
    inflight = {}
    order = [i for s in range(steps) for i in range(len(grids))]
    rng2 = np.random.default_rng(3)
    pending = list(order)
    while pending or inflight:
        # Submit a random number of ready requests (a grid's next step after its previous one).
        for _ in range(int(rng2.integers(0, 3))):
            ready = [i for i in pending if i not in inflight]
            if not ready:
                break
            i = ready[0]
            pending.remove(i)
            d_u[i].add_(torch.from_numpy(noise[i][step_of[i]]).to(dev))
            torch.cuda.synchronize()
            inflight[i] = server.submit(i, d_u[i].data_ptr(), d_p[i].data_ptr(), 0.1, 1e-8, 10000)
        server.progress()
        for i, t in list(inflight.items()):
            r = server.result(t)
            if r is None:
                continue
            code, info = r
            assert code == 0
            torch.cuda.synchronize()
            s = step_of[i]
            assert np.array_equal(bits(d_u[i].cpu().numpy()), bits(alone_u[i][s])), (i, s)
            assert np.array_equal(bits(d_p[i].cpu().numpy()), bits(alone_p[i][s])), (i, s)
            step_of[i] += 1
            del inflight[i]
    assert step_of == [steps] * len(grids)
    assert server.pending() == 0
    server.close()
    for d in dgs:
        d.close()


def test_cycle_settings_chunks_and_autotune(pkg):
    """Sweep counts set on the grids apply alike to solo solves, batches and servers (same
    bits), a server with a shorter chunk gives the same results, and the autotuner applies
    its fastest candidate."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(9)
    shapes = [(32, 32, 16), (48, 32, 16)]
    cases = [pkg.synth.case(sh, 2.0, inflow=5.0, preconditioner="multigrid",
                            boxes=pkg.synth.random_boxes(rng, 3, [v * 2.0 for v in sh], side=(6.0, 14.0),
                                                         height=(6.0, 20.0), dx=2.0)) for sh in shapes]
    grids = [pkg.grid.Grid.build(c) for c in cases]
    us = [pkg.synth.random_velocity(g, 60 + i) for i, g in enumerate(grids)]
    dev = torch.device("cuda", 0)
    alone = []
    for g, u in zip(grids, us):
        dg = pkg.pressure.DeviceGrid(g, preconditioner="multigrid", precision="mixed")
        dg.set_cycle(1, 3)
        uu, pp = u.copy(), np.zeros(g.count)
        info = dg.project(uu, pp, 0.1, 1e-8, 10000)
        assert info.relative_residual <= 1e-8
        alone.append((uu, pp, info.iterations))
        dg.close()
    dgs = [pkg.pressure.DeviceGrid(g, preconditioner="multigrid", precision="mixed") for g in grids]
    for d in dgs:
        d.set_cycle(1, 3)
    batch = pkg.pressure.Batch(dgs)
    bu, bp = [u.copy() for u in us], [np.zeros(g.count) for g in grids]
    res = batch.project(bu, bp, [0.1, 0.1], 1e-8, 10000)
    batch.close()
    for i, (code, info) in enumerate(res):
        assert code == 0 and info.iterations == alone[i][2]
        assert np.array_equal(bits(bu[i]), bits(alone[i][0])) and np.array_equal(bits(bp[i]), bits(alone[i][1]))
    server = pkg.pressure.Server(dgs, max_active=2)
    server.set_chunk(3)
    d_u = [torch.from_numpy(u).to(dev) for u in us]
    d_p = [torch.zeros(g.count, dtype=torch.float64, device=dev) for g in grids]
    torch.cuda.synchronize()
    tickets = [server.submit(i, d_u[i].data_ptr(), d_p[i].data_ptr(), 0.1, 1e-8, 10000) for i in range(2)]
    done = {}
    for _ in range(100000):
        server.progress()
        for i, t in enumerate(tickets):
            if i not in done:
                r = server.result(t)
                if r is not None:
                    done[i] = r
        if len(done) == 2:
            break
    assert len(done) == 2
    st = server.stats()
    assert st["iterations_per_chunk"] == 3 and st["finished"] == 2
    for i in range(2):
        assert done[i][0] == 0
        assert np.array_equal(bits(d_u[i].cpu().numpy()), bits(alone[i][0]))
        assert np.array_equal(bits(d_p[i].cpu().numpy()), bits(alone[i][1]))
    server.close()
    # Autotuning over two candidates picks the faster and sets it on the grids.
    d_u0 = [u.clone() for u in d_u]

    def reset():
        for u, u0, p in zip(d_u, d_u0, d_p):
            u.copy_(u0)
            p.zero_()

    out = pkg.pressure.autotune(dgs, [u.data_ptr() for u in d_u], [p.data_ptr() for p in d_p], reset, [0.1, 0.1],
                                candidates=((2, 2), (1, 2)))
    assert tuple(out["choice"]) in ((2, 2), (1, 2)) and len(out["ms"]) == 2
    best = min(out["ms"], key=out["ms"].get)
    assert best == "%d,%d" % tuple(out["choice"])
    for d in dgs:
        d.close()


def test_admission_by_hbm_budget_and_failed_requests(pkg):
    """Grids are admitted against the context's HBM budget (CFDG_ERR_ADMISSION beyond it,
    room again after a grid closes); a request that fails (E031, an inflow into a sealed
    region) returns its code with its arrays untouched while the others complete."""
    torch = pytest.importorskip("torch")
    case = pkg.synth.case((24, 24, 12), 1.0, preconditioner="multigrid")
    g = pkg.grid.Grid.build(case)
    probe = pkg.pressure.DeviceGrid(g, preconditioner="multigrid", precision="mixed")
    one = probe.device_bytes()
    probe.close()
    assert one > 0
    ctx = pkg.pressure.Context(0, hbm_budget_bytes=int(2.5 * one))
    a = pkg.pressure.DeviceGrid(g, ctx=ctx, preconditioner="multigrid", precision="mixed")
    b = pkg.pressure.DeviceGrid(g, ctx=ctx, preconditioner="multigrid", precision="mixed")
    with pytest.raises(pkg.pressure.PressureError) as e:
        pkg.pressure.DeviceGrid(g, ctx=ctx, preconditioner="multigrid", precision="mixed")
    assert e.value.code == pkg.engine.CFDG_ERR_ADMISSION
    a.close()
    c = pkg.pressure.DeviceGrid(g, ctx=ctx, preconditioner="multigrid", precision="mixed")
    b.close()
    c.close()
    ctx.close()
    # A failing request next to a good one in one server.
    bad = pkg.grid.Grid.build(pkg.synth.case((24, 12, 8), 1.0, preconditioner="multigrid",
                                             boxes=[((8, 0, 0), (9, 12, 8))]))
    good = pkg.grid.Grid.build(pkg.synth.case((32, 16, 16), 1.0, preconditioner="multigrid"))
    ub, ug = pkg.synth.random_velocity(bad, 1), pkg.synth.random_velocity(good, 2)
    dgood = pkg.pressure.DeviceGrid(good, preconditioner="multigrid", precision="mixed")
    au, ap = ug.copy(), np.zeros(good.count)
    dgood.project(au, ap, 0.1, 1e-8, 10000)
    dgs = [pkg.pressure.DeviceGrid(bad, preconditioner="multigrid", precision="mixed"), dgood]
    server = pkg.pressure.Server(dgs, max_active=2)
    dev = torch.device("cuda", 0)
    d_u = [torch.from_numpy(ub).to(dev), torch.from_numpy(ug).to(dev)]
    d_p = [torch.full((bad.count,), 7.0, dtype=torch.float64, device=dev),
           torch.zeros(good.count, dtype=torch.float64, device=dev)]
    torch.cuda.synchronize()
    tickets = [server.submit(i, d_u[i].data_ptr(), d_p[i].data_ptr(), 0.1, 1e-8, 10000) for i in range(2)]
    done = {}
    for _ in range(100000):
        server.progress()
        for i, t in enumerate(tickets):
            if i not in done:
                r = server.result(t)
                if r is not None:
                    done[i] = r
        if len(done) == 2:
            break
    assert done[0][0] == 31 and done[1][0] == 0
    assert np.array_equal(bits(d_u[0].cpu().numpy()), bits(ub))
    assert np.all(d_p[0].cpu().numpy() == 7.0)
    assert np.array_equal(bits(d_u[1].cpu().numpy()), bits(au))
    assert np.array_equal(bits(d_p[1].cpu().numpy()), bits(ap))
    server.close()
    for d in dgs:
        d.close()
