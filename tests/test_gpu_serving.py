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


def test_host_buffer_requests_equal_device_requests(pkg):
    """cfdg_server_submit_host: the fields stay in host memory (page-locked for two grids,
    ordinary pageable numpy memory for the third); the engine copies them to a device slot,
    runs the request and copies the results back before the ticket reports done. Two
    consecutive requests per grid (both device slots, the second fed with the first's
    results plus a perturbation) give the same bits as the same requests submitted on
    device arrays to another server; a failing request (E031) returns its inputs unchanged."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(9)
    shapes = [(32, 32, 16), (40, 24, 16), (24, 24, 24)]
    cases = [pkg.synth.case(sh, 2.0, inflow=5.0, preconditioner="multigrid",
                            boxes=pkg.synth.random_boxes(rng, 2, [v * 2.0 for v in sh], side=(6.0, 14.0),
                                                         height=(6.0, 20.0), dx=2.0)) for sh in shapes]
    cases.append(pkg.synth.case((24, 12, 8), 1.0, preconditioner="multigrid", boxes=[((8, 0, 0), (9, 12, 8))]))
    grids = [pkg.grid.Grid.build(c) for c in cases]
    n = len(grids)
    dev = torch.device("cuda", 0)
    u0 = [pkg.synth.random_velocity(g, 50 + i) for i, g in enumerate(grids)]
    noise = [np.where((g.face_kind == pkg.grid.INTERIOR) | (g.face_kind == pkg.grid.OUTLET),
                      np.random.default_rng(200 + i).uniform(-0.05, 0.05, g.n_faces), 0.0) for i, g in enumerate(grids)]

    def run(server, submit):
        us, ps = [u.copy() for u in u0], [np.zeros(g.count) for g in grids]
        outs = []
        for step in range(2):
            tickets = [submit(server, i, us[i], ps[i]) for i in range(n)]
            got = [None] * n
            for _ in range(1_000_000):
                server.progress()
                for i, (t, fetch) in enumerate(tickets):
                    if got[i] is None and (r := server.result(t)) is not None:
                        got[i] = (r[0],) + fetch()
                if all(x is not None for x in got):
                    break
            outs.append(got)
            us = [got[i][1] + noise[i] if got[i][0] == 0 else got[i][1] for i in range(n)]
            ps = [got[i][2] for i in range(n)]
        return outs

    keep = []

    def dev_submit(server, i, u, p):
        du, dp = torch.from_numpy(u.copy()).to(dev), torch.from_numpy(p.copy()).to(dev)
        torch.cuda.synchronize()
        keep.append((du, dp))
        t = server.submit(i, du.data_ptr(), dp.data_ptr(), 0.1, 1e-8, 10000)
        return t, lambda: (du.cpu().numpy(), dp.cpu().numpy())

    def host_submit(server, i, u, p):
        if i == 2:  # pageable numpy buffers
            hu, hp = u.copy(), p.copy()
            ou, op = np.empty_like(hu), np.empty_like(hp)
            ptrs = [a.ctypes.data for a in (hu, hp, ou, op)]
            keep.append((hu, hp, ou, op))
            t = server.submit_host(i, *ptrs, 0.1, 1e-8, 10000)
            return t, lambda: (ou.copy(), op.copy())
        hu, hp = torch.from_numpy(u.copy()).pin_memory(), torch.from_numpy(p.copy()).pin_memory()
        ou, op = torch.empty_like(hu).pin_memory(), torch.empty_like(hp).pin_memory()
        keep.append((hu, hp, ou, op))
        t = server.submit_host(i, hu.data_ptr(), hp.data_ptr(), ou.data_ptr(), op.data_ptr(), 0.1, 1e-8, 10000)
        return t, lambda: (ou.numpy().copy(), op.numpy().copy())

    results = []
    for submit in (dev_submit, host_submit):
        dgs = [pkg.pressure.DeviceGrid(g, preconditioner="multigrid", precision="mixed") for g in grids]
        server = pkg.pressure.Server(dgs, max_active=n)
        results.append(run(server, submit))
        server.close()
        for d in dgs:
            d.close()
    dev_out, host_out = results
    for step in range(2):
        for i in range(n):
            assert dev_out[step][i][0] == host_out[step][i][0], (step, i)
            assert np.array_equal(bits(dev_out[step][i][1]), bits(host_out[step][i][1])), (step, i)
            assert np.array_equal(bits(dev_out[step][i][2]), bits(host_out[step][i][2])), (step, i)
        assert host_out[step][n - 1][0] == 31
        assert all(host_out[step][i][0] == 0 for i in range(n - 1))
    assert np.array_equal(bits(host_out[0][n - 1][1]), bits(u0[n - 1]))  # the failed request's inputs


def test_host_buffer_requests_two_in_flight_per_grid(pkg):
    """Two host requests of one grid in flight at once (both device slots): the second's
    input copy overlaps the first's solve, a third before either finished is refused
    (CFDG_ERR_INVALID), and once the first is done its slot takes the third. Each result
    equals the same input served alone on device arrays, bit for bit."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(31)
    shapes = [(32, 32, 16), (24, 40, 16)]
    cases = [pkg.synth.case(sh, 2.0, inflow=5.0, preconditioner="multigrid",
                            boxes=pkg.synth.random_boxes(rng, 2, [v * 2.0 for v in sh], side=(6.0, 14.0),
                                                         height=(6.0, 20.0), dx=2.0)) for sh in shapes]
    grids = [pkg.grid.Grid.build(c) for c in cases]
    n = len(grids)
    dev = torch.device("cuda", 0)
    inputs = [[pkg.synth.random_velocity(g, 300 + 10 * i + k) for k in range(3)] for i, g in enumerate(grids)]

    def drain(server, tickets):
        out = {}
        for _ in range(1_000_000):
            server.progress()
            for t in tickets:
                if t not in out and (r := server.result(t)) is not None:
                    out[t] = r[0]
            if len(out) == len(tickets):
                return out
        raise AssertionError("requests did not finish")

    dgs = [pkg.pressure.DeviceGrid(g, preconditioner="multigrid", precision="mixed") for g in grids]
    server = pkg.pressure.Server(dgs, max_active=n)
    want = [[None] * 3 for _ in range(n)]
    for i in range(n):
        for k in range(3):
            du = torch.from_numpy(inputs[i][k]).to(dev)
            dp = torch.zeros(grids[i].count, dtype=torch.float64, device=dev)
            torch.cuda.synchronize()
            t = server.submit(i, du.data_ptr(), dp.data_ptr(), 0.1, 1e-8, 10000)
            assert drain(server, [t])[t] == 0
            want[i][k] = (du.cpu().numpy(), dp.cpu().numpy())
    server.close()

    server = pkg.pressure.Server(dgs, max_active=n)
    bufs = [[[torch.from_numpy(inputs[i][k]).pin_memory(), torch.zeros(g.count, dtype=torch.float64).pin_memory(),
              torch.empty(g.n_faces, dtype=torch.float64).pin_memory(),
              torch.empty(g.count, dtype=torch.float64).pin_memory()] for k in range(3)]
            for i, g in enumerate(grids)]

    def submit(i, k):
        return server.submit_host(i, *[b.data_ptr() for b in bufs[i][k]], 0.1, 1e-8, 10000)

    first = [[submit(i, 0), submit(i, 1)] for i in range(n)]
    for i in range(n):
        with pytest.raises(pkg.pressure.PressureError) as e:
            submit(i, 2)
        assert e.value.code == 203
    codes = drain(server, [first[i][0] for i in range(n)])
    third = [submit(i, 2) for i in range(n)]
    codes.update(drain(server, [first[i][1] for i in range(n)] + third))
    assert all(c == 0 for c in codes.values())
    server.close()
    for d in dgs:
        d.close()
    for i in range(n):
        for k in range(3):
            assert np.array_equal(bits(bufs[i][k][2].numpy()), bits(want[i][k][0])), (i, k)
            assert np.array_equal(bits(bufs[i][k][3].numpy()), bits(want[i][k][1])), (i, k)
