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
