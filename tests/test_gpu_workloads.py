"""The measured workloads against the FP64 oracle, at their full sizes.

Each benchmark configuration is checked on the inputs the benchmark runs:

* the serving mix (36 wind directions over a 128x128x64 grid with 30 buildings, open
  x/y, ground_open_top z, plus 16 cases at 96x96x48) served through cfdg_server in the
  mixed form with the cycle the benchmark's autotuner picks on it, V(2,2) with the coarse
  corrections scaled by 1.85, for two consecutive time steps of the u* sequence, and
  every candidate cycle of the autotuner on one wind direction;
* the 128x128x64 grid with 12 buildings in the plain FP64 form (multigrid), full size;
* the 256x256x128 grid with 40 buildings (8.4 M cells) in the mixed form;
* three cases of the uneven batch (160x160x80, 96x96x48, 48x48x48) in one batched call.

Bars: plain form, pressure and corrected face velocities within 1e-10 relative (to
max|.|) of the oracle's projection, post-projection divergence within 1e-10 of the
oracle's (relative to the input's), PCG iterations within +-1 and the work counters of
the profile equal; mixed form, pressure and face velocities within 1e-7 relative of the
oracle's FP64 projection at the same tolerance (1e-8), the FP64 true residual at most
the tolerance, and the post-projection divergence within 1e-7 of the oracle's
(relative to the input's divergence).
"""
import concurrent.futures as cf

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
PLAIN_REL = 1e-10
MIXED_REL = 1e-7
DT, TOL, MAX_IT = 0.1, 1e-8, 10000
# Wind directions 0, 90 and 200 degrees of the serving mix, and two of its 96x96x48 cases.
SERVED = (0, 9, 20, 36, 44)


def oracle_projections(O, jobs):
    """FP64 oracle projections of (case, u, p) jobs, one host thread each (the oracle's
    ctypes calls release the interpreter lock)."""

    def one(job):
        case, u, p = job
        code, ou, op, info = O.Grid(case).project(u, p, DT, TOL, MAX_IT)
        assert code == 0, (case["name"], code)
        return ou, op, info

    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        return list(ex.map(one, jobs))


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(float(np.max(np.abs(b))), 1e-300))


def check_mixed(O, case, g, u, p, uu, pp, ou, op, info, label):
    og = O.Grid(case)
    ep, eu = rel(pp, op), rel(uu, ou)
    div_in = max(float(np.max(np.abs(og.divergence(u)))), 1.0)
    ediv = float(np.max(np.abs(og.divergence(uu) - og.divergence(ou)))) / div_in
    print(f"{label}: iterations {info.iterations} (refinement {info.work['refinement_steps']}), "
          f"rel err p {ep:.2e} u {eu:.2e} div {ediv:.2e}, residual {info.relative_residual:.2e}")
    assert info.relative_residual <= TOL, (label, info.relative_residual)
    assert ep <= MIXED_REL and eu <= MIXED_REL, (label, ep, eu)
    assert ediv <= MIXED_REL, (label, ediv)
    return ep, eu


def serve(pkg, server, torch, dev, inputs):
    """Submits one request per (grid index, u, p) through the server and runs it to the end;
    returns the projected (u, p) per request, in order."""
    d_u = [torch.from_numpy(u.copy()).to(dev) for _, u, _ in inputs]
    d_p = [torch.from_numpy(p.copy()).to(dev) for _, _, p in inputs]
    torch.cuda.synchronize()
    tickets = [server.submit(i, d_u[k].data_ptr(), d_p[k].data_ptr(), DT, TOL, MAX_IT)
               for k, (i, _, _) in enumerate(inputs)]
    done = {}
    for _ in range(1_000_000):
        server.progress()
        for k, t in enumerate(tickets):
            if k not in done and (r := server.result(t)) is not None:
                done[k] = r
        if len(done) == len(tickets):
            break
    assert len(done) == len(tickets)
    out = []
    for k in range(len(tickets)):
        code, info = done[k]
        assert code == 0, (k, code)
        out.append((d_u[k].cpu().numpy(), d_p[k].cpu().numpy(), info))
    return out


def test_serving_mix_served_against_oracle(pkg, O):
    """Five cases of the serving mix through cfdg_server at the autotuned cycle, two steps."""
    import torch

    dev = torch.device("cuda", 0)
    mix = pkg.synth.config5()
    cases = [mix[i] for i in SERVED]
    grids = [pkg.grid.Grid.build(c) for c in cases]
    dgs = [pkg.pressure.DeviceGrid(g, preconditioner="multigrid", precision="mixed") for g in grids]
    for d in dgs:
        d.set_cycle(2, 2)
        d.set_coarse_scale(1.85)
    server = pkg.pressure.Server(dgs, max_active=len(dgs))
    # Step 1: the benchmark's first inputs (U[-1,1] faces, seeds 5000 + case index), p = 0.
    inputs = [(k, pkg.synth.random_velocity(g, seed=5000 + SERVED[k]), np.zeros(g.count))
              for k, g in enumerate(grids)]
    worst = 0.0
    for step in range(2):
        res = serve(pkg, server, torch, dev, inputs)
        ref = oracle_projections(O, [(cases[k], u, p) for k, u, p in inputs])
        nxt = []
        for k, ((uu, pp, info), (ou, op, _)) in enumerate(zip(res, ref)):
            _, u, p = inputs[k]
            ep, eu = check_mixed(O, cases[k], grids[k], u, p, uu, pp, ou, op, info,
                                 f"step {step} {cases[k]['name']}")
            worst = max(worst, ep, eu)
            # u*_{s+1} = project(u*_s) + 0.05 U[-1,1] on the free faces.
            g = grids[k]
            free = (g.face_kind == pkg.grid.INTERIOR) | (g.face_kind == pkg.grid.OUTLET)
            noise = np.random.default_rng(7000 + 10 * step + k).uniform(-0.05, 0.05, g.n_faces) * free
            nxt.append((k, uu + noise, pp))
        inputs = nxt
    print(f"serving mix: worst relative error against the FP64 oracle {worst:.2e}")
    server.close()
    for d in dgs:
        d.close()


@pytest.mark.parametrize("cand", [(1, 2, 1.85), (2, 1, 1.85), (2, 2, 1.7), (2, 2, 1.85), (2, 3, 1.85), (3, 2, 1.85),
                                  (2, 2, 1.0)])
def test_autotuner_candidates_against_oracle(pkg, O, cand, _dir200_reference):
    """Every cycle the benchmark's autotuner may pick (and the reference's own scale 1.0) on
    the 200-degree wind direction of the serving mix."""
    case, g, u, ou, op = _dir200_reference
    assert tuple(cand[:2]) + (cand[2],) in set(pkg.pressure.CYCLE_CANDIDATES) | {(2, 2, 1.0)}
    dg = pkg.pressure.DeviceGrid(g, preconditioner="multigrid", precision="mixed")
    dg.set_cycle(cand[0], cand[1])
    dg.set_coarse_scale(cand[2])
    uu, pp = u.copy(), np.zeros(g.count)
    info = dg.project(uu, pp, DT, TOL, MAX_IT)
    dg.close()
    check_mixed(O, case, g, u, np.zeros(g.count), uu, pp, ou, op, info, f"{case['name']} V{cand[:2]} a={cand[2]}")


@pytest.fixture(scope="module")
def _dir200_reference(pkg, O):
    case = pkg.synth.config5()[20]
    g = pkg.grid.Grid.build(case)
    u = pkg.synth.random_velocity(g, seed=5020)
    (ou, op, _), = oracle_projections(O, [(case, u, np.zeros(g.count))])
    return case, g, u, ou, op


COUNTERS = ("work_units", "operator_applications", "preconditioner_applications", "true_residual_checks",
            "hierarchy_levels", "hierarchy_cells", "hierarchy_nonzeros", "cycles", "smoothing_cell_updates",
            "residual_cell_updates", "restriction_cell_updates", "prolongation_cell_updates", "coarse_solves")


def test_plain_multigrid_projection_128x128x64_full_size(pkg, O):
    """The 128x128x64 grid with 12 buildings (seed 1), plain FP64 masked multigrid PCG."""
    case = pkg.synth.config2(seed=1)
    g = pkg.grid.Grid.build(case)
    u = pkg.synth.random_velocity(g, seed=3)
    p = np.random.default_rng(4).uniform(-1, 1, g.count) * (g.fluid == 1)
    (ou, op, oinfo), = oracle_projections(O, [(case, u, p)])
    dg = pkg.pressure.DeviceGrid(g, preconditioner="multigrid")
    uu, pp = u.copy(), p.copy()
    info = dg.project(uu, pp, DT, TOL, MAX_IT)
    dg.close()
    og = O.Grid(case)
    su = max(1.0, float(np.max(np.abs(ou))))
    sp = max(1.0, float(np.max(np.abs(op))))
    print(f"plain 128x128x64: iterations {info.iterations} (oracle {oinfo['iterations']}), "
          f"rel err p {np.max(np.abs(pp - op)) / sp:.2e} u {np.max(np.abs(uu - ou)) / su:.2e}")
    assert abs(info.iterations - oinfo["iterations"]) <= 1
    assert np.max(np.abs(uu - ou)) <= PLAIN_REL * su
    assert np.max(np.abs(pp - op)) <= PLAIN_REL * sp
    div_in = max(1.0, float(np.max(np.abs(og.divergence(u)))))
    assert np.max(np.abs(og.divergence(uu) - og.divergence(ou))) <= PLAIN_REL * div_in
    w = info.work
    if info.iterations == oinfo["iterations"]:
        for k in COUNTERS:
            assert w[k] == oinfo[k], (k, w[k], oinfo[k])
    else:
        for k in ("hierarchy_levels", "hierarchy_cells", "hierarchy_nonzeros"):
            assert w[k] == oinfo[k], k


def test_mixed_projection_256x256x128(pkg, O):
    """The 8.4 M-cell grid with 40 buildings (seed 2), U[-1,1] faces (seed 3), mixed form."""
    case = pkg.synth.config3()
    g = pkg.grid.Grid.build(case)
    u = pkg.synth.random_velocity(g, seed=3)
    p = np.zeros(g.count)
    (ou, op, oinfo), = oracle_projections(O, [(case, u, p)])
    dg = pkg.pressure.DeviceGrid(g, preconditioner="multigrid", precision="mixed")
    uu, pp = u.copy(), p.copy()
    info = dg.project(uu, pp, DT, TOL, MAX_IT)
    dg.close()
    check_mixed(O, case, g, u, p, uu, pp, ou, op, info, f"{case['name']} (oracle {oinfo['iterations']} iterations)")


def test_uneven_batch_cases_against_oracle(pkg, O):
    """Three shapes of the 64-case uneven batch (cases 22, 2 and 7: 160x160x80 with 17
    buildings, 96x96x48 with 3, 48x48x48 with 13), projected in one batched call."""
    allc = pkg.synth.config4()
    cases = [allc[i] for i in (22, 2, 7)]
    assert [c["grid"]["cells"] for c in cases] == [[160, 160, 80], [96, 96, 48], [48, 48, 48]]
    grids = [pkg.grid.Grid.build(c) for c in cases]
    us = [pkg.synth.random_velocity(g, seed=300 + k) for k, g in enumerate(grids)]
    ps = [np.zeros(g.count) for g in grids]
    ref = oracle_projections(O, list(zip(cases, us, ps)))
    dgs = [pkg.pressure.DeviceGrid(g, preconditioner="multigrid", precision="mixed") for g in grids]
    batch = pkg.pressure.Batch(dgs)
    bu = [u.copy() for u in us]
    bp = [p.copy() for p in ps]
    res = batch.project(bu, bp, [DT] * 3, TOL, MAX_IT)
    for k, (code, info) in enumerate(res):
        assert code == 0
        ou, op, _ = ref[k]
        check_mixed(O, cases[k], grids[k], us[k], ps[k], bu[k], bp[k], ou, op, info, cases[k]["name"])
    batch.close()
    for d in dgs:
        d.close()
