"""The mixed-precision (FP32 inner / FP64 outer) and batched forms against the FP64 oracle.

The mixed form is not the parity form: it stops on the same FP64 true residual
(|b_c - A x| / |b_c| <= tol, recomputed with the exact operator) but reaches it by a
different iteration. Bars: true relative residual <= tol; pressure and corrected
velocities within MIXED_REL of the FP64 oracle's projection solved to the same
tolerance; a case gives the same result alone and inside a batch.
"""
import numpy as np
import pytest

from cases import sin_field

pytestmark = pytest.mark.gpu
MIXED_REL = 1e-7  # relative to max|p| / max|u|, at tol 1e-8: the engine's stated bound for the mixed form


def bits(a):
    return np.ascontiguousarray(a, np.float64).view(np.uint64)


def mixed_cases(pkg):
    rng = np.random.default_rng(11)
    return {
        "c1-64x64x32": pkg.synth.case((64, 64, 32), 1.0, preconditioner="multigrid"),
        "buildings-64x64x32": pkg.synth.case((64, 64, 32), 2.0, inflow=5.0, preconditioner="multigrid",
                                             boxes=pkg.synth.random_boxes(rng, 6, (128.0, 128.0, 64.0), dx=2.0)),
        "pocket": pkg.synth.case((24, 24, 12), 1.0, preconditioner="multigrid",
                                 boxes=[((6, 6, 0), (18, 8, 8)), ((6, 16, 0), (18, 18, 8)), ((6, 6, 0), (8, 18, 8)),
                                        ((16, 6, 0), (18, 18, 8)), ((6, 6, 6), (18, 18, 8))]),
        "odd-37x29x21": pkg.synth.case((37, 29, 21), 1.5, preconditioner="multigrid",
                                       boxes=[((9, 6, 0), (21, 18, 15))]),
    }


def run_mixed(pkg, g, u, p, dt, tol):
    dg = pkg.pressure.DeviceGrid(g, preconditioner="multigrid", precision="mixed")
    uu, pp = u.copy(), p.copy()
    info = dg.project(uu, pp, dt, tol, 10000)
    dg.close()
    return uu, pp, info


@pytest.mark.parametrize("name", ["c1-64x64x32", "buildings-64x64x32", "pocket", "odd-37x29x21"])
def test_mixed_projection_against_fp64_oracle(pkg, O, name):
    case = mixed_cases(pkg)[name]
    g = pkg.grid.Grid.build(case)
    og = O.Grid(case)
    u = pkg.synth.random_velocity(g, 4)
    p = np.zeros(g.count)
    dt, tol = 0.1, 1e-8
    code, ou, op, oinfo = og.project(u, p, dt, tol, 10000)
    assert code == 0
    uu, pp, info = run_mixed(pkg, g, u, p, dt, tol)
    w = info.work
    assert info.relative_residual <= tol, info.relative_residual
    assert w["refinement_steps"] >= 1
    # Independent check of the residual with the oracle's operator.
    b, _ = og.projection_rhs(u, dt)
    bc = og.center_nullspaces(b)
    x = og.center_nullspaces(pp - p) if not all(g.anchored) else pp - p
    true_rel = np.linalg.norm(og.apply(x) - bc) / np.linalg.norm(bc)
    assert true_rel <= 1.5 * tol, true_rel
    ep = np.max(np.abs(pp - op)) / max(np.max(np.abs(op)), 1e-300)
    eu = np.max(np.abs(uu - ou)) / max(np.max(np.abs(ou)), 1e-300)
    print(f"{name}: inner iterations {info.iterations} outer {w['refinement_steps']} "
          f"(oracle {oinfo['iterations']}), rel err p {ep:.2e} u {eu:.2e}, true rel {true_rel:.2e}")
    assert ep <= MIXED_REL and eu <= MIXED_REL
    div0 = np.max(np.abs(og.divergence(u)))
    assert np.max(np.abs(og.divergence(uu))) <= 1e-6 * max(div0, 1.0)


def test_batch_equals_alone_and_is_transactional(pkg, O):
    cases = mixed_cases(pkg)
    names = ["buildings-64x64x32", "pocket", "odd-37x29x21", "c1-64x64x32"]
    grids = [pkg.grid.Grid.build(cases[n]) for n in names]
    us = [pkg.synth.random_velocity(g, 20 + i) for i, g in enumerate(grids)]
    ps = [sin_field(g.count, 0.1 * (i + 1)) * (g.fluid == 1) for i, g in enumerate(grids)]
    dts = [0.1, 0.2, 0.05, 0.1]
    alone = [run_mixed(pkg, g, u, p, dt, 1e-8) for g, u, p, dt in zip(grids, us, ps, dts)]
    dgs = [pkg.pressure.DeviceGrid(g, preconditioner="multigrid", precision="mixed") for g in grids]
    batch = pkg.pressure.Batch(dgs)
    bu = [u.copy() for u in us]
    bp = [p.copy() for p in ps]
    res = batch.project(bu, bp, dts, 1e-8, 10000)
    for i, (code, info) in enumerate(res):
        assert code == 0
        assert info.iterations == alone[i][2].iterations
        assert np.array_equal(bits(bu[i]), bits(alone[i][0])), names[i]
        assert np.array_equal(bits(bp[i]), bits(alone[i][1])), names[i]
    # An incompatible case (an inlet feeding a sealed region) fails alone; the others solve.
    bad = pkg.synth.case((24, 12, 8), 1.0, preconditioner="multigrid", boxes=[((8, 0, 0), (9, 12, 8))])
    gb = pkg.grid.Grid.build(bad)
    assert not all(gb.anchored)
    ub = pkg.synth.random_velocity(gb, 1)
    pb = np.zeros(gb.count)
    dgb = pkg.pressure.DeviceGrid(gb, preconditioner="multigrid", precision="mixed")
    batch2 = pkg.pressure.Batch([dgb, dgs[0]])
    u0, p0 = ub.copy(), pb.copy()
    u1, p1 = us[0].copy(), ps[0].copy()
    res = batch2.project([u0, u1], [p0, p1], [0.1, 0.1], 1e-8, 10000)
    assert res[0][0] == 31 and res[1][0] == 0
    assert np.array_equal(bits(u0), bits(ub)) and np.array_equal(bits(p0), bits(pb))
    assert np.array_equal(bits(u1), bits(alone[0][0]))
    batch.close()
    batch2.close()
    for d in dgs + [dgb]:
        d.close()


def test_batch_follows_changed_face_coefficients(pkg):
    """After cfdg_grid_update_faces the batch rebuilds that grid's hierarchy and FP32 state."""
    cases = mixed_cases(pkg)
    g1 = pkg.grid.Grid.build(cases["odd-37x29x21"])
    g2 = pkg.grid.Grid.build(cases["pocket"])
    d1 = pkg.pressure.DeviceGrid(g1, preconditioner="multigrid", precision="mixed")
    d2 = pkg.pressure.DeviceGrid(g2, preconditioner="multigrid", precision="mixed")
    batch = pkg.pressure.Batch([d1, d2])
    u1, u2 = pkg.synth.random_velocity(g1, 5), pkg.synth.random_velocity(g2, 6)
    p1, p2 = np.zeros(g1.count), np.zeros(g2.count)
    area = g1.face_area * (1.0 + (np.arange(g1.n_faces) % 5) * 0.01)
    d1.update_faces(area=area)
    bu = [u1.copy(), u2.copy()]
    bp = [p1.copy(), p2.copy()]
    res = batch.project(bu, bp, [0.1, 0.1], 1e-8, 10000)
    assert [c for c, _ in res] == [0, 0]
    # Alone, on a grid built with the same changed coefficients.
    g1b = pkg.grid.Grid.build(cases["odd-37x29x21"])
    g1b.face_area = area
    au, ap_, _ = run_mixed(pkg, g1b, u1, p1, 0.1, 1e-8)
    assert np.array_equal(bits(bu[0]), bits(au)) and np.array_equal(bits(bp[0]), bits(ap_))
    batch.close()
    d1.close()
    d2.close()


def test_batch_with_several_tiles_per_block(pkg, O):
    """Uneven cases whose row tiles outnumber the persistent grid (1216 blocks), so each block
    walks tiles of several cases, some of them already converged; results equal alone."""
    rng = np.random.default_rng(23)
    shapes = [(128, 128, 64), (96, 96, 48), (128, 128, 64), (24, 24, 12)]
    cases = [pkg.synth.case(sh, 2.0, inflow=5.0, preconditioner="multigrid",
                            boxes=pkg.synth.random_boxes(rng, 4, [v * 2.0 for v in sh], side=(6.0, 20.0),
                                                         height=(6.0, 40.0), dx=2.0)) for sh in shapes]
    grids = [pkg.grid.Grid.build(c) for c in cases]
    assert sum((g.n[1] * g.n[2] + 7) // 8 for g in grids) > 2 * 1216
    us = [pkg.synth.random_velocity(g, 40 + i) for i, g in enumerate(grids)]
    ps = [np.zeros(g.count) for g in grids]
    dts = [0.1, 0.1, 0.05, 0.1]
    alone = [run_mixed(pkg, g, u, p, dt, 1e-8) for g, u, p, dt in zip(grids, us, ps, dts)]
    dgs = [pkg.pressure.DeviceGrid(g, preconditioner="multigrid", precision="mixed") for g in grids]
    batch = pkg.pressure.Batch(dgs)
    for rep in range(2):
        bu = [u.copy() for u in us]
        bp = [p.copy() for p in ps]
        res = batch.project(bu, bp, dts, 1e-8, 10000)
        for i, (code, info) in enumerate(res):
            assert code == 0
            assert info.iterations == alone[i][2].iterations
            assert np.array_equal(bits(bu[i]), bits(alone[i][0])), (rep, i)
            assert np.array_equal(bits(bp[i]), bits(alone[i][1])), (rep, i)
    # The 96x96x48 case against the FP64 oracle.
    og = O.Grid(cases[1])
    code, ou, op, _ = og.project(us[1], ps[1], dts[1], 1e-8, 10000)
    assert code == 0
    ep = np.max(np.abs(alone[1][1] - op)) / np.max(np.abs(op))
    eu = np.max(np.abs(alone[1][0] - ou)) / np.max(np.abs(ou))
    assert ep <= MIXED_REL and eu <= MIXED_REL, (ep, eu)
    batch.close()
    for d in dgs:
        d.close()


def test_coarse_scale_keeps_accuracy_and_cuts_iterations(pkg, O):
    """cfdg_grid_set_coarse_scale: 1.0 is the reference's cycle; the default over-correction
    (1.8) on an aggregation hierarchy reaches the same FP64 tolerance and the same accuracy
    against the FP64 oracle in fewer iterations; scales outside (0, 2) are refused."""
    case = mixed_cases(pkg)["buildings-64x64x32"]
    g = pkg.grid.Grid.build(case)
    og = O.Grid(case)
    u = pkg.synth.random_velocity(g, 8)
    p = np.zeros(g.count)
    dt, tol = 0.1, 1e-8
    code, ou, op, _ = og.project(u, p, dt, tol, 10000)
    assert code == 0
    its = {}
    for alpha in (1.0, 1.8):
        dg = pkg.pressure.DeviceGrid(g, preconditioner="multigrid", precision="mixed")
        dg.set_coarse_scale(alpha)
        uu, pp = u.copy(), p.copy()
        info = dg.project(uu, pp, dt, tol, 10000)
        dg.close()
        assert info.relative_residual <= tol
        assert np.max(np.abs(pp - op)) / np.max(np.abs(op)) <= MIXED_REL
        assert np.max(np.abs(uu - ou)) / np.max(np.abs(ou)) <= MIXED_REL
        its[alpha] = info.iterations
    print("iterations by coarse scale", its)
    assert its[1.8] < its[1.0]
    dg = pkg.pressure.DeviceGrid(g, preconditioner="multigrid", precision="mixed")
    for bad in (0.0, 2.0, -1.0):
        with pytest.raises(pkg.pressure.PressureError):
            dg.set_coarse_scale(bad)
    dg.close()


def test_staged_half_sweeps_equal_register_sweeps(pkg):
    """The level-0 half sweeps staged through the tensor memory accelerator (k_rb_tma) give
    the same bits as the register kernel (k_rb): cases whose weights are uniform and whose
    ceil(nx/2) is a multiple of 8 run staged in a batch of their own, and the register
    kernel in a batch with a case that is not (37 x 29 x 21)."""
    rng = np.random.default_rng(5)
    # Row counts that leave partial stages (185 and 123 rows) and shapes one or a few rows high.
    specs = [((64, 64, 32), 6), ((48, 48, 48), 4), ((16, 10, 8), 1), ((96, 96, 48), 9), ((32, 5, 37), 1),
             ((16, 41, 3), 1)]
    cases = [pkg.synth.case(n, 2.0, inflow=5.0, preconditioner="multigrid",
                            boxes=pkg.synth.random_boxes(rng, nb, [2.0 * v for v in n], side=(6.0, 20.0), dx=2.0))
             for n, nb in specs]
    odd = mixed_cases(pkg)["odd-37x29x21"]
    grids = [pkg.grid.Grid.build(c) for c in cases + [odd]]
    us = [pkg.synth.random_velocity(g, 40 + i) for i, g in enumerate(grids)]
    ps = [np.zeros(g.count) for g in grids]
    results = {}
    ns = len(specs)
    for name, idx in (("staged", list(range(ns))), ("register", list(range(ns + 1)))):
        dgs = [pkg.pressure.DeviceGrid(grids[i], preconditioner="multigrid", precision="mixed") for i in idx]
        batch = pkg.pressure.Batch(dgs)
        assert batch.stats()["staged_sweeps"] is (name == "staged")
        bu = [us[i].copy() for i in idx]
        bp = [ps[i].copy() for i in idx]
        res = batch.project(bu, bp, [0.1] * len(idx), 1e-8, 10000)
        assert all(code == 0 for code, _ in res)
        if name == "staged":
            ms_staged, b1 = batch.time_kernel(0, 5)
            ms_reg, b2 = batch.time_kernel(4, 5)
            assert b1 == b2 > 0 and ms_staged > 0 and ms_reg > 0
            print(f"half sweep over {sum(g.count for g in grids[:ns])} cells: staged {ms_staged:.4f} ms, "
                  f"register {ms_reg:.4f} ms")
        results[name] = (bu, bp, [info.iterations for _, info in res])
        batch.close()
        for d in dgs:
            d.close()
    for k in range(ns):
        assert results["staged"][2][k] == results["register"][2][k]
        assert np.array_equal(bits(results["staged"][0][k]), bits(results["register"][0][k])), k
        assert np.array_equal(bits(results["staged"][1][k]), bits(results["register"][1][k])), k


@pytest.mark.parametrize("y", [0.1, 0.05, 0.3, 1.0 / 3.0, 0.7, 0.037, 1.0 - 2.0 ** -53, 1.0 + 2.0 ** -52,
                               2.0 - 2.0 ** -51, 0.25, 2.0 ** -60, 2.0 ** 60, 12345.678, 9.87e-15])
def test_division_from_reciprocal_is_correctly_rounded(pkg, y):
    """The mixed right-hand side divides by dt through a reciprocal and one correction step
    (Markstein's); every quotient equals CUDA's correctly rounded division, bit for bit, on
    random numerators and on numerators whose quotients lie next to a double or next to a
    midpoint between two doubles."""
    import ctypes as C

    L = pkg.engine.load()
    for mode in range(3):
        bad = C.c_uint64()
        assert L.cfdg_debug_div_check(y, 1234 + mode, 1 << 22, mode, C.byref(bad)) == 0, pkg.engine.last_error()
        assert bad.value == 0, (y, mode, bad.value)


def test_mixed_rhs_bitwise_against_oracle(pkg, O):
    """b = -div(u)/dt of the mixed form (power-of-two face spacings as exponent shifts, the
    division by dt from its reciprocal) equals the oracle's projection right-hand side bit
    for bit; the round-off terms too where the grid has closed components (the mixed form
    forms them only there)."""
    cases = mixed_cases(pkg)
    names = ["buildings-64x64x32", "pocket", "odd-37x29x21"]
    grids = [pkg.grid.Grid.build(cases[n]) for n in names]
    ogs = [O.Grid(cases[n]) for n in names]
    dgs = [pkg.pressure.DeviceGrid(g, preconditioner="multigrid", precision="mixed") for g in grids]
    batch = pkg.pressure.Batch(dgs)
    for dts in ([0.1, 0.037, 0.25], [1.0 / 3.0, 0.1, 0.7]):
        us = [pkg.synth.random_velocity(g, 70 + i) for i, g in enumerate(grids)]
        res = batch.project([u.copy() for u in us], [np.zeros(g.count) for g in grids], dts, 1e-8, 10000)
        for i, g in enumerate(grids):
            b, terms = batch.debug_rhs(i, g.count)
            ob, oterms = ogs[i].projection_rhs(us[i], dts[i])
            assert np.array_equal(bits(b), bits(ob)), (names[i], dts[i])
            if not all(g.anchored):
                assert np.array_equal(bits(terms), bits(oterms)), (names[i], dts[i])
            else:
                assert not np.any(terms)
        assert res[1][0] in (0, 31)  # the pocket may be incompatible for a random field
    batch.close()
    for d in dgs:
        d.close()


def test_bin_grid_first_coarse_level_gives_the_same_bits(pkg):
    """The first coarse level laid out as the 2x2x2 bin grid (restriction children and
    prolongation parents from bin positions, sweeps and residual through computed
    bin-stencil columns) against the aggregates' colour order with index lists: the same
    projected bits and iterations, alone and in a batch. The grid without buildings runs
    on the mixed form's aggregation hierarchy and takes the bin grid too; a grid with a
    sealed pocket (closed groups on level 0) keeps the index lists."""
    rng = np.random.default_rng(23)
    cases = [pkg.synth.case((64, 64, 32), 2.0, inflow=5.0, preconditioner="multigrid",
                            boxes=pkg.synth.random_boxes(rng, 8, (128.0, 128.0, 64.0), dx=2.0)),
             pkg.synth.case((48, 40, 24), 2.0, inflow=5.0, preconditioner="multigrid",
                            boxes=pkg.synth.random_boxes(rng, 5, (96.0, 80.0, 48.0), dx=2.0)),
             pkg.synth.case((32, 32, 16), 2.0, inflow=5.0, preconditioner="multigrid")]
    grids = [pkg.grid.Grid.build(c) for c in cases]
    us = [pkg.synth.random_velocity(g, 40 + i) for i, g in enumerate(grids)]
    out = {}
    for bins in (False, True):
        dgs = [pkg.pressure.DeviceGrid(g, preconditioner="multigrid", precision="mixed") for g in grids]
        for d in dgs:
            d.set_coarse_layout(bins)
        alone = []
        for d, g, u in zip(dgs, grids, us):
            uu, pp = u.copy(), np.zeros(g.count)
            info = d.project(uu, pp, 0.1, 1e-8, 10000)
            alone.append((uu, pp, info.iterations))
        batch = pkg.pressure.Batch(dgs)
        laid = [c["level1_bins"] for c in batch.stats()["cases"]]
        assert [c["level1_stencil"] for c in batch.stats()["cases"]] == laid
        # deeper levels take bin stencils too where their bins hold one aggregate each
        deep = [sum(lv["bin_stencil"] for lv in c["levels"]) for c in batch.stats()["cases"]]
        assert all(d >= (1 if b else 0) for d, b in zip(deep, laid)), deep
        bu, bp = [u.copy() for u in us], [np.zeros(g.count) for g in grids]
        res = batch.project(bu, bp, [0.1] * len(grids), 1e-8, 10000)
        assert all(code == 0 for code, _ in res)
        batch.close()
        for d in dgs:
            d.close()
        out[bins] = (alone, bu, bp, laid)
    assert out[False][3] == [False, False, False]
    assert out[True][3] == [True, True, True]
    gp = pkg.grid.Grid.build(mixed_cases(pkg)["pocket"])
    dp = pkg.pressure.DeviceGrid(gp, preconditioner="multigrid", precision="mixed")
    bp_ = pkg.pressure.Batch([dp])
    assert [c["level1_bins"] for c in bp_.stats()["cases"]] == [False]
    bp_.close()
    dp.close()
    for i in range(len(grids)):
        a0, a1 = out[False][0][i], out[True][0][i]
        assert a0[2] == a1[2], i
        assert np.array_equal(bits(a0[0]), bits(a1[0])) and np.array_equal(bits(a0[1]), bits(a1[1])), i
        assert np.array_equal(bits(out[False][1][i]), bits(out[True][1][i])), i
        assert np.array_equal(bits(out[False][2][i]), bits(out[True][2][i])), i
