"""Parity of the CUDA engine (through libcfdgpu.so's C ABI) with the oracle.

Bars (from the engine's specification): bitwise for the operator, the projection
right-hand side, the IC(0) substitutions and (on anchored grids) the multigrid
V-cycle; pressure, corrected face velocities and post-projection divergence within
1e-10 relative of the oracle's; PCG iteration counts within +-1.
"""
import copy
import math

import numpy as np
import pytest

from cases import (ANISOTROPIC, CANYON_93K, KERNEL_ITERATIONS, LID_CAVITY, anisotropic_case, kernel_case,
                   periodic_case, rough_rhs, sin_field)

pytestmark = pytest.mark.gpu
REL = 1e-10


def bits(a):
    return np.ascontiguousarray(a, np.float64).view(np.uint64)


def small_cases(pkg):
    out = {
        "periodic-2x3x2": periodic_case([2, 3, 2]),
        "periodic-3x1x4": periodic_case([3, 1, 4]),
        "periodic-1x3x1": periodic_case([1, 3, 1]),
        "masked-open": periodic_case([6, 3, 2], "open", True, True),
        "masked-wall": periodic_case([6, 3, 2], "wall", False, True),
        "cavity24": kernel_case("cavity24", "ic0"),
        "canyon93k": CANYON_93K,
        "pocket": pkg.synth.case((12, 12, 6), 1.0, boxes=[((3, 3, 0), (9, 4, 4)), ((3, 8, 0), (9, 9, 4)),
                                                          ((3, 3, 0), (4, 9, 4)), ((8, 3, 0), (9, 9, 4)),
                                                          ((3, 3, 3), (9, 9, 4))]),
        "buildings": pkg.synth.case((24, 20, 12), 2.0, boxes=[((10, 6, 0), (20, 14, 10)), ((30, 20, 0), (40, 34, 16))]),
    }
    c = periodic_case([18, 9, 33], "open", True)
    c["domain"]["size_m"] = [7.15, 42.45, 38.31]
    out["unequal-spacing"] = c
    # Non-periodic shapes that exercise partial wavefront tiles (8x8 pencils per tile).
    out["tiny-2x2x2"] = pkg.synth.case((2, 2, 2), 1.0)
    out["odd-3x17x9"] = pkg.synth.case((3, 17, 9), 1.0, boundaries=("wall", "wall", "wall"))
    out["odd-21x9x19"] = pkg.synth.case((21, 9, 19), 1.5, boxes=[((6, 3, 0), (12, 9, 9))])
    return out


def open_pair(pkg, O, case, pre=None):
    g = pkg.grid.Grid.build(case)
    og = O.Grid(case)
    if pre:
        og.set_preconditioner(pre)
    dg = pkg.pressure.DeviceGrid(g, preconditioner=pre)
    return g, og, dg


def test_operator_bitwise(pkg, O):
    for name, case in small_cases(pkg).items():
        g, og, dg = open_pair(pkg, O, case)
        x = sin_field(g.count)
        assert np.array_equal(bits(dg.apply(x)), bits(og.apply(x))), name
        # Changed public face coefficients (non-uniform weights path).
        area = g.face_area * (1.0 + (np.arange(g.n_faces) % 7) * 0.025)
        og.set_faces(area=area)
        dg.update_faces(area=area)
        assert np.array_equal(bits(dg.apply(x)), bits(og.apply(x))), name + " changed"
        dg.close()


def test_projection_rhs_bitwise(pkg, O):
    for name, case in small_cases(pkg).items():
        g, og, dg = open_pair(pkg, O, case)
        u = np.array([3.0 * math.sin(0.61 * i) - 0.4 for i in range(g.n_faces)])
        b, t = dg.projection_rhs(u, 0.125)
        ob, ot = og.projection_rhs(u, 0.125)
        assert np.array_equal(bits(b), bits(ob)) and np.array_equal(bits(t), bits(ot)), name
        dg.close()


def test_ic0_apply_bitwise(pkg, O):
    for name, case in small_cases(pkg).items():
        g, og, dg = open_pair(pkg, O, case, "ic0")
        r = np.where(g.fluid == 1, sin_field(g.count, 0.7), 0.0)
        assert np.array_equal(bits(dg.precondition(r)), bits(og.ic0_apply(r))), name
        dg.close()


def test_multigrid_cycle_matches(pkg, O):
    for name, case in small_cases(pkg).items():
        g, og, dg = open_pair(pkg, O, case, "multigrid")
        r = og.center_nullspaces(np.where(g.fluid == 1, sin_field(g.count, 0.7), 0.0))
        oz, _ = og.mg_apply(r)
        z = dg.precondition(r)
        if all(g.anchored):
            assert np.array_equal(bits(z), bits(oz)), name  # no gauge sums: bitwise
        else:
            assert np.max(np.abs(z - oz)) <= 1e-12 * max(1.0, np.max(np.abs(oz))), name
        assert dg.multigrid_stats()["level_cells"] == og.mg_levels()[0], name
        dg.close()


def test_published_pins_on_gpu(pkg, O):
    for name, it in KERNEL_ITERATIONS.items():
        for k, pre in enumerate(("ic0", "multigrid")):
            c = kernel_case(name, pre)
            g, og, dg = open_pair(pkg, O, c, pre)
            exact, rhs = O.manufactured_rhs(og, c)
            x, info = dg.solve_scaled(rhs, None, 1e-11, 10000)
            assert abs(info.iterations - it[k]) <= 1, (name, pre, info.iterations)
            assert info.relative_residual <= 1.01e-10
            assert math.sqrt(float(np.sum((x - exact) ** 2)) / g.count) <= 1e-8
            dg.close()
    g, og, dg = open_pair(pkg, O, CANYON_93K, "ic0")
    exact, rhs = O.manufactured_rhs(og, CANYON_93K)
    x, info = dg.solve_scaled(rhs, None, 1e-11, 10000)
    assert abs(info.iterations - 166) <= 1
    assert abs(info.relative_residual - 6.9540e-12) <= 0.05e-12
    assert abs(math.sqrt(float(np.sum((x - exact) ** 2)) / g.count) - 3.1094e-12) <= 0.05e-12


def check_projection(pkg, O, case, pre, dt=1.0, tol=1e-8, seed=0):
    g, og, dg = open_pair(pkg, O, case, pre)
    u = pkg.synth.random_velocity(g, seed)
    p = np.random.default_rng(seed + 1).uniform(-1, 1, g.count) * (g.fluid == 1)
    code, ou, op, oinfo = og.project(u, p, dt, tol, 10000)
    uu, pp = u.copy(), p.copy()
    if code != 0:
        # e.g. an inlet feeding a sealed region: the engine must refuse the same way.
        with pytest.raises(pkg.pressure.PressureError) as e:
            dg.project(uu, pp, dt, tol, 10000)
        assert e.value.code == code
        assert np.array_equal(bits(uu), bits(u)) and np.array_equal(bits(pp), bits(p))
        dg.close()
        return None
    info = dg.project(uu, pp, dt, tol, 10000)
    assert abs(info.iterations - oinfo["iterations"]) <= 1, (case["name"], pre, info.iterations, oinfo["iterations"])
    su = max(1.0, float(np.max(np.abs(ou))))
    sp = max(1.0, float(np.max(np.abs(op))))
    assert np.max(np.abs(uu - ou)) <= REL * su, case["name"]
    assert np.max(np.abs(pp - op)) <= REL * sp, case["name"]
    div, odiv = og.divergence(uu), og.divergence(ou)
    assert np.max(np.abs(div - odiv)) <= REL * max(1.0, float(np.max(np.abs(og.divergence(u))))), case["name"]
    w = info.work
    assert w["operator_applications"] == w["work_units"] + w["true_residual_checks"]
    for k in ("work_units", "operator_applications", "preconditioner_applications", "true_residual_checks"):
        assert abs(w[k] - oinfo[k]) <= 1, k
    if pre == "multigrid":
        assert w["cycles"] == w["preconditioner_applications"]
    dg.close()
    return info


@pytest.mark.parametrize("pre", ["ic0", "multigrid"])
def test_projection_parity_small(pkg, O, pre):
    for name, case in small_cases(pkg).items():
        if name in ("unequal-spacing",) and pre == "multigrid":
            continue
        check_projection(pkg, O, case, pre, dt=0.5)


@pytest.mark.parametrize("pre", ["ic0", "multigrid"])
def test_projection_parity_config1_full_size(pkg, O, pre):
    """64x64x32, open x / wall y,z, U[-1,1] faces (seed 0), tol 1e-8."""
    c = pkg.synth.config1()
    check_projection(pkg, O, c, pre, dt=1.0, tol=1e-8)


def test_projection_parity_buildings_multigrid(pkg, O):
    """A masked multigrid projection at 64x64x32 with 6 seeded buildings."""
    rng = np.random.default_rng(11)
    c = pkg.synth.case((64, 64, 32), 2.0, inflow=5.0,
                       boxes=pkg.synth.random_boxes(rng, 6, (128.0, 128.0, 64.0), dx=2.0), preconditioner="multigrid")
    check_projection(pkg, O, c, "multigrid", dt=0.1, tol=1e-8, seed=3)


def test_contract_errors_leave_state_unchanged(pkg, O):
    c = periodic_case([8, 6, 5], "open", True)
    g, og, dg = open_pair(pkg, O, c, "ic0")
    rng = np.random.default_rng(5)
    u = g.enforce_velocity(rng.uniform(-1, 1, g.n_faces))
    p = rng.uniform(-1, 1, g.count)
    u0, p0 = u.copy(), p.copy()
    with pytest.raises(pkg.pressure.PressureError) as e:
        dg.project(u, p, 0.5, 1e-12, 1)
    assert e.value.code == 33 and str(e.value).startswith("CFD-E033")
    assert np.array_equal(bits(u), bits(u0)) and np.array_equal(bits(p), bits(p0))
    calls = {"n": 0}

    def poll():
        calls["n"] += 1
        return "cancelled" if calls["n"] >= 2 else None

    with pytest.raises(pkg.pressure.PressureError) as e:
        dg.project(u, p, 0.5, 1e-12, 1000, pkg.pressure.Control(poll=poll))
    assert e.value.code == 100 and str(e.value) == "cancelled"
    assert np.array_equal(bits(u), bits(u0)) and np.array_equal(bits(p), bits(p0))
    with pytest.raises(pkg.pressure.PressureError) as e:
        dg.project(u, p, 0.5, 1e-12, 1000, pkg.pressure.Control(poll=lambda: "wall_time_limit"))
    assert e.value.code == 101
    dg.close()
    # E031: an incompatible closed right-hand side.
    c = periodic_case([6, 3, 2], "wall")
    g, og, dg = open_pair(pkg, O, c, "ic0")
    with pytest.raises(pkg.pressure.PressureError) as e:
        dg.solve_scaled(np.ones(g.count), None, 1e-10, 100)
    assert e.value.code == 31 and str(e.value).startswith("CFD-E031")
    # A zero right-hand side: 0 iterations, x = 0.
    x, info = dg.solve_scaled(np.zeros(g.count), None, 1e-10, 100)
    assert info.iterations == 0 and not x.any()
    dg.close()


def test_changed_faces_rebuild_multigrid_and_keep_ic0(pkg, O):
    c = periodic_case([5, 4, 3], "open", True)
    for pre in ("ic0", "multigrid"):
        g, og, dg = open_pair(pkg, O, c, pre)
        exact = sin_field(g.count)
        for changed in (False, True):
            if changed:
                area = g.face_area * (1.0 + (np.arange(g.n_faces) % 7) * 0.025)
                og.set_faces(area=area)
                dg.update_faces(area=area)
            b = og.apply(exact)
            x, info = dg.solve_scaled(b, None, 1e-12, 2000)
            code, ox, oinfo = og.solve(b, 1e-12, 2000)
            assert info.relative_residual <= 1.1e-11
            assert np.max(np.abs(x - exact)) < 1e-10
            assert abs(info.iterations - oinfo["iterations"]) <= 1
            if pre == "multigrid":
                assert info.work["hierarchy_builds"] == (1 if changed else 1)
        dg.close()


def test_setup_spans_only_when_built(pkg, O):
    """factor_setup_seconds / multigrid_setup_seconds (Phase::PressureFactorSetup and
    PressureMultigridSetup, pressure.rs:60-63,79-83) are positive in the call that builds
    the factor or (re)builds the hierarchy and 0 in calls that use the cached one; the
    IC(0) factor survives changed faces, the hierarchy does not."""
    c = periodic_case([5, 4, 3], "open", True)
    for pre in ("ic0", "multigrid"):
        g, og, dg = open_pair(pkg, O, c, pre)
        b = og.apply(sin_field(g.count))
        spans = []
        for step in range(3):
            if step == 2:
                area = g.face_area * (1.0 + (np.arange(g.n_faces) % 5) * 0.03)
                dg.update_faces(area=area)
            _, info = dg.solve_scaled(b, None, 1e-10, 2000)
            spans.append((info.work["factor_setup_seconds"], info.work["multigrid_setup_seconds"],
                          info.work["hierarchy_builds"]))
        dg.close()
        if pre == "ic0":
            assert spans[0][0] > 0 and spans[1][0] == 0 and spans[2][0] == 0, spans
            assert all(s[1] == 0 for s in spans), spans
        else:
            assert [s[2] for s in spans] == [1, 0, 1], spans
            assert spans[0][1] > 0 and spans[1][1] == 0 and spans[2][1] > 0, spans
            assert all(s[0] == 0 for s in spans), spans
    # The mixed form: the first projection builds the hierarchy and the FP32 state.
    cm = pkg.synth.case((32, 16, 16), 2.0, inflow=5.0, preconditioner="multigrid",
                        boxes=[((8, 0, 0), (12, 6, 8))])
    gm = pkg.grid.Grid.build(cm)
    dm = pkg.pressure.DeviceGrid(gm, preconditioner="multigrid", precision="mixed")
    u = pkg.synth.random_velocity(gm, 3)
    got = []
    for _ in range(2):
        p = np.zeros(gm.count)
        info = dm.project(u.copy(), p, 0.1, 1e-8, 1000)
        got.append((info.work["multigrid_setup_seconds"], info.work["hierarchy_builds"]))
    dm.close()
    assert got[0][0] > 0 and got[0][1] == 1 and got[1] == (0.0, 0), got


# The 18 anisotropic shapes of docs/evidence/anisotropic-pressure.md (line/plane block
# smoothing and semicoarsening, multigrid/line.rs) through the plain form's multigrid.


@pytest.mark.parametrize("name", list(ANISOTROPIC))
def test_anisotropic_pins_on_gpu(pkg, O, name):
    c = anisotropic_case(name, "multigrid")
    g, og, dg = open_pair(pkg, O, c, "multigrid")
    exact, rhs = rough_rhs(og)
    x, info = dg.solve_scaled(rhs, None, 1e-14, 1200)
    code, ox, oinfo = og.solve(rhs, 1e-14, 1200)
    dg.close()
    assert code == 0
    assert abs(info.iterations - ANISOTROPIC[name][4]) <= 1, (name, info.iterations)
    assert info.relative_residual <= 1.1e-12
    assert math.sqrt(float(np.mean((x - exact) ** 2))) <= 1e-8
    assert np.max(np.abs(x - ox)) <= REL * max(1.0, np.max(np.abs(ox)))


@pytest.mark.parametrize("name", ["outlet", "thin100", "plate64", "periodic", "stiff-two-cell", "long-domain"])
def test_block_smoothed_cycle_matches(pkg, O, name):
    """One V(1,1) cycle with line/plane block Gauss-Seidel against the oracle's: bitwise on
    an anchored grid (no gauge sums), else within 1e-12."""
    c = anisotropic_case(name, "multigrid")
    g, og, dg = open_pair(pkg, O, c, "multigrid")
    r = og.center_nullspaces(sin_field(g.count, 0.7))
    oz, _ = og.mg_apply(r)
    z = dg.precondition(r)
    assert dg.multigrid_stats()["level_cells"] == og.mg_levels()[0]
    dg.close()
    if all(g.anchored):
        assert np.array_equal(bits(z), bits(oz))
    else:
        assert np.max(np.abs(z - oz)) <= 1e-12 * max(1.0, np.max(np.abs(oz)))


BLOCK_COUNTERS = ("block_smoothing_cell_updates", "block_solves", "block_level_cell_visits", "cycles",
                  "smoothing_cell_updates", "residual_cell_updates", "coarse_solves")


@pytest.mark.parametrize("name", ["thin100", "plate64", "periodic", "stiff-two-cell", "near-isotropic"])
def test_multigrid_work_counters_and_stats_match_oracle(pkg, O, name):
    """MultigridWork's block counters (multigrid.rs:103-114) and MultigridStats'
    level_dimensions and block_smoothers (multigrid.rs:55-72) against the oracle's on the
    anisotropic campaign shapes, with the reference's own identities
    (tests/multigrid.rs:310-330): block smoothing = 2 x block level visits, block solves > 0,
    and, where every smoothed level is block-smoothed, smoothing = block smoothing."""
    c = anisotropic_case(name, "multigrid")
    g, og, dg = open_pair(pkg, O, c, "multigrid")
    exact, rhs = rough_rhs(og)
    x, info = dg.solve_scaled(rhs, None, 1e-14, 1200)
    code, ox, oinfo = og.solve(rhs, 1e-14, 1200)
    assert code == 0
    stats, ostats = dg.multigrid_stats(), og.mg_stats()
    dg.close()
    w = info.work
    for k in ("level_cells", "level_nonzeros", "level_dimensions"):
        assert stats.get(k, []) == ostats[k], (name, k)
    mine = [{k: b[k] for k in ("level", "axes", "block_unknowns", "block_count", "half_bandwidth")}
            for b in stats.get("block_smoothers", [])]
    assert mine == ostats["block_smoothers"], name
    assert all(b["allocated_bytes"] > 0 for b in stats.get("block_smoothers", []))
    assert stats["allocated_bytes"] > 0 and w["hierarchy_bytes"] == stats["allocated_bytes"]
    if info.iterations == oinfo["iterations"]:
        for k in BLOCK_COUNTERS:
            assert w[k] == oinfo[k], (name, k, w[k], oinfo[k])
    assert w["block_smoothing_cell_updates"] == 2 * w["block_level_cell_visits"]
    if ostats["block_smoothers"]:
        assert w["block_solves"] > 0
        smoothed = {b["level"] for b in ostats["block_smoothers"]}
        if smoothed == set(range(len(ostats["level_cells"]) - 1)):
            assert w["smoothing_cell_updates"] == w["block_smoothing_cell_updates"]
    else:
        assert w["block_solves"] == 0 and w["block_level_cell_visits"] == 0


def test_masked_stats_omit_dimensions(pkg, O):
    """Masked hierarchies have no level dimensions or block smoothers (masked.rs:259-262,285)."""
    c = pkg.synth.case((24, 20, 12), 2.0, boxes=[((10, 6, 0), (20, 14, 10))], preconditioner="multigrid")
    g, og, dg = open_pair(pkg, O, c, "multigrid")
    u = pkg.synth.random_velocity(g, 1)
    info = dg.project(u.copy(), np.zeros(g.count), 0.1, 1e-8, 1000)
    og.project(u, np.zeros(g.count), 0.1, 1e-8, 1000)
    stats = dg.multigrid_stats()
    dg.close()
    assert "level_dimensions" not in stats and "block_smoothers" not in stats
    assert og.mg_stats()["level_dimensions"] == [] and og.mg_stats()["block_smoothers"] == []
    assert stats["level_cells"] == og.mg_stats()["level_cells"]
    assert info.work["hierarchy_bytes"] == stats["allocated_bytes"] > 0


@pytest.mark.parametrize("which", ["barrier", "singleton"])
@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_sealed_components_against_pivoted_dense_reference(pkg, O, which, precision):
    """tests/urban_pressure_reference.rs:115-183 on the device: both forms solve the sealed
    inlet-only component and the isolated singleton within 2e-10 of an independent pivoted
    dense solve; the singleton's incompatible RHS is E031 with x untouched."""
    from cases import URBAN_BARRIER, URBAN_SINGLETON, dense_reference, urban_case

    n, open_x, blocks = URBAN_BARRIER if which == "barrier" else URBAN_SINGLETON
    c = urban_case(n, open_x, blocks)
    g = pkg.grid.Grid.build(c)
    exact, b, ref = dense_reference(g)
    dg = pkg.pressure.DeviceGrid(g, preconditioner="multigrid", precision=precision)
    try:
        x, info = dg.solve_scaled(b, None, 1e-13, 2000)
    except pkg.pressure.PressureError as e:
        assert precision == "mixed" and e.code == pkg.engine.CFDG_ERR_UNSUPPORTED
        dg.close()
        pytest.skip("the mixed form needs a hierarchy of two or more levels")
    assert info.relative_residual < 2e-12
    assert np.max(np.abs(x - ref)) < 2e-10 and np.max(np.abs(x - exact)) < 2e-10
    if which == "singleton":
        single = (2 * g.n[1] + 1) * g.n[0] + 3
        bad = np.zeros(g.count)
        bad[single] = 1e-30
        with pytest.raises(pkg.pressure.PressureError) as e:
            dg.solve_scaled(bad, None, 1e-13, 2000)
        assert e.value.code == pkg.engine.CFDG_E031
    dg.close()


@pytest.mark.parametrize("boundary", ["wall", "periodic", "open"])
def test_manufactured_pressure_and_projection_on_gpu(pkg, O, boundary):
    """tests/multigrid.rs:104-129 through the device (plain form): the manufactured solve
    and the projection of a pure gradient."""
    from cases import MANUFACTURED_SHAPES, lid_case

    for n in MANUFACTURED_SHAPES:
        c = lid_case(n, boundary)
        g, og, dg = open_pair(pkg, O, c, "multigrid")
        exact = og.center_nullspaces(np.array([math.sin(0.37 * i) for i in range(g.count)]))
        b = -og.divergence(og.gradient(exact))
        x, info = dg.solve_scaled(b, None, 1e-12, 2000)
        assert info.relative_residual <= 1.1e-11, n
        assert np.max(np.abs(x - exact)) < 1e-9, n
        dt = 0.125
        u, p = og.gradient(exact), np.zeros(g.count)
        dg.project(u, p, dt, 1e-12, 2000)
        dg.close()
        assert np.max(np.abs(u)) < 1e-8 and np.max(np.abs(p - exact / dt)) < 1e-8, n
        assert np.max(np.abs(og.divergence(u))) < 1e-7, n


def test_continuum_poisson_second_order_on_gpu(pkg):
    """tests/numerics.rs:172-200 through the device: second-order convergence of the
    periodic solve of b = 4 pi^2 sin(2 pi x) (log2 error ratios > 1.9)."""
    import copy

    from cases import PERIODIC

    errors = []
    for n in (8, 16, 32):
        c = copy.deepcopy(PERIODIC)
        c["grid"]["cells"] = [n, 2, 2]
        c["domain"]["size_m"] = [1.0, 1.0, 1.0]
        g = pkg.grid.Grid.build(c)
        dg = pkg.pressure.DeviceGrid(g, preconditioner="ic0")
        x = (np.arange(g.count) % n + 0.5) / n
        exact = np.array([math.sin(2.0 * math.pi * v) for v in x])
        p, _ = dg.solve_scaled(4.0 * math.pi ** 2 * exact, None, 1e-12, 1000)
        dg.close()
        errors.append(math.sqrt(float(np.sum((p - exact) ** 2))) / math.sqrt(g.count))
    assert math.log2(errors[1] / errors[2]) > 1.9 and math.log2(errors[0] / errors[1]) > 1.9, errors


def test_concurrent_plain_projections_equal_alone(pkg, O):
    """Plain FP64 projections of several grids from several host threads at once, each on
    its own CUDA stream (the coarse levels run as one thread-block cluster per grid, the
    fine sweeps as wavefront kernels whose blocks wait only for tiles already running),
    give the same bits as the same projections one after another."""
    import threading

    import torch

    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(8)
    cases = [pkg.synth.case((40, 32, 24), 2.0, inflow=5.0, preconditioner="multigrid",
                            boxes=pkg.synth.random_boxes(rng, 3, (80.0, 64.0, 48.0), side=(6.0, 20.0), dx=2.0)),
             pkg.synth.case((32, 32, 16), 1.0, preconditioner="multigrid"),
             pkg.synth.case((24, 20, 12), 2.0, preconditioner="ic0", boxes=[((10, 6, 0), (20, 14, 10))]),
             anisotropic_case("thin100", "multigrid")]
    grids = [pkg.grid.Grid.build(c) for c in cases]
    pres = ["multigrid", "multigrid", "ic0", "multigrid"]
    us = [pkg.synth.random_velocity(g, 60 + i) for i, g in enumerate(grids[:3])]
    exact, _ = rough_rhs(O.Grid(cases[3]))
    us.append(grids[3].gradient(exact))  # a compatible field on the closed anisotropic box
    seq = []
    for g, u, pre in zip(grids, us, pres):
        dg = pkg.pressure.DeviceGrid(g, preconditioner=pre)
        uu, pp = u.copy(), np.zeros(g.count)
        info = dg.project(uu, pp, 0.5, 1e-10, 2000)
        seq.append((uu, pp, info.iterations))
        dg.close()
    dgs, streams, d_u, d_p = [], [], [], []
    for g, u, pre in zip(grids, us, pres):
        dg = pkg.pressure.DeviceGrid(g, preconditioner=pre)
        st = torch.cuda.Stream(dev)
        dg.set_stream(st.cuda_stream)
        dgs.append(dg)
        streams.append(st)
        d_u.append(torch.from_numpy(u.copy()).to(dev))
        d_p.append(torch.zeros(g.count, dtype=torch.float64, device=dev))
    torch.cuda.synchronize()
    out = [None] * len(grids)

    def run(i):
        out[i] = dgs[i].project_device(d_u[i].data_ptr(), d_p[i].data_ptr(), 0.5, 1e-10, 2000)

    for rep in range(2):
        for i in range(len(grids)):
            d_u[i].copy_(torch.from_numpy(us[i]))
            d_p[i].zero_()
        torch.cuda.synchronize()
        ths = [threading.Thread(target=run, args=(i,)) for i in range(len(grids))]
        for th in ths:
            th.start()
        for th in ths:
            th.join()
        torch.cuda.synchronize()
        for i in range(len(grids)):
            assert out[i].iterations == seq[i][2], (i, rep)
            assert np.array_equal(bits(d_u[i].cpu().numpy()), bits(seq[i][0])), (i, rep)
            assert np.array_equal(bits(d_p[i].cpu().numpy()), bits(seq[i][1])), (i, rep)
    for dg in dgs:
        dg.close()
