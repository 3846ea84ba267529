"""The reference's own unit-test identities, restated against the oracle.

pressure.rs:528-619 dense IC(0) reference; :621-676 compact == public operator
(bitwise); :678-712 projection RHS and round-off scale (bitwise); :714-743 changed
face coefficients; :745-798 fused projection == composed divergence/gradient;
tests/regressions.rs:30-56 and numerics.rs:99-171 the closed-component contract;
masked.rs:365-408 masked Galerkin; multigrid.rs:844-923 the cycle is symmetric.
"""
import math

import numpy as np
import pytest

from cases import LID_CAVITY, periodic_case, sin_field


def dense_operator(g):
    n = g.count
    a = np.zeros((n, n))
    for j in range(n):
        e = np.zeros(n)
        e[j] = 1.0
        a[:, j] = -g.divergence(g.gradient(e))
    return a


def dense_ic0(a, rhs):
    """pressure.rs:530-563: IC(0) of the shifted dense matrix, then two substitutions."""
    n = a.shape[0]
    maximum = max(1.0, max(a[i, i] for i in range(n)))
    l = np.zeros((n, n))
    for i in range(n):
        for j in range(i):
            if a[i, j] != 0.0:
                dot = sum(l[i, k] * l[j, k] for k in range(j))
                l[i, j] = (a[i, j] - dot) / l[j, j]
        sq = sum(l[i, j] * l[i, j] for j in range(i))
        l[i, i] = math.sqrt(max(a[i, i] + 1e-6 * maximum - sq, 1e-12 * maximum))
    y = np.zeros(n)
    for i in range(n):
        y[i] = (rhs[i] - sum(l[i, j] * y[j] for j in range(i))) / l[i, i]
    x = np.zeros(n)
    for i in reversed(range(n)):
        x[i] = (y[i] - sum(l[j, i] * x[j] for j in range(i + 1, n))) / l[i, i]
    return x


@pytest.mark.parametrize("n", [[2, 3, 2], [3, 3, 3], [4, 2, 3], [3, 1, 4], [1, 3, 1]])
def test_ic0_matches_dense_reference_periodic(O, n):
    g = O.Grid(periodic_case(n))
    r = sin_field(g.count, 0.7)
    expected = dense_ic0(dense_operator(g), r)
    z = g.ic0_apply(r)
    assert np.all(np.abs(z - expected) <= 1e-10 * np.maximum(np.abs(expected), 1.0))


@pytest.mark.parametrize("open_", [False, True])
def test_ic0_matches_dense_reference_masked(O, open_):
    c = periodic_case([6, 3, 2], boundary_x="open" if open_ else "wall", open_flow=open_, barrier=True)
    g = O.Grid(c)
    r = np.where(g.fluid == 1, np.array([math.cos(0.73 * i) for i in range(g.count)]), 0.0)
    expected = dense_ic0(dense_operator(g), r)
    z = g.ic0_apply(r)
    assert np.all(np.abs(z - expected) <= 1e-10 * np.maximum(np.abs(expected), 1.0))


@pytest.mark.parametrize("periodic", [False, True])
def test_compact_operator_equals_public_operator(O, periodic):
    c = periodic_case([6, 3, 2], boundary_x="periodic" if periodic else "open", open_flow=not periodic,
                      barrier=True)
    g = O.Grid(c)
    x = sin_field(g.count)
    assert np.array_equal(g.apply(x).view(np.uint64), g.operator_apply(x).view(np.uint64))


@pytest.mark.parametrize("open_", [False, True])
def test_compact_operator_bitwise_unequal_spacing(O, open_):
    c = periodic_case([18, 9, 33], boundary_x="open" if open_ else "periodic", open_flow=open_)
    c["domain"]["size_m"] = [7.15, 42.45, 38.31]
    g = O.Grid(c)
    x = sin_field(g.count)
    assert np.array_equal(g.apply(x).view(np.uint64), g.operator_apply(x).view(np.uint64))


def test_projection_rhs_and_roundoff_scale(O):
    c = periodic_case([18, 9, 33])
    c["domain"]["size_m"] = [7.15, 42.45, 38.31]
    c["geometry"] = [{"id": "barrier", "min_m": [2.0, 0.0, 0.0], "max_m": [3.0, 20.0, 15.0]}]
    g = O.Grid(c)
    u = np.array([3.0 * math.sin(0.61 * i) - 0.4 for i in range(g.n_faces)])
    dt = 0.125
    b, terms = g.projection_rhs(u, dt)
    div = g.divergence(u)
    assert np.array_equal(b, -div / dt)
    cf = g.cell_faces
    dx = [c["domain"]["size_m"][a] / c["grid"]["cells"][a] for a in range(3)]
    for i in range(g.count):
        if g.fluid[i]:
            s = -0.0
            for a in range(3):
                lo, hi = cf[i, 2 * a], cf[i, 2 * a + 1]
                s += (abs(u[lo]) + abs(u[hi])) / dx[a]
            expected = s / dt
        else:
            expected = 0.0
        assert np.float64(terms[i]).view(np.uint64) == np.float64(expected).view(np.uint64)
    assert (g.fluid == 0).any()


def test_second_solve_uses_changed_face_coefficients(O):
    c = periodic_case([5, 4, 3], boundary_x="open", open_flow=True)
    g = O.Grid(c)
    exact = sin_field(g.count)
    for changed in (False, True):
        if changed:
            area = g.face_area * (1.0 + (np.arange(g.n_faces) % 7) * 0.025)
            g.set_faces(area=area)
        b = g.apply(exact)
        code, x, info = g.solve(b, 1e-12, 2000)
        assert code == 0
        assert info["relative_residual"] <= 1.1e-11
        assert np.max(np.abs(x - exact)) < 1e-10


@pytest.mark.parametrize("boundary", ["periodic", "wall", "open"])
def test_fused_projection_matches_composed(O, boundary):
    c = periodic_case([6, 3, 2], boundary_x=boundary, open_flow=True, barrier=True)
    g = O.Grid(c)
    potential = sin_field(g.count, 0.37)
    u = g.gradient(potential)
    dt = 0.125
    b = -g.divergence(u) / dt
    _, terms = g.projection_rhs(u, dt)
    code, ref_p, ref_info = g.solve_scaled(b, terms, 1e-12, 2000)
    assert code == 0
    ref_u = u - dt * g.gradient(ref_p)
    ref_p = g.center_nullspaces(ref_p)
    code, pu, pp, info = g.project(u, np.zeros(g.count), dt, 1e-12, 2000)
    assert code == 0
    assert info["iterations"] == ref_info["iterations"]
    assert info["relative_residual"] == ref_info["relative_residual"]
    assert np.array_equal(pu, ref_u)
    assert np.array_equal(pp, ref_p)


def test_incompatible_closed_rhs_is_e031(O):
    c = periodic_case([6, 3, 2], boundary_x="wall")
    g = O.Grid(c)
    b = np.ones(g.count)
    code, _, _ = g.solve(b, 1e-10, 100)
    assert code == O.E031
    # A compatible (mean-free) closed right-hand side solves (numerics.rs:149-171).
    b = b - b.mean()
    b[0] += 1.0
    b[1] -= 1.0
    code, x, info = g.solve(b, 1e-10, 1000)
    assert code == 0 and info["iterations"] > 0


def test_iteration_limit_and_cancel_leave_state_unchanged(O):
    c = periodic_case([8, 6, 5], boundary_x="open", open_flow=True)
    g = O.Grid(c)
    rng = np.random.default_rng(5)
    u = rng.uniform(-1, 1, g.n_faces)
    u = g.enforce_velocity(u)
    p = rng.uniform(-1, 1, g.count)
    code, u2, p2, _ = g.project(u, p, 0.5, 1e-12, 1)
    assert code == O.E033
    calls = {"n": 0}

    def poll(_):
        calls["n"] += 1
        return 1 if calls["n"] >= 2 else 0

    code, u3, p3, _ = g.project(u, p, 0.5, 1e-12, 1000, poll)
    assert code == O.CANCELLED


def _dense_masked_level(O, g, level):
    d = g.mg_masked_level(level)
    n = d["diagonal"].size
    a = np.diag(d["diagonal"].copy())
    for i in range(n):
        for k in range(d["offsets"][i], d["offsets"][i + 1]):
            a[i, d["columns"][k]] += d["values"][k]
    return d, a


def test_masked_galerkin_equals_dense_product(O):
    c = periodic_case([9, 2, 7], boundary_x="wall")
    c["geometry"] = [{"id": "w", "min_m": [4.0, 0.0, 0.0], "max_m": [5.0, 2.0, 5.0]}]
    c["numerics"]["pressure_preconditioner"] = "multigrid"
    g = O.Grid(c)
    r = np.where(g.fluid == 1, sin_field(g.count), 0.0)
    g.mg_apply(r)
    cells, _ = g.mg_levels()
    assert len(cells) >= 2
    for level in range(len(cells) - 1):
        d, a = _dense_masked_level(O, g, level)
        dc, ac = _dense_masked_level(O, g, level + 1)
        P = np.zeros((a.shape[0], ac.shape[0]))
        P[np.arange(a.shape[0]), d["parent"]] = 1.0
        assert np.allclose(P.T @ a @ P, ac, atol=2e-11, rtol=0)


@pytest.mark.parametrize("masked", [False, True])
def test_multigrid_cycle_is_symmetric(O, masked):
    c = periodic_case([12, 2, 12], boundary_x="wall")
    if masked:
        c["geometry"] = [{"id": "s", "min_m": [5.0, 0.0, 5.0], "max_m": [7.0, 2.0, 7.0]}]
    c["numerics"]["pressure_preconditioner"] = "multigrid"
    g = O.Grid(c)
    rng = np.random.default_rng(3)
    f = g.fluid == 1
    r1 = g.center_nullspaces(np.where(f, rng.standard_normal(g.count), 0.0))
    r2 = g.center_nullspaces(np.where(f, rng.standard_normal(g.count), 0.0))
    z1, _ = g.mg_apply(r1)
    z2, _ = g.mg_apply(r2)
    assert abs(z1 @ r2 - r1 @ z2) <= 1e-10 * max(abs(z1 @ r2), 1.0)
    assert z1 @ r1 > 0


def test_scalar_step_matches_vectorised_restatement(pkg, O):
    """advance_scalar (solver.rs:808-855) in the oracle's sequential form against an SSPRK2
    composed from oracle/transport.py's vectorised rhs (which sums a cell's faces in
    another order, hence 1e-13 relative, not bitwise)."""
    from oracle import transport as T

    case = pkg.synth.case((14, 10, 8), 1.0, inflow=2.0, boxes=[((4.0, 3.0, 0.0), (7.0, 6.0, 4.0))])
    g = pkg.grid.Grid.build(case)
    og = O.Grid(case)
    rng = np.random.default_rng(2)
    fluid = g.fluid.astype(bool)
    u = np.where(g.face_kind != pkg.grid.WALL, rng.uniform(-2.0, 2.0, g.n_faces), 0.0)
    d = np.where(fluid, rng.uniform(0.01, 0.3, g.count), 0.0)
    source = np.where(fluid, rng.uniform(0.0, 1e-2, g.count), 0.0)
    c = np.where(fluid, rng.uniform(0.0, 1.0, g.count), 0.0)
    tr = T.Transport(g, d)
    dt = 0.01
    ref = c.copy()
    for _ in range(3):
        r1 = tr.rhs(ref, u, source)
        stage = ref + dt * r1
        ref = 0.5 * (ref + stage + dt * tr.rhs(stage, u, source))
        c = og.scalar_step(c, u, d, source, dt)
    assert np.max(np.abs(c - ref)) <= 1e-13 * np.max(np.abs(ref))


def test_muscl_rhs_hand_computed_and_vectorised(pkg, O):
    """MUSCL (transport.rs:502-526, 670-694) on a quadratic profile c = i^2 along a
    six-cell channel with unit flow: interior slopes 2i, zero slope beside the inlet and
    the outlet (no interior neighbour there), donors 0, 0, 2, 6, 12, 20, 25, so dc/dt is
    0, -2, -4, -6, -8, -5 (linear upwind gives 0, -1, -3, -5, -7, -9); the vectorised
    restatement gives these values and the oracle's sequential step agrees with an SSPRK2
    composed from it."""
    from oracle import transport as T

    case = pkg.synth.case((6, 1, 1), 1.0, boundaries=("open", "slip", "slip"), inflow=1.0)
    g = pkg.grid.Grid.build(case)
    og = O.Grid(case)
    u = np.where(np.asarray(g.face_axis) == 0, 1.0, 0.0)
    c = np.arange(6.0) ** 2
    zero = np.zeros(6)
    tr = T.Transport(g, 0.0)
    assert np.array_equal(tr.rhs(c, u, zero, muscl=True), [0.0, -2.0, -4.0, -6.0, -8.0, -5.0])
    assert np.array_equal(tr.rhs(c, u, zero), [0.0, -1.0, -3.0, -5.0, -7.0, -9.0])
    dt = 0.1
    stage = c + dt * tr.rhs(c, u, zero, muscl=True)
    want = 0.5 * (c + stage + dt * tr.rhs(stage, u, zero, muscl=True))
    got = og.scalar_step(c, u, zero, zero, dt, muscl=True)
    assert np.max(np.abs(got - want)) <= 1e-14 * np.max(np.abs(want))
    assert not np.array_equal(got, og.scalar_step(c, u, zero, zero, dt))


@pytest.mark.parametrize("boundaries", [("open", "wall", "wall"), ("open", "periodic", "slip")])
def test_muscl_step_matches_vectorised_restatement(pkg, O, boundaries):
    """The oracle's sequential MUSCL step against an SSPRK2 composed from the vectorised
    MUSCL rhs on a grid with a building, random face velocities (back-flow at the outlet
    included) and diffusivities; a periodic axis exercises the wrap neighbours."""
    from oracle import transport as T

    case = pkg.synth.case((14, 10, 8), 1.0, boundaries=boundaries, inflow=2.0,
                          boxes=[((4.0, 3.0, 0.0), (7.0, 6.0, 4.0))])
    g = pkg.grid.Grid.build(case)
    og = O.Grid(case)
    rng = np.random.default_rng(7)
    fluid = g.fluid.astype(bool)
    u = np.where(g.face_kind != pkg.grid.WALL, rng.uniform(-2.0, 2.0, g.n_faces), 0.0)
    d = np.where(fluid, rng.uniform(0.01, 0.3, g.count), 0.0)
    source = np.where(fluid, rng.uniform(0.0, 1e-2, g.count), 0.0)
    c = np.where(fluid, rng.uniform(0.0, 1.0, g.count), 0.0)
    tr = T.Transport(g, d)
    dt = 0.01
    ref = c.copy()
    for _ in range(3):
        stage = ref + dt * tr.rhs(ref, u, source, muscl=True)
        ref = 0.5 * (ref + stage + dt * tr.rhs(stage, u, source, muscl=True))
        c = og.scalar_step(c, u, d, source, dt, muscl=True)
    assert np.max(np.abs(c - ref)) <= 1e-13 * np.max(np.abs(ref))


def test_muscl_uniform_field_and_closed_box(pkg, O):
    """A uniform field has zero slopes everywhere, so its MUSCL right-hand side equals the
    linear-upwind one bit for bit; in a closed box (walls on every side) a MUSCL step moves mass between
    cells only, and the emitted-mass rate is the source sum times the cell volume."""
    case = pkg.synth.case((12, 9, 7), 1.0, boundaries=("wall", "wall", "wall"), inflow=0.0,
                          boxes=[((3.0, 2.0, 0.0), (6.0, 5.0, 3.0))])
    g = pkg.grid.Grid.build(case)
    og = O.Grid(case)
    rng = np.random.default_rng(3)
    fluid = g.fluid.astype(bool)
    u = np.where(g.face_kind == pkg.grid.INTERIOR, rng.uniform(-1.0, 1.0, g.n_faces), 0.0)
    d = np.where(fluid, rng.uniform(0.01, 0.2, g.count), 0.0)
    zero = np.zeros(g.count)
    flat = np.where(fluid, 0.25, 0.0)
    from oracle import transport as T

    tr = T.Transport(g, d)
    assert np.array_equal(tr.rhs(flat, u, zero, muscl=True), tr.rhs(flat, u, zero))
    assert np.array_equal(og.scalar_rates(flat, u, d, zero, muscl=True), og.scalar_rates(flat, u, d, zero))
    c = np.where(fluid, rng.uniform(0.0, 1.0, g.count), 0.0)
    mass0 = c.sum() * g.volume
    budget = np.zeros(3)
    for _ in range(4):
        c = og.scalar_step(c, u, d, zero, 0.02, budget, muscl=True)
    assert abs(c.sum() * g.volume - mass0) <= 1e-12 * mass0
    assert budget[1] == 0.0 and budget[2] == 0.0
    src = np.where(fluid, rng.uniform(0.0, 1e-3, g.count), 0.0)
    emitted, inflow, outflow = og.scalar_rates(c, u, d, src, muscl=True)
    assert abs(emitted - src.sum() * g.volume) <= 1e-14 * emitted and inflow == 0.0 and outflow == 0.0


def test_receptor_point_weights_match_oracle(pkg):
    """The package's receptor_weights (transport.rs:374-436) against the oracle's restatement."""
    from importlib import import_module

    from oracle import transport as T

    R = import_module(pkg.__name__ + ".receptors")
    case = pkg.synth.case((14, 10, 8), 2.0, inflow=2.0, boxes=[((8.0, 6.0, 0.0), (14.0, 12.0, 8.0))])
    g = pkg.grid.Grid.build(case)
    for p in ((1.0, 1.0, 1.0), (27.9, 19.5, 15.2), (5.3, 17.7, 3.9), (20.0, 3.0, 12.0)):
        w = R.receptor_weights(g, {"kind": "point", "point_m": list(p)})
        ref = T.point_weights(g, p)
        assert [c for c, _ in w] == [c for c, _ in ref]
        assert np.array_equal(np.array([v for _, v in w]), np.array([v for _, v in ref]))
    with pytest.raises(R.ReceptorError):
        R.receptor_weights(g, {"kind": "point", "point_m": [11.0, 9.0, 3.0]})  # a solid cell's centre
    vol = R.receptor_weights(g, {"kind": "volume_average", "min_m": [0.5, 0.5, 0.5], "max_m": [3.0, 2.0, 1.5]})
    # Overlaps 1.5 x 1.5 x 1.0 with cell (0,0,0) and 1.0 x 1.5 x 1.0 with cell (1,0,0).
    assert [c for c, _ in vol] == [0, 1]
    assert [v for _, v in vol] == [2.25 / 3.75, 1.5 / 3.75]


def test_archive_of_oracle_steps_passes_restated_checker(pkg, O, tmp_path):
    """The package's archive writer (output.rs:162-242 format) on laminar steps computed by
    the oracle: the restated checks of validation/check_fields.py pass."""
    from importlib import import_module

    from archive_check import check_archive

    A = import_module(pkg.__name__ + ".archive")
    case = pkg.synth.case((16, 12, 8), 2.0, inflow=3.0, boxes=[((10.0, 6.0, 0.0), (16.0, 14.0, 8.0))],
                          name="archive-probe")
    g = pkg.grid.Grid.build(case)
    og = O.Grid(case)
    code, u, p, info = og.project(g.initial_velocity(), np.zeros(g.count), 0.1, 1e-10, 10000)
    assert code == 0
    its = info["iterations"]
    for _ in range(3):
        code, u, p, it = og.step(u, p, 0.1, 1e-10, 10000)
        assert code == 0
        its += it
    out = tmp_path / "run"
    names = A.write_run(str(out), case, g, u, p, steps=3, time_s=0.3, pressure_iterations=its)
    assert names[-2:] == ["manifest.json", "complete.json"]
    max_div = check_archive(out, lambda c: pkg.grid.Grid.build(c).fluid.astype(bool))
    assert max_div < 1e-6
    with pytest.raises(ValueError):
        A.write_run(str(tmp_path / "bad"), dict(case, constituents=[{"id": "x"}]), g, u, p, steps=0, time_s=0.0)


@pytest.mark.parametrize("which", ["barrier", "singleton"])
def test_sealed_components_match_pivoted_dense_reference(pkg, O, which):
    """tests/urban_pressure_reference.rs:115-183: a sealed inlet-only component beside an
    anchored one, and an isolated sealed singleton, solved to 1e-13 against an independent
    pivoted dense solve (2e-10); an incompatible RHS on the singleton is E031."""
    from cases import URBAN_BARRIER, URBAN_SINGLETON, dense_reference, urban_case

    n, open_x, blocks = URBAN_BARRIER if which == "barrier" else URBAN_SINGLETON
    c = urban_case(n, open_x, blocks)
    g = pkg.grid.Grid.build(c)
    og = O.Grid(c)
    if which == "barrier":
        assert list(g.anchored) == [0, 1]
    else:
        single = (2 * g.n[1] + 1) * g.n[0] + 3
        assert np.count_nonzero(np.asarray(g.component) == g.component[single]) == 1
        assert not g.anchored[g.component[single]] and any(g.anchored)
    exact, b, ref = dense_reference(g)
    code, x, info = og.solve(b, 1e-13, 2000)
    assert code == 0 and info["relative_residual"] < 2e-12
    assert np.max(np.abs(x - ref)) < 2e-10 and np.max(np.abs(x - exact)) < 2e-10
    if which == "singleton":
        bad = np.zeros(g.count)
        bad[single] = 1e-30
        code, _, _ = og.solve(bad, 1e-13, 2000)
        assert code == O.E031


@pytest.mark.parametrize("boundary", ["wall", "periodic", "open"])
def test_manufactured_pressure_and_projection(O, boundary):
    """tests/multigrid.rs:104-129: exact = sin(0.37 i) (centred), b = -div grad exact, solved
    to 1e-12 (|x - exact| < 1e-9); projecting u = grad exact with dt = 0.125 leaves u ~ 0
    (1e-8), p = exact / dt (1e-8) and div u < 1e-7."""
    from cases import MANUFACTURED_SHAPES, lid_case

    for n in MANUFACTURED_SHAPES:
        g = O.Grid(lid_case(n, boundary))
        g.set_preconditioner("multigrid")
        exact = g.center_nullspaces(np.array([math.sin(0.37 * i) for i in range(g.count)]))
        b = -g.divergence(g.gradient(exact))
        code, x, info = g.solve(b, 1e-12, 2000)
        assert code == 0 and info["relative_residual"] <= 1.1e-11, n
        assert np.max(np.abs(x - exact)) < 1e-9, n
        dt = 0.125
        code, u, p, _ = g.project(g.gradient(exact), np.zeros(g.count), dt, 1e-12, 2000)
        assert code == 0
        assert np.max(np.abs(u)) < 1e-8 and np.max(np.abs(p - exact / dt)) < 1e-8, n
        assert np.max(np.abs(g.divergence(u))) < 1e-7, n


def test_continuum_poisson_second_order(O):
    """tests/numerics.rs:172-200: on the periodic fixture re-gridded to [n, 2, 2] cells of a
    1 m cube, the solve of b = 4 pi^2 sin(2 pi x) converges to sin(2 pi x) at second order
    (log2 of successive RMS error ratios > 1.9 for n = 8, 16, 32)."""
    import copy

    from cases import PERIODIC

    errors = []
    for n in (8, 16, 32):
        c = copy.deepcopy(PERIODIC)
        c["grid"]["cells"] = [n, 2, 2]
        c["domain"]["size_m"] = [1.0, 1.0, 1.0]
        g = O.Grid(c)
        x = (np.arange(g.count) % n + 0.5) / n
        exact = np.array([math.sin(2.0 * math.pi * v) for v in x])
        b = 4.0 * math.pi ** 2 * exact
        code, p, _ = g.solve(b, 1e-12, 1000)
        assert code == 0
        errors.append(math.sqrt(float(np.sum((p - exact) ** 2))) / math.sqrt(g.count))
    assert math.log2(errors[1] / errors[2]) > 1.9 and math.log2(errors[0] / errors[1]) > 1.9, errors


def gauged_cycle_matrix(g, comp, anchored):
    """multigrid/masked.rs:411-442: the masked V-cycle on the gauged basis (e_i - e_r0 in a
    sealed component with first cell r0, e_i in an anchored one) as a dense matrix; each
    image is finite, zero on solid cells and mean-free on sealed components."""
    regions = [np.nonzero(comp == c)[0] for c in range(len(anchored))]
    basis = []
    for region, anch in zip(regions, anchored):
        for i in region[0 if anch else 1:]:
            v = np.zeros(g.count)
            v[i] = 1.0
            if not anch:
                v[region[0]] = -1.0
            basis.append(v)
    basis = np.array(basis)
    m = np.zeros((len(basis), len(basis)))
    for j, b in enumerate(basis):
        y, _ = g.mg_apply(b)
        assert np.all(np.isfinite(y)) and np.all(y[g.fluid == 0] == 0.0)
        for region, anch in zip(regions, anchored):
            if not anch:
                assert abs(y[region].mean()) < 1e-12
        m[:, j] = basis @ y
    return m


def assert_spd(m):
    """multigrid/masked.rs:443-467: symmetric to 1e-11 of the largest entry, Cholesky
    pivots above 1e-12 of it."""
    scale = np.max(np.abs(m))
    assert np.max(np.abs(m - m.T)) < 1e-11 * scale
    assert np.all(np.linalg.eigvalsh(0.5 * (m + m.T)) > 1e-12 * scale)
    np.linalg.cholesky(m)


@pytest.mark.parametrize("which", ["periodic-wrap", "porous-periodic"])
def test_masked_cycle_spd_on_gauged_subspace(pkg, O, which):
    """multigrid/masked.rs:538-574: the masked cycle is SPD on its gauged subspace for two
    sealed periodic components joined through the wrap, and for a fixed pseudo-random
    porous mask with sealed singletons, diagonal-only contacts and one-cell passages."""
    from cases import porous_mask, topology_case

    if which == "periodic-wrap":
        c = topology_case((9, 1, 8), ("periodic", "periodic", "wall"), lambda q: q[0] in (2, 6))
    else:
        mask = porous_mask()
        c = topology_case((8, 6, 6), ("periodic", "periodic", "periodic"),
                          lambda q: mask[q[0] + 8 * (q[1] + 6 * q[2])])
    g = pkg.grid.Grid.build(c)
    comp, anchored = np.asarray(g.component), [bool(a) for a in g.anchored]
    og = O.Grid(c)
    og.set_preconditioner("multigrid")
    if which == "periodic-wrap":
        assert anchored == [False, False]
        assert any(comp[0] == comp[8] and comp[0] == k for k in range(2))
    else:
        sizes = np.bincount(comp[comp >= 0])
        assert np.any(sizes == 1) and np.any(sizes > 32) and not any(anchored)
    assert_spd(gauged_cycle_matrix(og, comp, anchored))


def test_source_fields_integrate_to_the_declared_rates(pkg):
    """cfd-craft_gb300/sources.py (transport.rs:90-178): point, line and volume sources give
    density fields whose integral is the declared rate (case.rs:684-705); a source touching
    a building is CFD-E040; a steady source in a sealed component is CFD-E043."""
    from importlib import import_module

    S = import_module(pkg.__name__ + ".sources")
    case = pkg.synth.case((20, 12, 8), 2.0, inflow=3.0, boxes=[((24.0, 8.0, 0.0), (32.0, 16.0, 10.0))])
    case["constituents"] = [{"id": "gas"}, {"id": "tracer"}]
    case["sources"] = [
        {"id": "pt", "kind": "point", "constituent": "gas", "point_m": [5.3, 7.7, 3.1], "rate_kg_s": 2e-3},
        {"id": "ln", "kind": "line", "constituent": "gas", "from_m": [2.0, 2.0, 1.0], "to_m": [20.0, 5.5, 6.2],
         "rate_kg_s_m": 1e-4},
        {"id": "vol", "kind": "volume", "constituent": "tracer", "min_m": [3.0, 18.5, 0.0],
         "max_m": [9.5, 22.0, 4.0], "rate_kg_s_m3": 5e-6},
    ]
    g = pkg.grid.Grid.build(case)
    fields = S.source_fields(case, g)
    assert len(fields) == 2
    rates = [S.rate(case["sources"][0]) + S.rate(case["sources"][1]), S.rate(case["sources"][2])]
    for f, r in zip(fields, rates):
        assert abs(f.sum() * g.volume - r) <= 1e-13 * r
        assert np.all(f[g.fluid == 0] == 0.0)
    assert abs(S.rate(case["sources"][1]) - 1e-4 * math.sqrt(18.0 ** 2 + 3.5 ** 2 + 5.2 ** 2)) < 1e-18
    # The point source sits in one cell; the line source spreads over the cells it crosses.
    assert np.count_nonzero(fields[1]) == 4 * 2 * 2
    bad = dict(case, sources=[{"id": "in-building", "kind": "point", "constituent": "gas",
                               "point_m": [27.0, 11.0, 3.0], "rate_kg_s": 1e-3}])
    with pytest.raises(S.SourceError, match="CFD-E040"):
        S.source_fields(bad, g)
    sealed = pkg.synth.case((8, 6, 4), 1.0, boundaries=("wall", "wall", "wall"), inflow=0.0)
    sealed["constituents"] = [{"id": "gas"}]
    sealed["sources"] = [{"id": "s", "kind": "point", "constituent": "gas", "point_m": [2.0, 2.0, 2.0],
                          "rate_kg_s": 1e-3}]
    sealed["run"] = dict(sealed["run"], mode="steady")
    with pytest.raises(S.SourceError, match="CFD-E043"):
        S.source_fields(sealed, pkg.grid.Grid.build(sealed))


def test_scalar_budget_closes_the_mass_balance(pkg, O):
    """advance_scalar's budget increments (solver.rs:851-853, rates of transport.rs:717-723):
    over several steps with an inflow, an outlet and a release, mass - initial - emitted -
    inflow + outflow stays at round-off (the reference checker's independent mass
    accounting, validation/check_fields.py:633-651, bounds it by 1e-9 of the scale)."""
    from importlib import import_module

    S = import_module(pkg.__name__ + ".sources")
    case = pkg.synth.case((16, 10, 6), 2.0, inflow=3.0, boxes=[((12.0, 6.0, 0.0), (18.0, 12.0, 8.0))])
    case["constituents"] = [{"id": "gas", "diffusivity_m2_s": 0.05}]
    case["sources"] = [{"id": "pt", "kind": "point", "constituent": "gas", "point_m": [5.0, 9.0, 3.0],
                        "rate_kg_s": 1e-3}]
    g = pkg.grid.Grid.build(case)
    og = O.Grid(case)
    code, u, _, _ = og.project(g.initial_velocity(), np.zeros(g.count), 0.1, 1e-10, 10000)
    assert code == 0
    src = S.source_fields(case, g)[0]
    d = S.diffusivity(case, 0, cells=g.count)
    rng = np.random.default_rng(4)
    c = np.where(g.fluid == 1, rng.uniform(0.0, 1e-4, g.count), 0.0)
    initial = c.sum() * g.volume
    budget = np.zeros(3)
    for _ in range(40):
        c = og.scalar_step(c, u, d, src, 0.05, budget)
    emitted, inflow, outflow = budget
    assert abs(emitted - 40 * 0.05 * 1e-3) < 1e-15
    assert outflow > 0.0
    mass = c.sum() * g.volume
    scale = initial + emitted + inflow + outflow
    assert abs(mass - initial - emitted - inflow + outflow) < 1e-12 * scale


@pytest.mark.parametrize("boundary", ["wall", "periodic", "open"])
def test_block_smoother_matches_independent_dense_sweeps(O, boundary):
    """multigrid/line.rs:305-349: on every level of the hierarchy, line and small-plane
    block sweeps (axes x, y, z and the x-z plane, y periodic, x periodic with a periodic x
    boundary; forward and backward) equal an independent block Gauss-Seidel with dense
    pivoted block solves to 1e-9."""
    import copy

    from cases import LID_CAVITY

    for n in ([7, 3, 5], [2, 3, 5]):
        c = copy.deepcopy(LID_CAVITY)
        c["grid"]["cells"] = n
        c["boundaries"]["x"] = boundary
        c["flow"]["initial_velocity_m_s"] = [1.0, 0.0, 0.0]
        g = O.Grid(c)
        g.set_preconditioner("multigrid")
        g.mg_apply(np.zeros(g.count))
        levels = len(g.mg_levels()[0])
        for level in range(levels):
            dims, a = g.mg_level_dense(level)
            count = a.shape[0]
            for axes in ([0], [1], [2], [0, 2]):
                periodic = [boundary == "periodic", True, False]
                rhs = np.array([math.sin(i * 0.31) for i in range(count)])
                x0 = np.array([math.cos(i * 0.19) for i in range(count)])
                for backward in (False, True):
                    got = g.block_sweep(level, axes, periodic, backward, rhs, x0)
                    # line.rs:272-303 `reference`: blocks in the order of their first cell.
                    length = int(np.prod([dims[ax] for ax in axes]))
                    groups = []
                    for i in range(count):
                        q = [i % dims[0], i // dims[0] % dims[1], i // (dims[0] * dims[1])]
                        if any(q[ax] != 0 for ax in axes):
                            continue
                        nodes = []
                        for k in range(length):
                            at, qq = k, list(q)
                            for ax in axes:
                                qq[ax] = at % dims[ax]
                                at //= dims[ax]
                            nodes.append((qq[2] * dims[1] + qq[1]) * dims[0] + qq[0])
                        groups.append(nodes)
                    if backward:
                        groups.reverse()
                    x = x0.copy()
                    for nodes in groups:
                        outside = np.setdiff1d(np.arange(count), nodes)
                        b = rhs[nodes] - a[np.ix_(nodes, outside)] @ x[outside]
                        x[nodes] = np.linalg.solve(a[np.ix_(nodes, nodes)], b)
                    assert np.all(np.abs(got - x) < 1e-9 * np.maximum(np.abs(x), 1.0)), (n, level, axes, backward)


@pytest.mark.parametrize("boundary", ["wall", "periodic", "open"])
def test_every_level_is_the_galerkin_product(O, boundary):
    """multigrid.rs:798-842: every level's matrix equals P^T A P of the level above (starting
    from the operator -div grad assembled column by column) to 2e-11, constants lie in
    its null space on closed grids and outlet anchors make the row sum positive on open
    ones; odd aggregates, unequal spacings, periodic duplicates and several levels."""
    import copy

    from cases import LID_CAVITY

    for n in ([9, 2, 7], [5, 3, 3], [2, 2, 9]):
        c = copy.deepcopy(LID_CAVITY)
        c["grid"]["cells"] = n
        c["boundaries"]["x"] = boundary
        c["flow"]["initial_velocity_m_s"] = [1.0, 0.0, 0.0]
        g = O.Grid(c)
        g.set_preconditioner("multigrid")
        g.mg_apply(np.zeros(g.count))
        a = np.zeros((g.count, g.count))
        for j in range(g.count):
            e = np.zeros(g.count)
            e[j] = 1.0
            a[:, j] = -g.divergence(g.gradient(e))
        levels = len(g.mg_levels()[0])
        for level in range(levels):
            _, m = g.mg_level_dense(level)
            assert np.all(np.abs(m - a) <= 2e-11 * np.maximum(np.maximum(np.abs(m), np.abs(a)), 1.0)), (n, level)
            y = m @ np.ones(m.shape[0])
            if boundary == "open":
                assert y.sum() > 0.0
            else:
                assert np.all(np.abs(y) <= 2e-11 * np.maximum(np.abs(y), 1.0))
            if level + 1 < levels:
                p = g.mg_transfer_dense(level)
                a = p.T @ a @ p


def test_projection_and_weighted_adjoint_identity(pkg, O):
    """tests/numerics.rs:64-98 on the periodic-tracer fixture re-gridded to 6 x 5 x 4 cells
    (12 x 6 x 6 m): the divergence and gradient are weighted adjoints
    (sum div(u) p V + sum area distance u grad(p) = 0 to 1e-11), and the projection of
    u_i = cos(0.38 i) leaves |div u| < 1e-10."""
    import copy

    from cases import PERIODIC

    c = copy.deepcopy(PERIODIC)
    c["grid"]["cells"] = [6, 5, 4]
    c["domain"]["size_m"] = [12.0, 6.0, 6.0]
    g = pkg.grid.Grid.build(c)
    og = O.Grid(c)
    p = np.array([math.sin(0.73 * i) for i in range(g.count)])
    u = np.array([math.cos(0.38 * i) for i in range(g.n_faces)])
    lhs = float(np.sum(og.divergence(u) * p * g.volume))
    rhs = float(np.sum(np.asarray(g.face_area) * np.asarray(g.face_distance) * u * og.gradient(p)))
    assert abs(lhs + rhs) < 1e-11
    code, uu, _, _ = og.project(u, np.zeros(g.count), 0.1, 1e-12, 2000)
    assert code == 0 and np.max(np.abs(og.divergence(uu))) < 1e-10


@pytest.mark.parametrize("which", ["cavity", "open-channel"])
def test_pressure_verification_fixture(pkg, O, which):
    """verification.rs:14-36 (`cfd-craft verify`): sin(2 pi x / Lx), gauge removed, its
    operator image solved to 1e-11 recovers it with an RMS error below 1e-9 (over every
    cell, so the fixture is for grids without solid cells)."""
    from cases import kernel_case

    if which == "cavity":
        c = kernel_case("cavity24", "ic0")
    else:
        c = pkg.synth.case((20, 12, 10), 2.0, inflow=4.0, preconditioner="multigrid")
    g = pkg.grid.Grid.build(c)
    og = O.Grid(c)
    lx = c["domain"]["size_m"][0]
    x = (np.arange(g.count) % g.n[0] + 0.5) * g.dx[0]
    exact = og.center_nullspaces(np.array([math.sin(2.0 * math.pi * v / lx) for v in x]))
    code, xs, info = og.solve(og.apply(exact), 1e-11, 5000)
    assert code == 0
    assert math.sqrt(float(np.sum((xs - exact) ** 2)) / g.count) < 1e-9


def test_folded_periodic_lines_keep_a_narrow_band(O):
    """multigrid/line.rs:352-365: x lines of a periodic 17 x 3 x 3 grid, folded, have a
    half-bandwidth of at most 2 on the fine level and 4 on the coarse ones."""
    import copy

    from cases import LID_CAVITY

    c = copy.deepcopy(LID_CAVITY)
    c["grid"]["cells"] = [17, 3, 3]
    c["boundaries"]["x"] = "periodic"
    g = O.Grid(c)
    g.set_preconditioner("multigrid")
    g.mg_apply(np.zeros(g.count))
    for level in range(len(g.mg_levels()[0])):
        bw = g.block_bandwidth(level, [0], [True, True, False])
        assert bw <= (2 if level == 0 else 4), (level, bw)


def test_line_source_through_cell_corners(pkg):
    """transport.rs:101-121: a line source along a cell diagonal crosses x and y faces at the
    same parameters; the duplicates merge (within 1e-14) and every cell on the diagonal
    receives an equal share of the line."""
    from importlib import import_module

    S = import_module(pkg.__name__ + ".sources")
    case = pkg.synth.case((8, 8, 4), 1.0, inflow=1.0)
    case["constituents"] = [{"id": "gas"}]
    case["sources"] = [{"id": "diag", "kind": "line", "constituent": "gas", "from_m": [0.0, 0.0, 1.5],
                        "to_m": [8.0, 8.0, 1.5], "rate_kg_s_m": 1e-3}]
    g = pkg.grid.Grid.build(case)
    f = S.source_fields(case, g)[0]
    cells = np.nonzero(f)[0]
    assert len(cells) == 8  # the eight cells (i, i, 1)
    assert all(c % 8 == (c // 8) % 8 and c // 64 == 1 for c in cells)
    assert np.allclose(f[cells], f[cells[0]], rtol=1e-14, atol=0.0)
    assert abs(f.sum() * g.volume - 1e-3 * math.sqrt(128.0)) < 1e-16
