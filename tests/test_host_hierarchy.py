"""The engine's host-side multigrid setup (cfd-craft_gb300/csrc/setup.cpp: aggregation,
Galerkin products, semicoarsening, block smoothers) against the oracle, on the CPU: the
setup is compiled with a small harness (tests/native/setup_harness.cpp) and every level's
matrix is compared with the oracle's, bit for bit; block smoothers with the reference's
shapes (line lengths and bandwidths of the anisotropic campaign's hierarchies)."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from cases import ANISOTROPIC, anisotropic_case, porous_mask, topology_case, urban_case, URBAN_BARRIER

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    out = str(tmp_path_factory.mktemp("harness") / "libsetup_harness.so")
    src = os.path.join(ROOT, "cfd-craft_gb300", "csrc")
    cmd = [cxx, "-O1", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-I", src, "-o", out,
           os.path.join(HERE, "native", "setup_harness.cpp"), os.path.join(src, "setup.cpp")]
    subprocess.run(cmd, check=True, capture_output=True)
    L = C.CDLL(out)
    P = C.c_void_p
    L.hh_build.argtypes = [P, P, C.c_double, P, C.c_int64, P, P, P, P, P, P, P, C.c_int32, P]
    L.hh_level_dense.restype = C.c_int64
    L.hh_level_dense.argtypes = [C.c_int32, P]
    L.hh_level_lines.argtypes = [C.c_int32, P]
    return L


def vp(a):
    return a.ctypes.data_as(C.c_void_p)


def build(L, g):
    arrs = [np.ascontiguousarray(np.array(g.n, np.int32)), np.ascontiguousarray(np.array(g.dx, np.float64)),
            np.array([1 if p else 0 for p in g.periodic], np.int32),
            np.ascontiguousarray(g.fluid, np.uint8), np.ascontiguousarray(g.face_kind, np.uint8),
            np.ascontiguousarray(g.face_lo, np.int64), np.ascontiguousarray(g.face_hi, np.int64),
            np.ascontiguousarray(g.face_area, np.float64), np.ascontiguousarray(g.face_distance, np.float64),
            np.ascontiguousarray(g.component, np.int32), np.ascontiguousarray(g.anchored, np.uint8)]
    code = L.hh_build(vp(arrs[0]), vp(arrs[1]), g.volume, vp(arrs[2]), g.n_faces, vp(arrs[3]), vp(arrs[4]),
                      vp(arrs[5]), vp(arrs[6]), vp(arrs[7]), vp(arrs[8]), vp(arrs[9]), g.n_components, vp(arrs[10]))
    assert code == 0, code
    return L.hh_levels()


def engine_level(L, level):
    n = L.hh_level_dense(level, None)
    a = np.zeros((n, n))
    L.hh_level_dense(level, vp(a))
    return a


def oracle_masked_level(og, level):
    d = og.mg_masked_level(level)
    n = d["diagonal"].size
    a = np.zeros((n, n))
    a[np.arange(n), np.arange(n)] = d["diagonal"]
    for i in range(n):
        for k in range(d["offsets"][i], d["offsets"][i + 1]):
            a[i, d["columns"][k]] += d["values"][k]
    return a


def grids(pkg):
    rng = np.random.default_rng(5)
    mask = porous_mask()
    return {
        "buildings": pkg.synth.case((24, 16, 10), 2.0, inflow=5.0, preconditioner="multigrid",
                                    boxes=pkg.synth.random_boxes(rng, 4, (48.0, 32.0, 20.0), side=(6.0, 12.0),
                                                                 height=(6.0, 16.0), dx=2.0)),
        "barrier": urban_case(*URBAN_BARRIER),
        "porous-periodic": topology_case((8, 6, 6), ("periodic", "periodic", "periodic"),
                                         lambda q: mask[q[0] + 8 * (q[1] + 6 * q[2])]),
        "unmasked-open": pkg.synth.case((18, 10, 12), 1.0, preconditioner="multigrid"),
        "anisotropic-odd": anisotropic_case("odd", "multigrid"),
        "anisotropic-periodic": anisotropic_case("periodic", "multigrid"),
        "anisotropic-plate64": anisotropic_case("plate64", "multigrid"),
    }


@pytest.mark.parametrize("name", ["buildings", "barrier", "porous-periodic", "unmasked-open", "anisotropic-odd",
                                  "anisotropic-periodic", "anisotropic-plate64"])
def test_engine_hierarchy_equals_oracle_levels(pkg, O, harness, name):
    case = grids(pkg)[name]
    g = pkg.grid.Grid.build(case)
    og = O.Grid(case)
    og.set_preconditioner("multigrid")
    og.mg_apply(np.zeros(g.count))
    cells, _ = og.mg_levels()
    levels = build(harness, g)
    assert levels == len(cells)
    masked = harness.hh_masked() == 1
    for level in range(levels):
        ea = engine_level(harness, level)
        assert ea.shape[0] == cells[level], (name, level)
        if ea.shape[0] > 3000:
            continue  # dense comparison only for the smaller levels
        oa = oracle_masked_level(og, level) if masked else og.mg_level_dense(level)[1]
        assert np.array_equal(ea, oa), (name, level, float(np.max(np.abs(ea - oa))))


@pytest.mark.parametrize("name", ["thin100", "plate64", "periodic", "stiff-two-cell"])
def test_engine_block_smoothers_have_the_reference_shapes(pkg, harness, name):
    """Every level but the last has one block smoother; lines shrink with semicoarsening,
    planes appear once the stiff axes are small (plate64), and a periodic line is folded
    to a narrow band (multigrid/line.rs:41-70, :352-365)."""
    g = pkg.grid.Grid.build(anisotropic_case(name, "multigrid"))
    levels = build(harness, g)
    out = np.zeros(4, np.int32)
    shapes = []
    for level in range(levels):
        has = harness.hh_level_lines(level, vp(out))
        assert has == (1 if level + 1 < levels else 0), (name, level)
        if has:
            shapes.append(tuple(int(v) for v in out))
    assert shapes[0][0] == max(s[0] for s in shapes)
    for length, bw, blocks, deps in shapes:
        assert length >= 2 and blocks >= 1 and deps >= 1
        assert bw <= (4 if name == "periodic" else 10)
    if name == "plate64":
        assert any(s[0] == 16 for s in shapes[1:])  # a 4 x 4 plane block on a coarse level


@pytest.mark.parametrize("name", ["buildings", "barrier", "porous-periodic", "unmasked-open"])
def test_engine_ic0_factor_equals_oracle(pkg, O, harness, name):
    """The engine's host IC(0) factor (setup.cpp build_ic0, pressure.rs:118-222) applied in
    the reference's order equals the oracle's IC(0) application bit for bit."""
    harness.hh_ic0_apply.argtypes = [C.c_void_p, C.c_void_p]
    case = grids(pkg)[name]
    g = pkg.grid.Grid.build(case)
    og = O.Grid(case)
    build(harness, g)
    r = np.where(g.fluid == 1, np.sin(0.37 * np.arange(g.count)), 0.0)
    z = np.zeros(g.count)
    assert harness.hh_ic0_apply(vp(r), vp(z)) == 0
    ref = og.ic0_apply(r)
    assert np.array_equal(z.view(np.uint64), ref.view(np.uint64)), float(np.max(np.abs(z - ref)))
