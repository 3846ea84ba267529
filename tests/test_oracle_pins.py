"""The oracle against the reference's published known answers (parity pins).

docs/evidence/native-cpu-performance.md:210-212 -- the 93k canyon manufactured solve:
166 PCG iterations, recomputed relative residual 6.9540e-12, RMS error 3.1094e-12.
docs/evidence/pressure-multigrid.md:32-38 -- manufactured cavity/cube kernels at
tol 1e-11: IC(0) 53/102/193/61/113 and multigrid 6/6/6/7/7 iterations.
The RHS is performance_probe.rs:83-95 (sin(2 pi x/Lx) + 0.3 cos(4 pi z/Lz)).
"""
import math

import numpy as np
import pytest

from cases import CANYON_93K, KERNEL_ITERATIONS, kernel_case


def test_canyon_93k_ic0_pin(O):
    g = O.Grid(CANYON_93K)
    assert (g.count, g.n_faces, g.n_components) == (93312, 286200, 1)
    exact, rhs = O.manufactured_rhs(g, CANYON_93K)
    code, x, info = g.solve(rhs, 1e-11, 10000)
    assert code == 0
    assert info["iterations"] == 166
    assert f"{info['relative_residual']:.4e}" == "6.9540e-12"
    rms = math.sqrt(float(np.sum((x - exact) ** 2)) / g.count)
    assert f"{rms:.4e}" == "3.1094e-12"


@pytest.mark.parametrize("name", list(KERNEL_ITERATIONS))
@pytest.mark.parametrize("pre", ["ic0", "multigrid"])
def test_kernel_iteration_pins(O, name, pre):
    c = kernel_case(name, pre)
    g = O.Grid(c)
    exact, rhs = O.manufactured_rhs(g, c)
    code, x, info = g.solve(rhs, 1e-11, 10000)
    assert code == 0
    assert info["iterations"] == KERNEL_ITERATIONS[name][0 if pre == "ic0" else 1]
    # Manufactured recovery and residual gates of the campaign (pressure-multigrid.md:28-30).
    assert info["relative_residual"] <= 1.01e-10
    assert math.sqrt(float(np.sum((x - exact) ** 2)) / g.count) <= 1e-8


# docs/evidence/anisotropic-pressure.md:122-141 (shapes) and :41-60 (iterations IC(0) /
# point MG / candidate MG): the rough manufactured pressure sin(0.73 i) + 0.3 cos(0.17 i),
# centred, its operator image as the RHS (examples/pressure_probe.rs:60-68), tol 1e-14,
# at most 1200 iterations. The oracle's multigrid is the candidate (line/plane block
# smoothing with semicoarsening on anisotropic grids, multigrid/line.rs); on the three
# shapes below the anisotropy threshold it is the point cycle, whose counts equal the
# candidate's there.
ANISOTROPIC = {
    "isotropic": ([24, 2, 24], [1.0, 1.0, 1.0], "wall", 60, 8),
    "near-isotropic": ([96, 2, 24], [4.0, 0.1, 1.0], "wall", 122, 13),
    "threshold25": ([64, 2, 64], [1.0, 0.1, 0.2], "wall", 108, 24),
    "thin100": ([64, 2, 64], [1.0, 0.1, 0.1], "wall", 92, 5),
    "thin400": ([64, 2, 64], [1.0, 0.1, 0.05], "wall", 86, 5),
    "cube100": ([48, 48, 48], [1.0, 1.0, 0.1], "wall", 147, 5),
    "slab100": ([32, 32, 16], [1.0, 1.0, 0.05], "wall", 118, 6),
    "plate64": ([64, 8, 64], [1.0, 1.0, 1.0], "wall", 126, 11),
    "plate256": ([64, 16, 64], [1.0, 4.0, 1.0], "wall", 199, 12),
    "thin1600": ([64, 8, 64], [1.0, 1.0, 0.2], "wall", 152, 19),
    "thin6400": ([64, 8, 64], [1.0, 1.0, 0.1], "wall", 162, 18),
    "review-stretched": ([64, 8, 64], [1.0, 1.0, 0.02], "wall", 161, 17),
    "odd": ([33, 5, 17], [1.0, 1.0, 0.1], "wall", 87, 14),
    "periodic": ([31, 5, 17], [0.05, 1.0, 1.0], "periodic", 145, 7),
    "outlet": ([33, 5, 17], [1.0, 1.0, 0.1], "open", 92, 13),
    "stiff-two-cell": ([32, 2, 32], [1.0, 0.001, 1.0], "wall", 95, 9),
    "long-domain": ([128, 2, 16], [100.0, 1.0, 1.0], "wall", 220, 23),
    "short-stiff-axis": ([64, 64, 8], [1.0, 1.0, 0.01], "wall", 204, 6),
}


def anisotropic_case(name, pre):
    import copy

    from cases import LID_CAVITY

    n, size, bx, _, _ = ANISOTROPIC[name]
    c = copy.deepcopy(LID_CAVITY)
    c["grid"]["cells"] = list(n)
    c["domain"]["size_m"] = list(size)
    c["boundaries"]["x"] = bx
    if bx == "open":
        c["flow"]["initial_velocity_m_s"] = [1.0, 0.0, 0.0]
    c["numerics"]["pressure_preconditioner"] = pre
    return c


def rough_rhs(g):
    """pressure_probe.rs:60-68: the rough exact pressure, centred, and its operator image."""
    exact = np.array([math.sin(0.73 * v) + 0.3 * math.cos(0.17 * v) for v in range(g.count)])
    exact = g.center_nullspaces(exact)
    return exact, g.apply(exact)


@pytest.mark.parametrize("name", list(ANISOTROPIC))
@pytest.mark.parametrize("pre", ["ic0", "multigrid"])
def test_anisotropic_iteration_pins(O, name, pre):
    c = anisotropic_case(name, pre)
    g = O.Grid(c)
    exact, rhs = rough_rhs(g)
    code, x, info = g.solve(rhs, 1e-14, 1200)
    assert code == 0
    assert info["iterations"] == ANISOTROPIC[name][3 if pre == "ic0" else 4]
    # The campaign's gates (anisotropic-pressure.md:22-24).
    assert info["relative_residual"] <= 1.1e-12
    assert math.sqrt(float(np.mean((x - exact) ** 2))) <= 1e-8
