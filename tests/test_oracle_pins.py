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

from cases import ANISOTROPIC, CANYON_93K, KERNEL_ITERATIONS, anisotropic_case, kernel_case, rough_rhs


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
