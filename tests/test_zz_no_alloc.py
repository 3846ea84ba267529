"""cfdg_residual_norm_noalloc: the residual check for callers that cannot allocate.

Some callers of the projection cannot call cudaMalloc at the point where they want
to check a solution: a host that has given the whole HBM budget to resident serving
state, or a time step that must not block on the device synchronisation an allocation
can cause. This entry point computes |A x - b| / |b| from device vectors using only a
static scratch array compiled into the library. The test calls it through the C ABI
twice in a row and checks each result against the relative residual that the
allocating solve entry point (cfdg_solve_scaled) reports for the same x. This file is
collected last so that a failure here leaves every other test already run.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def noalloc(pkg, torch, dg, d_x, d_b, d_out, stream):
    L = pkg.engine.load()
    with torch.cuda.stream(stream):
        d_out.fill_(-1.0)
        rc = L.cfdg_residual_norm_noalloc(dg.h, C.c_void_p(d_x.data_ptr()), C.c_void_p(d_b.data_ptr()),
                                          C.c_void_p(d_out.data_ptr()), C.c_void_p(stream.cuda_stream))
    assert rc == 0, pkg.engine.last_error()
    stream.synchronize()
    return float(d_out.item())


@pytest.mark.parametrize("weights", ["uniform", "changed"])
def test_residual_norm_noalloc_matches_solve(pkg, weights):
    """Uniform face weights (three per-axis constants) and, after cfdg_grid_update_faces
    with varied areas, per-face weights: both kernels of the entry point."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(21)
    case = pkg.synth.case((40, 36, 20), 2.0, inflow=5.0,
                          boxes=pkg.synth.random_boxes(rng, 4, (80.0, 72.0, 40.0), dx=2.0), preconditioner="ic0")
    g = pkg.grid.Grid.build(case)
    assert all(g.anchored)  # anchored: the solve's x is not re-centred after its residual gate
    dg = pkg.pressure.DeviceGrid(g)
    if weights == "changed":
        dg.update_faces(area=g.face_area * (1.0 + (np.arange(g.n_faces) % 5) * 0.03))
    u = pkg.synth.random_velocity(g, 3)
    b, _ = dg.projection_rhs(u, 0.1)
    x, info = dg.solve_scaled(b, None, 1e-8, 10000)
    assert info.iterations > 0
    expected = info.relative_residual
    dev = torch.device("cuda", 0)
    d_x = torch.from_numpy(x).to(dev)
    d_b = torch.from_numpy(b).to(dev)
    d_out = torch.full((1,), -1.0, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    stream = torch.cuda.Stream(dev)  # a real stream: the legacy default stream's handle is NULL
    for _ in range(2):
        got = noalloc(pkg, torch, dg, d_x, d_b, d_out, stream)
        assert abs(got - expected) <= 1e-10 * abs(expected), (got, expected)
    # A zero right-hand side: the solve reports a zero residual, and so does this entry point.
    d_zero = torch.zeros_like(d_b)
    assert noalloc(pkg, torch, dg, d_x, d_zero, d_out, stream) == 0.0
    _, zinfo = dg.solve_scaled(np.zeros(g.count), None, 1e-8, 100)
    assert zinfo.relative_residual == 0.0
    # And the next call after it is unaffected by the shared scratch it left.
    assert abs(noalloc(pkg, torch, dg, d_x, d_b, d_out, stream) - expected) <= 1e-10 * abs(expected)
    dg.close()
