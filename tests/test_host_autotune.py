"""pressure.autotune's host logic on the CPU with stand-in grids and batches: every
candidate is applied to every grid (sweeps and coarse-correction scale), timed on its
second call, candidates whose projection fails are dropped, and the fastest is applied
and reported with its key; the sweep tile shape is picked the same way from the staged
half sweep's kernel time, and not at all when the mix does not take the staged path."""
import pytest


class FakeGrid:
    def __init__(self):
        self.cycle, self.scale, self.tile = (2, 2), 1.8, (32, 2)

    def set_sweep_tile(self, rows, stages):
        self.tile = (rows, stages)

    def set_cycle(self, a, b):
        self.cycle = (a, b)

    def set_coarse_scale(self, s):
        self.scale = s


class Info:
    def __init__(self, it):
        self.iterations = it


def make_batch(grids, timings, failing, clock, staged=False, tile_us=None):
    class FakeBatch:
        def __init__(self, dgs):
            assert dgs is grids
            self.cand = (grids[0].cycle[0], grids[0].cycle[1], grids[0].scale)
            assert all((g.cycle[0], g.cycle[1], g.scale) == self.cand for g in grids)
            self.tile = grids[0].tile
            assert all(g.tile == self.tile for g in grids)

        def stats(self):
            return {"staged_sweeps": staged}

        def time_kernel(self, which, reps):
            assert which == 0
            return tile_us[self.tile] * 1e-3, 1.0

        def set_stream(self, h):
            pass

        def project_device(self, u, p, dts, tol, max_iter):
            clock[0] += timings.get(self.cand, 0.0)
            code = 33 if self.cand in failing else 0
            return [(code, Info(10 * self.cand[0] + self.cand[1])) for _ in grids]

        def close(self):
            pass

    return FakeBatch


def test_autotune_picks_the_fastest_converging_candidate(pkg, monkeypatch):
    P = pkg.pressure
    grids = [FakeGrid(), FakeGrid()]
    cands = ((1, 2, 1.7), (2, 2, 1.85), (1, 3, 1.85))
    timings = {(1, 2, 1.7): 0.05, (2, 2, 1.85): 0.01, (1, 3, 1.85): 0.03}
    clock = [0.0]
    monkeypatch.setattr(P, "Batch", make_batch(grids, timings, {(2, 2, 1.85)}, clock))
    monkeypatch.setattr(__import__("time"), "perf_counter", lambda: clock[0])
    resets = []
    out = P.autotune(grids, [0, 0], [0, 0], lambda: resets.append(1), [0.1, 0.1], candidates=cands)
    # (2, 2, 1.85) is fastest but fails: (1, 3, 1.85) wins and is applied to every grid.
    assert out["choice"] == [1, 3, 1.85]
    assert all(g.cycle == (1, 3) and g.scale == 1.85 for g in grids)
    assert set(out["ms"]) == {"1,2,1.7", "1,3,1.85"}
    assert out["ms"]["1,3,1.85"] == pytest.approx(30.0)
    # Two calls per candidate (one for the failing one, which stops at its first call), then
    # one reset after the choice is applied.
    assert len(resets) == 2 + 1 + 2 + 1


def test_autotune_picks_the_fastest_sweep_tile(pkg, monkeypatch):
    P = pkg.pressure
    grids = [FakeGrid(), FakeGrid()]
    tile_us = {(8, 4): 98.0, (16, 2): 93.0, (16, 3): 90.0, (16, 4): 83.5, (32, 2): 81.9, (32, 3): 103.0}
    clock = [0.0]
    monkeypatch.setattr(P, "Batch", make_batch(grids, {}, set(), clock, staged=True, tile_us=tile_us))
    resets = []
    out = P.autotune_sweep_tile(grids, [0, 0], [0, 0], lambda: resets.append(1), [0.1, 0.1])
    assert out["choice"] == [32, 2] and all(g.tile == (32, 2) for g in grids)
    assert out["us"] == {"%dx%d" % k: v for k, v in tile_us.items()}
    assert len(resets) == len(tile_us) + 1  # one projection per candidate, then the applied choice
    # A mix without the staged path: nothing is tuned and the grids keep their shape.
    grids2 = [FakeGrid()]
    grids2[0].tile = (16, 4)
    monkeypatch.setattr(P, "Batch", make_batch(grids2, {}, set(), clock, staged=False, tile_us=tile_us))
    assert P.autotune_sweep_tile(grids2, [0], [0], lambda: None, [0.1]) is None
    assert grids2[0].tile == (16, 4)
