#!/usr/bin/env python3
"""Pressure-projection benchmark of the GB300 engine: Poisson solves/s at 1e-8.

Default (serving form): the wind-direction campaign mix - 36 cases on a 128x128x64 grid
(dx = 2 m, 30 seeded buildings, open x/y, ground_open_top z, neutral_rans 5 m/s, one case
per 10-degree wind direction) plus 16 cases at 96x96x48 with 0-20 buildings - served
through the continuous-batching server (cfdg_server) with every case's state resident.
One step is one time step of every case: the projection of its seeded u* sequence
(u*_{s+1} = project(u*_s) + 0.05 U[-1,1] on the free faces, one of four seeded noise
fields per case drawn before the timed region, in turn), dt = 0.1 s, mixed
FP32/FP64 multigrid PCG to 1e-8 relative residual. `value` is the closed-loop
throughput (a case's next step is submitted when its last one finishes); `serving`
adds an open-loop run with Poisson arrivals (mean 200/s, seed 5) and its p50/p99
latency; `plain_fp64` times the plain FP64 form on the same mix (all cases at once, one
stream per case) and `cpu_baseline` the
CPU restatement of the reference on all host cores. Inputs are synthetic (numpy PCG64
seeds); the reference publishes no dataset.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]
                  [--form serving|batched|mixed|plain]

`--form batched|mixed|plain` measure the 128x128x64 grid with 12 buildings (one case per
step, or 8 cases per batched step). Prints one JSON line (rank 0). `e2e` is the same
metric through the public C ABI with pinned host buffers, the host<->device copies
inside the timed region. `--impl reference` times the reference algorithm's CPU
restatement (the oracle; the Rust reference cannot be built here) on all host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Poisson solves/s at 1e-8 resid: batched mixed vs plain FP64; p50/p99 latency"
UNIT = "solves/s"
DT, TOL, MAX_IT = 0.1, 1e-8, 10000
LARGE_WORKLOAD = ("256x256x128 grid (8,388,608 cells), dx=2 m, 40 seeded box buildings, open x (inflow 5 m/s) / "
                  "wall y,z; projection of the seeded u* sequence, dt=0.1 s; mixed FP32/FP64 multigrid PCG to 1e-8")
WORKLOAD = ("128x128x64 grid, dx=2 m, 12 seeded box buildings, open x (inflow 5 m/s) / wall y,z; "
            "projection of the seeded u* sequence (0.05 U[-1,1] perturbation per step), dt=0.1 s; "
            "masked multigrid V(2,2)-PCG to 1e-8")


# DRAM bytes per cell of one staged red-black half sweep (ncu, k_rb_tma on 4 x 128x128x64:
# 29,541,888 B read + 18,944,000 B written over 4,194,304 cells).
RB_DRAM_BYTES_PER_CELL = (29541888 + 18944000) / 4194304
# DRAM bytes of one scalar transport step (both passes) per cell, from one ncu capture of
# k_scalar_pass on the 128x128x64 transport workload.
TRANSPORT_DRAM_BYTES_PER_CELL = (54496768 + 337408 + 62883584 + 301824) / 1048576
# The same for the MUSCL passes (one capture, blocks of 8 slices; the per-grid split of 4
# slices re-reads one more z face plane per block, mostly from L2).
MUSCL_DRAM_BYTES_PER_CELL = (54467328 + 542208 + 62851072 + 452352) / 1048576


def max_over_ranks(value, dist, device):
    """The largest of every rank's `value` (the job's time is its slowest replica's)."""
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            m = json.load(f)
        return float(m["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi samples of the SM clock and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def workload_case(pkg):
    return pkg.synth.config2(seed=1)


def noise_fields(pkg, g, count, seed):
    import numpy as np

    rng = np.random.default_rng(seed)
    fixed = ~((g.face_kind == pkg.grid.INTERIOR) | (g.face_kind == pkg.grid.OUTLET))
    out = rng.uniform(-0.05, 0.05, size=(count, g.n_faces))
    out[:, fixed] = 0.0
    return out


# ----------------------------------------------------------------------------- CPU legs
class CpuPool:
    """One oracle grid per host thread (the reference's hierarchy/factor caches live in the
    grid, so each thread keeps its own), solving concurrently; ctypes releases the GIL."""

    def __init__(self, case, threads):
        """`case`: one case for every thread, or a list with one case per thread."""
        from oracle import oracle as O
        import numpy as np

        import __graft_entry__ as entry

        pkg = entry.package()
        self.np = np
        self.cases = list(case) if isinstance(case, (list, tuple)) else [case] * threads
        assert len(self.cases) == threads
        self.threads = threads
        self.gs = [pkg.grid.Grid.build(c) for c in self.cases]
        self.pkg = pkg
        self.grids = [None] * threads
        self._each(lambda t: self.grids.__setitem__(t, O.Grid(self.cases[t])))

    def _each(self, fn):
        ths = [threading.Thread(target=fn, args=(t,)) for t in range(self.threads)]
        for th in ths:
            th.start()
        for th in ths:
            th.join()

    def solve(self, seeds):
        """One projection per thread on velocity seed seeds[t]; returns per-solve seconds."""
        times = [None] * self.threads
        codes = [None] * self.threads
        us = [self.pkg.synth.random_velocity(self.gs[t], s) for t, s in enumerate(seeds)]

        def work(t):
            p = self.np.zeros(self.gs[t].count)
            t0 = time.perf_counter()
            codes[t], ou, op, info = self.grids[t].project(us[t], p, DT, TOL, MAX_IT)
            times[t] = time.perf_counter() - t0
            if t == 0:
                self.first = (us[0], ou, op, info)  # thread 0's input and result (the oracle check)

        self._each(work)
        assert all(c == 0 for c in codes), codes
        return times


def cpu_baseline(case):
    threads = os.cpu_count() or 1
    pool = CpuPool(case, threads)
    pool.solve([500 + t for t in range(threads)])  # cold: hierarchy build, untimed
    times = pool.solve([1000 + t for t in range(threads)])
    med = statistics.median(times)
    return {"value": round(threads / med, 4), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{threads} concurrent warm solves of the workload (one per host thread, after one "
                      f"untimed cold solve each); median {med:.2f} s per solve"}


def mix_sample(pkg, threads):
    """One case of the serving mix per host thread, spread over the mix in order (the 36 large
    wind-direction cases come first, then the 16 smaller ones)."""
    mix = pkg.synth.config5()
    return [mix[(t * len(mix)) // threads] for t in range(threads)]


def cpu_baseline_mix(pkg, serve_one=None):
    """The oracle on all host threads over the mix. With `serve_one(case_index, u)` (the
    served path on the device), thread 0's timed input is also served and the result
    compared with the oracle's: the error of a served case against the FP64 reference
    algorithm (bound 1e-7 relative)."""
    import numpy as np

    threads = os.cpu_count() or 1
    cases = mix_sample(pkg, threads)
    pool = CpuPool(cases, threads)
    pool.solve([500 + t for t in range(threads)])  # cold: hierarchy build, untimed
    t0 = time.perf_counter()
    times = pool.solve([1000 + t for t in range(threads)])
    wall = time.perf_counter() - t0
    small = sum(1 for c in cases if c["grid"]["cells"][0] == 96)
    out = {"value": round(threads / wall, 4), "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"{threads} concurrent warm solves, one per host thread, over cases of the mix "
                     f"({threads - small} at 128x128x64, {small} at 96x96x48), after one untimed cold solve "
                     f"each; {wall:.2f} s wall, median {statistics.median(times):.2f} s per solve"}
    if serve_one is not None:
        u_in, ou, op, oinfo = pool.first
        gu, gp, code, info = serve_one(0, u_in)
        out["oracle_check"] = {
            "case": cases[0]["name"], "code": code, "gpu_iterations": info.iterations,
            "oracle_iterations": oinfo["iterations"],
            "max_rel_err_p": float(np.max(np.abs(gp - op)) / np.max(np.abs(op))),
            "max_rel_err_u": float(np.max(np.abs(gu - ou)) / np.max(np.abs(ou))), "bound": 1e-7,
            "how": "thread 0's timed input (U[-1,1] faces, seed 1000, p = 0) served through cfdg_server in the "
                   "mixed form, against the oracle's FP64 projection of the same input"}
    return out


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import __graft_entry__ as entry

    pkg = entry.package()
    from oracle import oracle as O

    O.build()
    threads = os.cpu_count() or 1
    serving = args.form == "serving"
    case = mix_sample(pkg, threads) if serving else workload_case(pkg)
    pool = CpuPool(case, threads)
    pool.solve(list(range(threads)))  # warm-up: the cold solve that builds each thread's hierarchy
    t0 = time.perf_counter()
    per = []
    for s in range(args.steps):
        per.extend(pool.solve([100 * (s + 1) + t for t in range(threads)]))
    total = time.perf_counter() - t0
    value = threads * args.steps / total
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * total / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": SERVE_WORKLOAD if serving else WORKLOAD,
                       "form": "CPU restatement of the reference (oracle), warm solves", "threads": threads,
                       "sample": ("one case of the mix per host thread, spread over the mix in order"
                                  if serving else "the workload's grid on every host thread")},
            "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"each step: {threads} concurrent warm solves (one per host thread), "
                                       f"median {statistics.median(per):.2f} s per solve; one cold warm-up step"},
            "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------------------- GPU leg
class Form:
    """One arithmetic form of the projection on `cases` copies of the workload (different
    velocity seeds): plain FP64 (one grid), mixed (one grid) or batched mixed (one batch)."""

    def __init__(self, pkg, torch, dev, stream, form, cases, steps, rank, case=None):
        import numpy as np

        self.pkg, self.torch, self.form = pkg, torch, form
        self.ncases = cases
        case = case or workload_case(pkg)
        self.grids = [pkg.grid.Grid.build(case)] * 1
        g = self.grids[0]
        self.g = g
        precision = "plain" if form == "plain" else "mixed"
        self.dgs = [pkg.pressure.DeviceGrid(g, preconditioner="multigrid", precision=precision) for _ in range(cases)]
        for d in self.dgs:
            d.set_stream(stream.cuda_stream)
        self.batch = None
        if form == "batched":
            self.batch = pkg.pressure.Batch(self.dgs)
            self.batch.set_stream(stream.cuda_stream)
        self.u0 = [pkg.synth.random_velocity(g, seed=100 * rank + i) for i in range(cases)]
        self.noise = [noise_fields(pkg, g, steps, seed=1000 * rank + 10 + i) for i in range(cases)]
        self.d_u = [torch.from_numpy(u).to(dev) for u in self.u0]
        self.d_p = [torch.zeros(g.count, dtype=torch.float64, device=dev) for _ in range(cases)]
        self.d_noise = [torch.from_numpy(n).to(dev) for n in self.noise]

    def step(self, s):
        for i in range(self.ncases):
            self.d_u[i].add_(self.d_noise[i][s])
        if self.batch is not None:
            res = self.batch.project_device([u.data_ptr() for u in self.d_u], [p.data_ptr() for p in self.d_p],
                                            [DT] * self.ncases, TOL, MAX_IT)
            for code, _ in res:
                assert code == 0, code
            return [info for _, info in res]
        return [d.project_device(u.data_ptr(), p.data_ptr(), DT, TOL, MAX_IT)
                for d, u, p in zip(self.dgs, self.d_u, self.d_p)]

    def e2e(self, stream, flush, K, W):
        """Through the public C ABI with pinned host buffers (H2D + solve + D2H per step)."""
        torch = self.torch
        n, g = self.ncases, self.g
        host_u = [[torch.from_numpy(self.u0[i] + self.noise[i][s]).pin_memory() for i in range(n)] for s in range(K)]
        host_p = [[torch.zeros(g.count, dtype=torch.float64).pin_memory() for _ in range(n)] for _ in range(K)]

        def one(s, copy=False):
            us = [h.clone().numpy() if copy else h.numpy() for h in host_u[s]]
            ps = [h.clone().numpy() if copy else h.numpy() for h in host_p[s]]
            if self.batch is not None:
                for code, _ in self.batch.project(us, ps, [DT] * n, TOL, MAX_IT):
                    assert code == 0
            else:
                for d, u, p in zip(self.dgs, us, ps):
                    d.project(u, p, DT, TOL, MAX_IT)

        for s in range(min(W, K)):
            one(s, copy=True)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for s in range(K):
            flush.zero_()
            one(s)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), 2 * n * 8 * (g.n_faces + g.count)

    def close(self):
        if self.batch is not None:
            self.batch.close()
        for d in self.dgs:
            d.close()


def timed_steps(form, torch, stream, flush, W, K, dist=None):
    for s in range(W):
        form.step(s)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    marks = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    infos = []
    ev0.record(stream)
    for s in range(K):
        flush.zero_()
        marks[s][0].record(stream)
        infos.extend(form.step(W + s))
        marks[s][1].record(stream)
    ev1.record(stream)
    torch.cuda.synchronize()
    total = ev0.elapsed_time(ev1)
    if dist:
        total = max_over_ranks(total, dist, flush.device)
    lat = sorted(a.elapsed_time(b) for a, b in marks)
    return total, lat, infos


SERVE_WORKLOAD = ("serving mix: 36 wind-direction cases (0..350 deg, 10 deg steps) on a 128x128x64 grid, dx=2 m, "
                  "30 seeded buildings, open x/y, ground_open_top z, neutral_rans 5 m/s; plus 16 cases at 96x96x48 "
                  "with 0-20 buildings; each case's u* sequence: its projected field plus one of four seeded "
                  "0.05 U[-1,1] noise fields on the free faces (drawn before the timed region, used in turn), "
                  "state resident across steps; mixed FP32/FP64 multigrid PCG to 1e-8 through the "
                  "continuous-batching server")


NOISE_POOL = 4


class Serving:
    """The serving mix through cfdg_server: every case's fields, hierarchy and FP32 state stay
    resident; a case's next step is its projected field plus the seeded perturbation."""

    def __init__(self, pkg, torch, dev, stream, slots, rank, autotune=True, chunk=0):
        import numpy as np

        self.pkg, self.torch, self.dev, self.stream = pkg, torch, dev, stream
        self.cases = pkg.synth.config5()
        self.grids = [pkg.grid.Grid.build(c) for c in self.cases]
        self.n = len(self.grids)
        self.dgs = [pkg.pressure.DeviceGrid(g, preconditioner="multigrid", precision="mixed") for g in self.grids]
        for d in self.dgs:
            d.set_stream(stream.cuda_stream)
        self.u0 = [pkg.synth.random_velocity(g, seed=5000 + 100 * rank + i) for i, g in enumerate(self.grids)]
        self.d_u = [torch.from_numpy(u).to(dev) for u in self.u0]
        self.d_p = [torch.zeros(g.count, dtype=torch.float64, device=dev) for g in self.grids]
        self.tuned = None
        if autotune:
            # The sweep counts with the shortest time to 1e-8 on this mix (first step's inputs).
            d_u0 = [u.clone() for u in self.d_u]

            def reset():
                for u, u0, p in zip(self.d_u, d_u0, self.d_p):
                    u.copy_(u0)
                    p.zero_()

            t0 = time.perf_counter()
            self.tuned = pkg.pressure.autotune(self.dgs, [u.data_ptr() for u in self.d_u],
                                               [p.data_ptr() for p in self.d_p], reset, [DT] * self.n, TOL, MAX_IT,
                                               stream_handle=stream.cuda_stream)
            torch.cuda.synchronize()
            self.tuned["seconds"] = round(time.perf_counter() - t0, 2)
            del d_u0
        self.server = pkg.pressure.Server(self.dgs, slots or self.n)
        self.server.set_stream(stream.cuda_stream)
        if chunk:
            self.server.set_chunk(chunk)
        self.free = []
        for g in self.grids:
            m = ((g.face_kind == pkg.grid.INTERIOR) | (g.face_kind == pkg.grid.OUTLET)).astype(np.float64)
            self.free.append(torch.from_numpy(m).to(dev))
        # The client's perturbations, drawn before any timed region: NOISE_POOL seeded fields
        # 0.05 U[-1,1] on the free faces per case (4.4 GB for the mix), used in turn, so
        # the timed loop adds one of them (one elementwise kernel) instead of drawing.
        self.noise = []
        for i, g in enumerate(self.grids):
            gn = torch.Generator(device=dev)
            gn.manual_seed(7000 + 100 * rank + i)
            self.noise.append([torch.rand(g.n_faces, dtype=torch.float64, device=dev, generator=gn)
                               .mul_(0.1).sub_(0.05).mul_(self.free[i]) for _ in range(NOISE_POOL)])
        self.drawn = [0] * self.n
        self.cells = [g.count for g in self.grids]

    def perturb(self, cs):
        """u*_{s+1} = project(u*_s) + 0.05 U[-1,1] on the free faces (on the device): each
        case's next pre-drawn noise field, the cases of one round in one multi-tensor add."""
        if not cs:
            return
        self.torch._foreach_add_([self.d_u[c] for c in cs],
                                 [self.noise[c][self.drawn[c] % NOISE_POOL] for c in cs])
        for c in cs:
            self.drawn[c] += 1

    def submit(self, c):
        return self.server.submit(c, self.d_u[c].data_ptr(), self.d_p[c].data_ptr(), DT, TOL, MAX_IT)

    def closed_loop(self, steps):
        """Every case runs `steps` consecutive time steps; a case's next step is submitted as soon
        as its previous one is finished. Returns (per-request latency s, infos, cell updates)."""
        srv = self.server
        left = [steps] * self.n
        inflight = {}
        lat, infos = [], []
        self.perturb(list(range(self.n)))
        for c in range(self.n):
            inflight[self.submit(c)] = (c, time.perf_counter())
            left[c] -= 1
        while inflight:
            if srv.progress() == 0:
                continue
            nxt = []
            for t in list(inflight):
                r = srv.result(t)
                if r is None:
                    continue
                code, info = r
                assert code == 0, code
                c, t0 = inflight.pop(t)
                lat.append(time.perf_counter() - t0)
                infos.append((c, info))
                if left[c] > 0:
                    nxt.append(c)
            self.perturb(nxt)
            for c in nxt:
                inflight[self.submit(c)] = (c, time.perf_counter())
                left[c] -= 1
        return lat, infos

    def e2e_loop(self, steps, seed=77):
        """The closed loop with the fields in host memory, through cfdg_server_submit_host:
        each request's u* and p are copied by the engine from page-locked host buffers to a
        device slot of its grid before it runs, and its projected u and p back to host
        buffers after it finishes; a ticket reports done once its results are in host memory.
        Every case keeps two requests in flight (the engine's two slots per grid), so the
        next input's copy overlaps the running solve; when one finishes the case's next is
        submitted. The copies run on the engine's copy streams beside the solves, all inside
        the timed region. The inputs are the fields the device loop left plus a seeded
        perturbation (two sets per case, used in turn, prepared before the timed region).
        Returns (milliseconds, H2D bytes, D2H bytes)."""
        import numpy as np

        torch = self.torch
        rng = np.random.default_rng(seed)
        base = [u.cpu().numpy() for u in self.d_u]
        h_in, h_p, o_u, o_p = [], [], [], []
        for c, g in enumerate(self.grids):
            m = self.free[c].cpu().numpy()
            h_in.append([torch.from_numpy(base[c] + m * rng.uniform(-0.05, 0.05, g.n_faces)).pin_memory()
                         for _ in range(2)])
            h_p.append(torch.zeros(g.count, dtype=torch.float64).pin_memory())
            o_u.append([torch.empty(g.n_faces, dtype=torch.float64).pin_memory() for _ in range(2)])
            o_p.append([torch.empty(g.count, dtype=torch.float64).pin_memory() for _ in range(2)])
        srv = self.server
        torch.cuda.synchronize()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        h2d = d2h = 0
        nxt = [0] * self.n
        inflight = {}

        def submit(c):
            nonlocal h2d
            k = nxt[c] % 2
            t = srv.submit_host(c, h_in[c][k].data_ptr(), h_p[c].data_ptr(), o_u[c][k].data_ptr(),
                                o_p[c][k].data_ptr(), DT, TOL, MAX_IT)
            inflight[t] = c
            nxt[c] += 1
            h2d += 8 * (h_in[c][k].numel() + h_p[c].numel())

        ev0.record(self.stream)
        for c in range(self.n):
            for _ in range(min(2, steps)):
                submit(c)
        while inflight:
            srv.progress()
            for t in list(inflight):
                r = srv.result(t)
                if r is None:
                    continue
                assert r[0] == 0, r[0]
                c = inflight.pop(t)
                d2h += 8 * (o_u[c][0].numel() + o_p[c][0].numel())
                if nxt[c] < steps:
                    submit(c)
        ev1.record(self.stream)
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1), h2d, d2h

    def poisson(self, requests, rate, seed):
        """Open loop: `requests` arrivals with exponential gaps (mean 1/rate), each for a case drawn
        uniformly; a case's arrivals are served in order, one at a time. Latency = completion -
        arrival, as the client sees it."""
        import numpy as np

        rng = np.random.default_rng(seed)
        arrive = np.cumsum(rng.exponential(1.0 / rate, size=requests))
        which = rng.integers(0, self.n, size=requests)
        srv = self.server
        backlog = [[] for _ in range(self.n)]
        inflight, busy = {}, [False] * self.n
        lat = []
        nxt = 0
        t_start = time.perf_counter()
        done = 0
        while done < requests:
            now = time.perf_counter() - t_start
            while nxt < requests and arrive[nxt] <= now:
                backlog[which[nxt]].append(arrive[nxt])
                nxt += 1
            for c in range(self.n):
                if backlog[c] and not busy[c]:
                    self.perturb([c])
                    inflight[self.submit(c)] = (c, backlog[c].pop(0))
                    busy[c] = True
            if not inflight:
                if nxt < requests:
                    time.sleep(max(0.0, min(arrive[nxt] - (time.perf_counter() - t_start), 0.002)))
                continue
            if srv.progress() == 0:
                continue
            for t in list(inflight):
                r = srv.result(t)
                if r is None:
                    continue
                assert r[0] == 0, r[0]
                c, a = inflight.pop(t)
                lat.append(time.perf_counter() - t_start - a)
                busy[c] = False
                done += 1
        span = time.perf_counter() - t_start
        return lat, span, float(arrive[-1])

    def close(self):
        self.server.close()
        for d in self.dgs:
            d.close()


def coarse_summary(stats):
    """Per coarse level over all cases: rows, max smoother colours, ELL entries per
    nonzero, closed groups."""
    out = []
    depth = max(len(c["levels"]) for c in stats["cases"])
    for l in range(depth):
        lv = [c["levels"][l] for c in stats["cases"] if len(c["levels"]) > l]
        nnz = sum(v["nnz"] for v in lv)
        out.append({"rows": sum(v["rows"] for v in lv), "max_colors": max(v["colors"] for v in lv),
                    "jacobi_cases": sum(1 for v in lv if v.get("smoother") == "l1-jacobi"),
                    "ell_per_nnz": round(sum(v["ell_entries"] for v in lv) / max(nnz, 1), 2),
                    "groups": sum(v["groups"] for v in lv), "blocks": sum(v["blocks"] for v in lv)})
    return out


def pct(xs, q):
    xs = sorted(xs)
    return xs[min(len(xs) - 1, int(q * len(xs)))]


def plain_mix(pkg, torch, dev, sv, world, flush):
    """The plain FP64 (parity) form on the whole serving mix concurrently: each case's
    projection of its first u* on its own grid handle and CUDA stream from its own host
    thread (ctypes releases the interpreter lock), so the solves overlap on the device.
    Returns solves/s of the mix (all cases / wall time of the concurrent run) and the
    latency of one large case alone."""
    n = sv.n
    dgs, streams, us, ps = [], [], [], []
    for c in range(n):
        d = pkg.pressure.DeviceGrid(sv.grids[c], preconditioner="multigrid", precision="plain")
        st = torch.cuda.Stream(dev)
        d.set_stream(st.cuda_stream)
        dgs.append(d)
        streams.append(st)
        us.append(torch.from_numpy(sv.u0[c]).to(dev))
        ps.append(torch.zeros(sv.grids[c].count, dtype=torch.float64, device=dev))
    infos = [None] * n

    def reset():
        for c in range(n):
            us[c].copy_(torch.from_numpy(sv.u0[c]))
            ps[c].zero_()
        torch.cuda.synchronize()

    def solve(c):
        infos[c] = dgs[c].project_device(us[c].data_ptr(), ps[c].data_ptr(), DT, TOL, MAX_IT)

    def all_at_once():
        ths = [threading.Thread(target=solve, args=(c,)) for c in range(n)]
        t0 = time.perf_counter()
        for th in ths:
            th.start()
        for th in ths:
            th.join()
        torch.cuda.synchronize()
        return time.perf_counter() - t0

    all_at_once()  # cold: hierarchy builds and graph captures, untimed
    reset()
    flush.zero_()
    torch.cuda.synchronize()
    wall = all_at_once()
    its = [i.iterations for i in infos]
    # One large case alone (latency of the parity form without concurrency).
    reset()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(streams[0])
    alone = dgs[0].project_device(us[0].data_ptr(), ps[0].data_ptr(), DT, TOL, MAX_IT)
    b.record(streams[0])
    torch.cuda.synchronize()
    # The plain form's kernels on the first 128x128x64 case: the FP64 operator with p.Ap,
    # one lexicographic Gauss-Seidel sweep of the fine level (the pipelined wavefront) and
    # one V-cycle (all levels), algorithmic bytes over CUDA-event time.
    peak, _ = peaks()
    kernels = {}
    for name, which, reps in (("operator_fp64", 0, 20), ("gs_sweep_fine_fp64", 1, 10), ("vcycle_fp64", 3, 5)):
        ms, by = dgs[0].time_kernel(which, reps)
        gbs = by / ms / 1e6 if by else None
        kernels[name] = {"ms": round(ms, 4), "GB/s": round(gbs, 1) if gbs else None, "algorithmic_bytes": by,
                         "frac": round(gbs / peak, 4) if gbs else None}
    for d in dgs:
        d.close()
    return {"value": round(world * n / wall, 4), "unit": UNIT, "wall_s": round(wall, 3), "kernels": kernels,
            "bound": "FP64 latency and rate: every product and sum rounded in the reference's order (no FMA), "
                     "lexicographic sweeps with a correctly rounded division per cell",
            "iterations_mean": round(statistics.mean(its), 2), "iterations_max": max(its),
            "ms_per_solve_alone_128x128x64": round(a.elapsed_time(b), 2), "iterations_alone": alone.iterations,
            "sample": f"all {n} cases of the mix projected at once (first u* of each, after an untimed cold solve), "
                      "one host thread and CUDA stream per case; solves / wall time"}


def run_serving(args, pkg, torch, dev, stream, flush, rank, world, dist, L):
    import numpy as np

    K, W = args.steps, args.warmup
    sv = Serving(pkg, torch, dev, stream, args.slots, rank, autotune=not args.no_autotune, chunk=args.chunk)
    n = sv.n
    t_setup = time.perf_counter()
    sv.closed_loop(W)  # first solves build every hierarchy and FP32 state
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t_setup
    if dist:
        dist.barrier()
    launches0 = L.cfdg_launch_count()
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    st0 = sv.server.stats()
    lat, infos = sv.closed_loop(K)
    ev1.record(stream)
    torch.cuda.synchronize()
    st1 = sv.server.stats()
    loop = {k: round(st1[k] - st0[k], 3) for k in ("rounds", "chunks", "chunk_device_ms", "progress_host_ms",
                                                   "progress_work_ms", "between_chunks_ms", "chunk_pairs",
                                                   "finished", "admitted")}
    loop["iterations_per_chunk"] = st1["iterations_per_chunk"]
    clk = clocks.stop()
    launches = L.cfdg_launch_count() - launches0
    total_ms = ev0.elapsed_time(ev1)
    if dist:
        total_ms = max_over_ranks(total_ms, dist, dev)
    solves = world * K * n
    value = solves / (total_ms / 1e3)
    cell_updates = sum(sv.cells[c] * i.iterations for c, i in infos)
    if args.only_loop:  # profiling runs: the closed loop alone
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": K,
                              "warmup": W, "ms_per_step": round(total_ms / K, 4), "only_loop": True,
                              "gpu_launches": int(launches), "server_loop": loop}), flush=True)
        sv.close()
        return 0
    # Open loop at the stated arrival rate (skipped with --requests 0).
    serving = None
    if args.requests > 0:
        plat, span, last_arrival = sv.poisson(args.requests, args.rate, seed=5)
        serving = {"arrivals": "Poisson, seed 5", "offered_per_s": args.rate, "requests": args.requests,
                   "throughput": round(args.requests / span, 2), "arrival_span_s": round(last_arrival, 3),
                   "p50_ms": round(1e3 * pct(plat, 0.50), 2), "p99_ms": round(1e3 * pct(plat, 0.99), 2),
                   "max_ms": round(1e3 * max(plat), 2), "slots": args.slots or n}
        # Latency against load: open loops at fractions of the closed-loop capacity just
        # measured, each about 1.5 s of arrivals.
        serving["latency_vs_load"] = []
        for q, frac in enumerate(float(f) for f in args.load_points.split(",") if f):
            rate = frac * value / world
            reqs = max(200, int(rate * 1.5))
            pl, sp, la = sv.poisson(reqs, rate, seed=11 + q)
            serving["latency_vs_load"].append(
                {"fraction_of_capacity": frac, "offered_per_s": round(rate, 1), "requests": reqs,
                 "throughput": round(reqs / sp, 1), "p50_ms": round(1e3 * pct(pl, 0.50), 2),
                 "p99_ms": round(1e3 * pct(pl, 0.99), 2)})
    # End to end through the host-buffer batch call: every case of the mix per step, H2D + D2H inside.
    bt = pkg.pressure.Batch(sv.dgs)
    bt.set_stream(stream.cuda_stream)
    coarse = coarse_summary(bt.stats())
    host_u = [torch.from_numpy(u).pin_memory() for u in sv.u0]
    work_u = [torch.empty_like(h).pin_memory() for h in host_u]
    work_p = [torch.zeros(g.count, dtype=torch.float64).pin_memory() for g in sv.grids]
    e2e_steps = max(1, min(K, 3))
    e2e_ms = 0.0
    for s in range(e2e_steps + 1):
        for w, h, p in zip(work_u, host_u, work_p):
            w.copy_(h)
            p.zero_()
        torch.cuda.synchronize()
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for code, _ in bt.project([w.numpy() for w in work_u], [p.numpy() for p in work_p], [DT] * n, TOL, MAX_IT):
            assert code == 0
        e1.record(stream)
        torch.cuda.synchronize()
        if s > 0:  # the first call builds the batch's state
            e2e_ms += e0.elapsed_time(e1)
    io = sum(8 * (g.n_faces + g.count) for g in sv.grids)
    e2e_batch = {"value": round(world * e2e_steps * n / (e2e_ms / 1e3), 4), "unit": UNIT,
                 "call": "cfdg_batch_project (host buffers) over all cases of the mix per step, lockstep"}
    # The headline end-to-end figure: the serving loop with the fields in host memory.
    srv_steps = max(2, K)
    srv_ms, h2d_b, d2h_b = sv.e2e_loop(srv_steps)
    if dist:
        srv_ms = max_over_ranks(srv_ms, dist, dev)
    e2e = {"value": round(world * srv_steps * n / (srv_ms / 1e3), 4), "unit": UNIT,
           "h2d_bytes_per_step": h2d_b // srv_steps, "d2h_bytes_per_step": d2h_b // srv_steps,
           "call": "cfdg_server_submit_host/progress/result: the engine copies each request's u and p from "
                   "page-locked host buffers into a device slot of its grid and the results back after the "
                   "request, on copy streams beside the solves; a ticket is done when its results are in host "
                   "memory; two requests per case in flight", "steps": srv_steps}
    kernels = {}
    for name, which, reps in (("rb_half_sweep_fp32", 0, 20), ("rb_half_sweep_fp32_unstaged", 4, 20),
                              ("operator_fp32", 1, 20), ("coarse_levels", 2, 10), ("vcycle_fp32", 3, 5),
                              ("true_residual_fp64", 5, 10), ("rhs_fp64", 6, 10),
                              ("level0_residual_restriction", 7, 20), ("level0_prolongation", 8, 20)):
        ms, b = bt.time_kernel(which, reps)
        kernels[name] = {"ms": round(ms, 4), "GB/s": round(b / ms / 1e6, 1) if b else None, "algorithmic_bytes": b}
    bt.close()
    peak, peak_kind = peaks()
    for kv in kernels.values():
        kv["frac"] = round(kv["GB/s"] / peak, 4) if kv["GB/s"] else None
    k = kernels["rb_half_sweep_fp32"]
    achieved = k["algorithmic_bytes"] / (k["ms"] * 1e-3) / 1e9
    # DRAM bytes per launch from the ncu capture of the same kernel on 4 x 128x128x64
    # (29.54 MB read + 18.94 MB written over 4,194,304 cells), scaled by the cells of this
    # launch (traffic grows with cells).
    traffic = round(RB_DRAM_BYTES_PER_CELL * sum(sv.cells), 0)
    roofline = {"bound": "hbm", "kernel": "fine-level red-black Gauss-Seidel half sweep, FP32, all cases of the mix",
                "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                "peak_source": peak_kind, "traffic": traffic,
                "traffic_source": "ncu dram__bytes_read+write of k_rb_tma on 4x128x128x64, scaled by cells",
                "algorithmic_bytes": k["algorithmic_bytes"], "ms_per_launch": k["ms"]}
    # Plain FP64 on the same mix, every case at once: one host thread and one stream per
    # case (the engine serialises calls per grid only), after an untimed cold solve each.
    plain = None
    if not args.skip_plain:
        plain = plain_mix(pkg, torch, dev, sv, world, flush)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        def serve_one(c, u_host):
            d_u = torch.from_numpy(u_host.copy()).to(dev)
            d_p = torch.zeros(sv.grids[c].count, dtype=torch.float64, device=dev)
            torch.cuda.synchronize()
            t = sv.server.submit(c, d_u.data_ptr(), d_p.data_ptr(), DT, TOL, MAX_IT)
            while (r := sv.server.result(t)) is None:
                sv.server.progress()
            return d_u.cpu().numpy(), d_p.cpu().numpy(), r[0], r[1]

        cpu = cpu_baseline_mix(pkg, serve_one)
    if rank == 0:
        its = [i.iterations for _, i in infos]
        line = {
            "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": round(total_ms / K, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": SERVE_WORKLOAD, "form": "serving (continuous batching, cfdg_server)",
                       "cases": n, "step": f"one time step of every case ({n} solves)",
                       "cells_per_step": sum(sv.cells), "l2": "inputs larger than L2: the mix holds "
                       f"{sum(sv.cells) * 8 * 10 / 1e9:.1f} GB of FP64 fields alone",
                       "parallelism": f"replicas x{world}"},
            "latency_ms": {"p50": serving["p50_ms"] if serving else None, "p99": serving["p99_ms"] if serving else None,
                           "unit": "per request, open loop at the offered rate",
                           "closed_loop_p50": round(1e3 * pct(lat, 0.5), 2),
                           "closed_loop_p99": round(1e3 * pct(lat, 0.99), 2)},
            "serving": serving, "setup_s": round(setup_s, 2), "server_loop": loop, "autotune": sv.tuned,
            "coarse_levels": coarse,
            "iterations_mean": round(statistics.mean(its), 2),
            "cell_updates_per_s": round(world * cell_updates / (total_ms / 1e3), 1),
            "e2e": e2e, "e2e_batch": e2e_batch, "roofline": roofline, "kernels": kernels, "plain_fp64": plain,
            "cpu_baseline": cpu, "gpu_launches": int(launches), "clocks": clk,
        }
        if plain:
            line["serving_vs_plain"] = round(value / plain["value"], 2)
        print(json.dumps(line), flush=True)
    sv.close()
    return 0


UNEVEN_WORKLOAD = ("64 uneven cases: shapes uniform over 48^3, 64x64x32, 96x96x48, 128x128x64, 160x160x80 (seeds "
                   "100-163), 0-20 seeded buildings, dx=2 m, inflow 5 m/s; each case's u* sequence as above; all 64 "
                   "projected by one batched call per step (mixed FP32/FP64 multigrid PCG to 1e-8)")


def run_uneven(args, pkg, torch, dev, stream, flush, rank, world, dist, L):
    """Survey configuration 4: 64 uneven cases in one batch (one graph-captured projection per step)."""
    import numpy as np

    K, W = args.steps, args.warmup
    cases = pkg.synth.config4()
    grids = [pkg.grid.Grid.build(c) for c in cases]
    n = len(grids)
    dgs = [pkg.pressure.DeviceGrid(g, preconditioner="multigrid", precision="mixed") for g in grids]
    for d in dgs:
        d.set_stream(stream.cuda_stream)
    u0 = [pkg.synth.random_velocity(g, seed=8000 + 100 * rank + i) for i, g in enumerate(grids)]
    d_u = [torch.from_numpy(u).to(dev) for u in u0]
    d_p = [torch.zeros(g.count, dtype=torch.float64, device=dev) for g in grids]
    free = [torch.from_numpy(((g.face_kind == pkg.grid.INTERIOR) | (g.face_kind == pkg.grid.OUTLET))
                             .astype(np.float64)).to(dev) for g in grids]
    gens = [torch.Generator(device=dev) for _ in grids]
    for i, gn in enumerate(gens):
        gn.manual_seed(9000 + 100 * rank + i)
    tuned = None
    if not args.no_autotune:
        d_u0 = [u.clone() for u in d_u]

        def reset():
            for u, v, p in zip(d_u, d_u0, d_p):
                u.copy_(v)
                p.zero_()

        t0 = time.perf_counter()
        tuned = pkg.pressure.autotune(dgs, [u.data_ptr() for u in d_u], [p.data_ptr() for p in d_p], reset,
                                      [DT] * n, TOL, MAX_IT, stream_handle=stream.cuda_stream)
        tuned["seconds"] = round(time.perf_counter() - t0, 2)
        del d_u0
    batch = pkg.pressure.Batch(dgs)
    batch.set_stream(stream.cuda_stream)

    def step():
        for i in range(n):
            noise = torch.rand(d_u[i].numel(), dtype=torch.float64, device=dev, generator=gens[i])
            d_u[i].add_(noise.mul_(0.1).sub_(0.05).mul_(free[i]))
        res = batch.project_device([u.data_ptr() for u in d_u], [p.data_ptr() for p in d_p], [DT] * n, TOL, MAX_IT)
        assert all(c == 0 for c, _ in res), [c for c, _ in res]
        return [i for _, i in res]

    for _ in range(W):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    launches0 = L.cfdg_launch_count()
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    infos = []
    ev0.record(stream)
    for _ in range(K):
        infos.extend(step())
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = L.cfdg_launch_count() - launches0
    total_ms = ev0.elapsed_time(ev1)
    if dist:
        total_ms = max_over_ranks(total_ms, dist, dev)
    value = world * K * n / (total_ms / 1e3)
    # End to end: the same batch on pinned host buffers, H2D and D2H inside the timed region.
    host_u = [torch.from_numpy(u).pin_memory() for u in u0]
    work_u = [torch.empty_like(h).pin_memory() for h in host_u]
    work_p = [torch.zeros(g.count, dtype=torch.float64).pin_memory() for g in grids]
    e2e_ms = 0.0
    e2e_steps = 2
    for s_ in range(e2e_steps):
        for w, h, p in zip(work_u, host_u, work_p):
            w.copy_(h)
            p.zero_()
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for code, _ in batch.project([w.numpy() for w in work_u], [p.numpy() for p in work_p], [DT] * n, TOL, MAX_IT):
            assert code == 0
        b.record(stream)
        torch.cuda.synchronize()
        e2e_ms += a.elapsed_time(b)
    io = sum(8 * (g.n_faces + g.count) for g in grids)
    batch.close()
    if rank == 0:
        shapes = {}
        for g in grids:
            shapes[str(tuple(g.n))] = shapes.get(str(tuple(g.n)), 0) + 1
        its = [i.iterations for i in infos]
        line = {"metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
                "ms_per_step": round(total_ms / K, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32+f64", "data": "synthetic",
                "config": {"workload": UNEVEN_WORKLOAD, "form": "batched mixed, one call per step", "cases": n,
                           "shapes": shapes, "cells_per_step": sum(g.count for g in grids),
                           "l2": "inputs larger than L2", "parallelism": f"replicas x{world}"},
                "iterations_mean": round(statistics.mean(its), 2), "iterations_max": max(its),
                "e2e": {"value": round(world * e2e_steps * n / (e2e_ms / 1e3), 4), "unit": UNIT,
                        "h2d_bytes_per_step": io, "d2h_bytes_per_step": io},
                "autotune": tuned, "gpu_launches": int(launches), "clocks": clk}
        print(json.dumps(line), flush=True)
    for d in dgs:
        d.close()
    return 0


STEP_WORKLOAD = ("128x128x64 grid, dx=2 m, 12 seeded box buildings, laminar inflow 5 m/s, open x / wall y,z; "
                 "SSPRK2 time steps of dt=0.1 s from the projected initial flow, two projections per step "
                 "(multigrid PCG to 1e-8), u and p resident on the device")


def run_stepping(args, pkg, torch, dev, stream, flush, rank, world, dist, L):
    """Survey configuration 2 as true laminar time stepping (cfdg_step_device)."""
    K, W = args.steps, args.warmup
    case = workload_case(pkg)
    g = pkg.grid.Grid.build(case)

    def stepper(precision):
        d = pkg.pressure.DeviceGrid(g, preconditioner="multigrid", precision=precision)
        d.set_stream(stream.cuda_stream)
        d.set_flow(case)
        u0, p0 = g.initial_velocity(), torch.zeros(g.count, dtype=torch.float64).numpy()
        d.project(u0, p0, DT, TOL, MAX_IT)  # the initial projection (solver.rs:1437)
        return d, torch.from_numpy(u0).to(dev), torch.from_numpy(p0).to(dev)

    d, d_u, d_p = stepper("mixed")
    for _ in range(W):
        d.step_device(d_u.data_ptr(), d_p.data_ptr(), DT, TOL, MAX_IT)
    torch.cuda.synchronize()
    # The end-to-end leg replays the same K steps from this state with u and p in host memory.
    h_u = torch.from_numpy(d_u.cpu().numpy()).pin_memory()
    h_p = torch.from_numpy(d_p.cpu().numpy()).pin_memory()
    if dist:
        dist.barrier()
    launches0 = L.cfdg_launch_count()
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    its = []
    ev0.record(stream)
    for _ in range(K):
        flush.zero_()
        its.append(d.step_device(d_u.data_ptr(), d_p.data_ptr(), DT, TOL, MAX_IT).iterations)
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = L.cfdg_launch_count() - launches0
    total_ms = ev0.elapsed_time(ev1)
    if dist:
        total_ms = max_over_ranks(total_ms, dist, dev)
    value = world * 2 * K / (total_ms / 1e3)
    # End to end: u and p from pinned host memory each step, back after it.
    e2e_steps = K
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(stream)
    for _ in range(e2e_steps):
        flush.zero_()
        d_u.copy_(h_u, non_blocking=True)
        d_p.copy_(h_p, non_blocking=True)
        d.step_device(d_u.data_ptr(), d_p.data_ptr(), DT, TOL, MAX_IT)
        h_u.copy_(d_u, non_blocking=True)
        h_p.copy_(d_p, non_blocking=True)
    b.record(stream)
    torch.cuda.synchronize()
    e2e_ms = a.elapsed_time(b)
    io = 8 * (g.n_faces + g.count)
    d.close()
    plain = None
    if not args.skip_plain:
        dp_, pu, pp = stepper("plain")
        dp_.step_device(pu.data_ptr(), pp.data_ptr(), DT, TOL, MAX_IT)
        torch.cuda.synchronize()
        a.record(stream)
        pits = [dp_.step_device(pu.data_ptr(), pp.data_ptr(), DT, TOL, MAX_IT).iterations for _ in range(2)]
        b.record(stream)
        torch.cuda.synchronize()
        pms = a.elapsed_time(b)
        plain = {"value": round(world * 4 / (pms / 1e3), 4), "unit": UNIT, "ms_per_step": round(pms / 2, 2),
                 "iterations_per_step": pits}
        dp_.close()
    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
                "ms_per_step": round(total_ms / K, 4), "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
                "config": {"workload": STEP_WORKLOAD, "form": "laminar SSPRK2 stepping, mixed-form projections",
                           "cells": g.count, "faces": g.n_faces, "l2": "256 MiB buffer written before every step",
                           "parallelism": f"replicas x{world}"},
                "time_steps_per_s": round(world * K / (total_ms / 1e3), 4),
                "iterations_per_step_mean": round(statistics.mean(its), 2),
                "e2e": {"value": round(world * 2 * e2e_steps / (e2e_ms / 1e3), 4), "unit": UNIT,
                        "h2d_bytes_per_step": io, "d2h_bytes_per_step": io},
                "plain_fp64": plain, "gpu_launches": int(launches), "clocks": clk}
        print(json.dumps(line), flush=True)
    return 0


TRANSPORT_WORKLOAD = ("128x128x64 grid, dx=2 m, 12 seeded box buildings, laminar inflow 5 m/s, open x / wall y,z; "
                      "one constituent on the flow projected from the initial velocity, linear upwind, cell "
                      "diffusivities 0.05-0.15 m2/s, a release of 1e-3 kg/m3/s in 64 cells near the inflow, "
                      "dt at CFL 0.4")
TRANSPORT_METRIC = "scalar transport SSPRK2 steps/s ({}, bit-identical to the reference arithmetic)"


def transport_fields(pkg, g, seed):
    """Diffusivity, source and a starting concentration of the transport workload."""
    import numpy as np

    rng = np.random.default_rng(seed)
    fluid = g.fluid.astype(bool)
    d = np.where(fluid, rng.uniform(0.05, 0.15, g.count), 0.0)
    source = np.zeros(g.count)
    nx, ny = int(g.n[0]), int(g.n[1])
    cell = np.arange(g.count)
    near = np.nonzero(fluid & (cell % nx < 8) & (np.abs((cell // nx) % ny - ny // 2) < 4))[0]
    source[rng.choice(near, 64, replace=False)] = 1e-3
    c = np.where(fluid, rng.uniform(0.0, 1e-3, g.count), 0.0)
    return d, source, c


def transport_cpu_baseline(case, u, d, source, c, dt, muscl=False):
    """The oracle's advance_scalar on every host thread, each on its own grid and copy."""
    from oracle import oracle as O

    threads = os.cpu_count() or 1
    grids = [None] * threads
    steps = 10

    def build(t):
        grids[t] = O.Grid(case)

    def work(t):
        x = c
        for _ in range(steps):
            x = grids[t].scalar_step(x, u, d, source, dt, muscl=muscl)

    for fn in (build, work):
        ths = [threading.Thread(target=fn, args=(t,)) for t in range(threads)]
        t0 = time.perf_counter()
        for th in ths:
            th.start()
        for th in ths:
            th.join()
        wall = time.perf_counter() - t0
    return {"value": round(threads * steps / wall, 4), "unit": "steps/s", "cores": threads, "kind": "port",
            "sample": f"{threads} host threads, each {steps} SSPRK2 steps of the workload on its own oracle grid; "
                      f"{wall:.2f} s wall"}


def run_transport(args, pkg, torch, dev, stream, flush, rank, world, dist, L):
    """Survey row f2: receptor transport on the device (cfdg_scalar_step_device)."""
    import numpy as np

    K, W = args.steps, args.warmup
    case = workload_case(pkg)
    g = pkg.grid.Grid.build(case)
    dg = pkg.pressure.DeviceGrid(g, preconditioner="multigrid", precision="mixed")
    dg.set_stream(stream.cuda_stream)
    u, p = g.initial_velocity(), np.zeros(g.count)
    dg.project(u, p, DT, TOL, MAX_IT)
    d, source, c = transport_fields(pkg, g, 7)
    # CFL 0.4 on the largest transporting-face speed, and the explicit diffusion limit.
    moving = np.isin(g.face_kind, (pkg.grid.INTERIOR, pkg.grid.INLET, pkg.grid.OUTLET))
    dmin = float(min(g.dx))
    dt = min(0.4 * dmin / float(np.max(np.abs(u[moving]))), 0.1 * dmin * dmin / float(np.max(d)))
    d_u = torch.from_numpy(u).to(dev)
    d_d, d_s = torch.from_numpy(d).to(dev), torch.from_numpy(source).to(dev)
    d_c = torch.from_numpy(c.copy()).to(dev)
    muscl = args.advection == "muscl"
    dg.set_advection(args.advection)

    def step():
        dg.scalar_step_device(d_u.data_ptr(), d_c.data_ptr(), d_d.data_ptr(), d_s.data_ptr(), dt)

    for _ in range(W):
        flush.zero_()
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    launches0 = L.cfdg_launch_count()
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for k in range(K):
        flush.zero_()
        ev[k][0].record(stream)
        step()
        ev[k][1].record(stream)
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = L.cfdg_launch_count() - launches0
    total_ms = ev0.elapsed_time(ev1)
    kern_ms = sum(a.elapsed_time(b) for a, b in ev) / K
    if dist:
        total_ms = max_over_ranks(total_ms, dist, dev)
    value = world * K / (total_ms / 1e3)
    # End to end: the step's inputs (u, d, source, c) from pinned host memory, c back.
    h_u, h_d, h_s = (torch.from_numpy(x).pin_memory() for x in (u, d, source))
    h_c = torch.from_numpy(d_c.cpu().numpy()).pin_memory()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(stream)
    for _ in range(K):
        flush.zero_()
        d_u.copy_(h_u, non_blocking=True)
        d_d.copy_(h_d, non_blocking=True)
        d_s.copy_(h_s, non_blocking=True)
        d_c.copy_(h_c, non_blocking=True)
        step()
        h_c.copy_(d_c, non_blocking=True)
    b.record(stream)
    torch.cuda.synchronize()
    e2e_ms = a.elapsed_time(b)
    if dist:
        e2e_ms = max_over_ranks(e2e_ms, dist, dev)
    n, f = g.count, g.n_faces
    # Algorithmic bytes of one step (two passes): per cell c, d, source, the stage or c
    # written, the fluid flag, and three faces' velocity and kind; the second pass also
    # reads the cell's own c.
    step_bytes = (60 + 68) * n
    peak, peak_kind = peaks()
    achieved = step_bytes / (kern_ms / 1e3) / 1e9
    dg.close()
    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            cpu = transport_cpu_baseline(case, u, d, source, c, dt, muscl)
        scheme = "MUSCL, monotonized-central limiter" if muscl else "linear upwind"
        if muscl:
            roofline_kernel = "k_scalar_pass<MUSCL> stage + combine (one step)"
            limiter = ("FP64 pipe (78 % active under ncu; each face once, with one limited slope of its "
                       "upwind cell; minmod's sign test on the bits)")
        else:
            roofline_kernel = "k_scalar_pass stage + combine (one step)"
            limiter = "FP64 pipe (72 % active under ncu; about 24 FP64 adds and multiplies per cell and pass)"
        line = {"metric": TRANSPORT_METRIC.format(scheme), "value": round(value, 4), "unit": "steps/s", "n_gpus": world,
                "steps": K, "warmup": W, "ms_per_step": round(total_ms / K, 4), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": TRANSPORT_WORKLOAD.replace("linear upwind", scheme), "cells": n, "faces": f, "dt_s": dt,
                           "l2": "256 MiB buffer written before every step", "parallelism": f"replicas x{world}"},
                "cell_updates_per_s": round(world * K * n / (total_ms / 1e3), 1),
                "e2e": {"value": round(world * K / (e2e_ms / 1e3), 4), "unit": "steps/s",
                        "h2d_bytes_per_step": 8 * (f + 3 * n), "d2h_bytes_per_step": 8 * n},
                "roofline": {"bound": "hbm", "kernel": roofline_kernel, "limiter": limiter,
                             "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                             "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                             "algorithmic_bytes_per_step": step_bytes, "kernel_ms_per_step": round(kern_ms, 4),
                             "traffic": round((MUSCL_DRAM_BYTES_PER_CELL if muscl
                                               else TRANSPORT_DRAM_BYTES_PER_CELL) * n, 0)},
                "cpu_baseline": cpu, "gpu_launches": int(launches), "clocks": clk}
        print(json.dumps(line), flush=True)
    return 0


ANISO_WORKLOAD = ("cube100: 48x48x48 cells over 1.0 x 1.0 x 0.1 m (weights 100x apart), wall x/z, periodic y, "
                  "rough manufactured pressure sin(0.73 i) + 0.3 cos(0.17 i) (its operator image as the RHS), "
                  "tol 1e-14, plain FP64 multigrid with z-line block smoothing and semicoarsening, hierarchy cached")


def run_anisotropic(args, pkg, torch, dev, stream, flush, rank, world, dist, L):
    """Survey row a14 / f4: the anisotropic shape cube100 of the reference's campaign."""
    import math

    import numpy as np

    K, W = args.steps, args.warmup
    # The lid-cavity case re-gridded as the campaign's cube100 (benchmark_anisotropy.py:23,
    # case_for), and the iterations it recorded (anisotropic-pressure.md:50).
    pin = 5
    case = pkg.synth.case((48, 48, 48), 1.0, boundaries=("wall", "periodic", "wall"), inflow=0.0,
                          preconditioner="multigrid", name="cube100")
    case["domain"]["size_m"] = [1.0, 1.0, 0.1]
    g = pkg.grid.Grid.build(case)
    dg = pkg.pressure.DeviceGrid(g, preconditioner="multigrid")
    dg.set_stream(stream.cuda_stream)
    exact = np.array([math.sin(0.73 * v) + 0.3 * math.cos(0.17 * v) for v in range(g.count)])
    dg.center_nullspaces(exact)
    rhs = dg.apply(exact)
    t0 = time.perf_counter()
    x, info = dg.solve_scaled(rhs, None, 1e-14, 1200)  # cold: builds the hierarchy
    cold_s = time.perf_counter() - t0
    for _ in range(W):
        dg.solve_scaled(rhs, None, 1e-14, 1200)
    torch.cuda.synchronize()
    launches0 = L.cfdg_launch_count()
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    its = []
    ev0.record(stream)
    for _ in range(K):
        flush.zero_()
        x, info = dg.solve_scaled(rhs, None, 1e-14, 1200)
        its.append(info.iterations)
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = L.cfdg_launch_count() - launches0
    total_ms = ev0.elapsed_time(ev1)
    if dist:
        total_ms = max_over_ranks(total_ms, dist, dev)
    rms = math.sqrt(float(np.mean((x - exact) ** 2)))
    dg.close()
    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            from oracle import oracle as O

            og = O.Grid(case)
            og.set_preconditioner("multigrid")
            og.solve(rhs, 1e-14, 1200)  # cold
            t0 = time.perf_counter()
            og.solve(rhs, 1e-14, 1200)
            cs = time.perf_counter() - t0
            cpu = {"value": round(1.0 / cs, 4), "unit": "solves/s", "cores": 1, "kind": "port",
                   "sample": f"one warm solve of the workload by the oracle on one host thread ({cs * 1e3:.1f} ms); "
                             "the reference's own record for this shape: 141.581 ms per cached solve on one "
                             "EPYC 9V74 thread (docs/evidence/anisotropic-pressure.md:50)"}
        line = {"metric": "anisotropic Poisson solves/s at 1e-14 (plain FP64 multigrid, block smoothing)",
                "value": round(world * K / (total_ms / 1e3), 4), "unit": "solves/s", "n_gpus": world, "steps": K,
                "warmup": W, "ms_per_step": round(total_ms / K, 3), "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": ANISO_WORKLOAD, "cells": g.count,
                           "l2": "256 MiB buffer written before every solve", "parallelism": f"replicas x{world}"},
                "iterations": its[-1], "iterations_published": pin, "rms_error": rms, "cold_solve_s": round(cold_s, 3),
                "e2e": {"value": round(world * K / (total_ms / 1e3), 4), "unit": "solves/s",
                        "h2d_bytes_per_step": 8 * g.count, "d2h_bytes_per_step": 8 * g.count,
                        "note": "cfdg_solve_scaled takes host arrays: the copies are inside every timed solve"},
                "cpu_baseline": cpu, "gpu_launches": int(launches), "clocks": clk}
        print(json.dumps(line), flush=True)
    return 0


def run_engine(args):
    import torch

    import __graft_entry__ as entry

    entry.build()
    pkg = entry.package()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    # One real stream for torch's helpers, the engine and the events (the legacy default
    # stream's handle is NULL, which would leave the engine on its own stream).
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    flush = torch.empty(64 << 20, dtype=torch.float32, device=dev)  # 256 MiB > L2 (129 MB)
    K, W = args.steps, args.warmup
    L = pkg.engine.load()
    if args.form in ("serving", "uneven", "stepping", "transport", "anisotropic"):
        run = {"serving": run_serving, "uneven": run_uneven, "stepping": run_stepping,
               "transport": run_transport, "anisotropic": run_anisotropic}[args.form]
        rc = run(args, pkg, torch, dev, stream, flush, rank, world, dist, L)
        if dist:
            dist.destroy_process_group()
        return rc
    ncases = args.cases if args.form == "batched" else 1
    # --form large: the mixed form on the 256x256x128 grid with 40 buildings (8.4 M cells).
    big = pkg.synth.config3() if args.form == "large" else None
    fname = "mixed" if args.form == "large" else args.form
    form = Form(pkg, torch, dev, stream, fname, ncases, K + W, rank, case=big)
    g = form.g
    launches0 = L.cfdg_launch_count()
    clocks = Clocks(local)
    clocks.start()
    total_ms, lat, infos = timed_steps(form, torch, stream, flush, W, K, dist)
    clk = clocks.stop()
    launches = L.cfdg_launch_count() - launches0
    solves = world * K * ncases
    value = solves / (total_ms / 1e3)
    e2e_ms, io_bytes = form.e2e(stream, flush, K, W)
    if dist:
        e2e_ms = max_over_ranks(e2e_ms, dist, dev)
    e2e = {"value": round(solves / (e2e_ms / 1e3), 4), "unit": UNIT, "h2d_bytes_per_step": io_bytes // 2,
           "d2h_bytes_per_step": io_bytes // 2}
    peak, peak_kind = peaks()
    kernels = {}
    if args.form == "plain":
        d = form.dgs[0]
        for name, which, reps in (("operator_fp64", 0, 50), ("gs_sweep_fine_fp64", 1, 10), ("vcycle_fp64", 3, 3)):
            ms, b = d.time_kernel(which, reps)
            kernels[name] = {"ms": round(ms, 4), "GB/s": round(b / ms / 1e6, 1) if b else None,
                             "algorithmic_bytes": b}
        dom = "gs_sweep_fine_fp64"
        dom_desc = "fine-level lexicographic Gauss-Seidel sweep, FP64 (pipelined wavefront)"
    else:
        bt = form.batch if form.batch is not None else None
        if bt is None:
            bt = pkg.pressure.Batch(form.dgs)
            bt.set_stream(stream.cuda_stream)
            form.step(0)  # leave every case with live vectors
        for name, which, reps in (("rb_half_sweep_fp32", 0, 50), ("operator_fp32", 1, 50),
                                  ("coarse_levels", 2, 20), ("vcycle_fp32", 3, 10)):
            ms, b = bt.time_kernel(which, reps)
            kernels[name] = {"ms": round(ms, 4), "GB/s": round(b / ms / 1e6, 1) if b else None,
                             "algorithmic_bytes": b}
        if form.batch is None:
            bt.close()
        dom = "rb_half_sweep_fp32"
        dom_desc = "fine-level red-black Gauss-Seidel half sweep, FP32, all cases of the batch"
    k = kernels[dom]
    achieved = k["algorithmic_bytes"] / (k["ms"] * 1e-3) / 1e9
    roofline = {"bound": "hbm", "kernel": dom_desc, "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": peak_kind, "traffic": None,
                "algorithmic_bytes": k["algorithmic_bytes"], "ms_per_launch": k["ms"]}
    # The plain FP64 form on the same workload, for the batched-mixed vs plain comparison.
    plain = None
    if args.form != "plain" and not args.skip_plain:
        pf = Form(pkg, torch, dev, stream, "plain", 1, 2 + 1, rank + 7, case=big)
        pms, plat, pinfos = timed_steps(pf, torch, stream, flush, 1, 2, dist)
        plain = {"value": round(world * 2 / (pms / 1e3), 4), "unit": UNIT, "ms_per_solve": round(pms / 2, 2),
                 "iterations_mean": round(statistics.mean(i.iterations for i in pinfos), 1), "steps": 2}
        pf.close()
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline and args.form != "large":
        cpu = cpu_baseline(workload_case(pkg))
    if rank == 0:
        its = [i.iterations for i in infos]
        outer = [i.work.get("refinement_steps", 0) for i in infos]
        line = {
            "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": round(total_ms / K, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.form == "plain" else "f32+f64",
            "data": "synthetic",
            "config": {"workload": LARGE_WORKLOAD if args.form == "large" else WORKLOAD,
                       "form": {"plain": "plain FP64 multigrid PCG (parity form)",
                                "mixed": "mixed FP32/FP64 multigrid PCG, one case",
                                "large": "mixed FP32/FP64 multigrid PCG, one 8.4 M-cell case",
                                "batched": f"batched mixed FP32/FP64, {ncases} cases per step"}[args.form],
                       "cases_per_step": ncases, "cells_per_case": g.count, "faces_per_case": g.n_faces,
                       "l2": "256 MiB buffer written before every step (inside the timed region)",
                       "parallelism": f"replicas x{world}"},
            "latency_ms": {"p50": round(lat[len(lat) // 2], 3), "p99": round(lat[min(len(lat) - 1, int(0.99 * len(lat)))], 3),
                           "unit": "per step"},
            "iterations_mean": round(statistics.mean(its), 2),
            "refinement_steps_mean": round(statistics.mean(outer), 2),
            "solve_breakdown": {"device_ms": round(1e3 * statistics.mean(i.work.get("device_seconds", 0) for i in infos), 3),
                                "loop_ms": round(1e3 * statistics.mean(i.work.get("loop_seconds", 0) for i in infos), 3),
                                "graph_chunks": round(statistics.mean(i.work.get("graph_launches", 0) for i in infos), 2)},
            "cell_updates_per_s": round(g.count * statistics.mean(its) * value, 1),
            "e2e": e2e, "roofline": roofline, "kernels": kernels, "plain_fp64": plain, "cpu_baseline": cpu,
            "gpu_launches": int(launches), "clocks": clk,
        }
        if plain:
            line["batched_vs_plain"] = round(value / plain["value"], 2)
        print(json.dumps(line), flush=True)
    form.close()
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--form", default="serving",
                    choices=["plain", "mixed", "batched", "serving", "uneven", "large", "stepping", "transport",
                             "anisotropic"])
    ap.add_argument("--advection", default="linear_upwind", choices=["linear_upwind", "muscl"],
                    help="transport: the constituents' advection scheme")
    ap.add_argument("--slots", type=int, default=0, help="serving: cases on the GPU at once (0: all)")
    ap.add_argument("--requests", type=int, default=520, help="serving: open-loop requests")
    ap.add_argument("--rate", type=float, default=200.0, help="serving: mean arrivals per second")
    ap.add_argument("--load-points", default="0.5,0.75,0.9",
                    help="serving: open loops at these fractions of the measured capacity ('' for none)")
    ap.add_argument("--chunk", type=int, default=0, help="serving: iterations per graph chunk (0: the engine's)")
    ap.add_argument("--no-autotune", action="store_true", help="serving: keep the default V(2,2) sweeps")
    ap.add_argument("--only-loop", action="store_true", help="serving: the closed loop only (for launch lists)")
    ap.add_argument("--cases", type=int, default=8, help="cases per step of the batched form")
    ap.add_argument("--skip-plain", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_engine(args)


if __name__ == "__main__":
    sys.exit(main())
