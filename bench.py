#!/usr/bin/env python3
"""Pressure-projection benchmark of the GB300 engine: Poisson solves/s at 1e-8.

Workload (one step = one projection solve): the 128x128x64 grid (dx = 2 m) with 12
seeded box buildings, open x / wall y,z, inflow 5 m/s; the projection of the
seeded u* sequence u*_{s+1} = project(u*_s) + 0.05 U[-1,1] (fixed faces untouched),
dt = 0.1 s, multigrid V(2,2)-preconditioned CG to 1e-8 relative residual. Inputs
are synthetic (numpy PCG64 seeds); the reference publishes no dataset.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference] [--form plain]

Prints one JSON line (rank 0). `value` is device-resident throughput; `e2e` is the
same metric through the public C ABI (cfdg_project) with pinned host buffers, the
host<->device copies inside the timed region. `--impl reference` times the
reference algorithm's CPU restatement (the oracle; the Rust reference cannot be
built here) on all host cores.
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
WORKLOAD = ("128x128x64 grid, dx=2 m, 12 seeded box buildings, open x (inflow 5 m/s) / wall y,z; "
            "projection of the seeded u* sequence (0.05 U[-1,1] perturbation per step), dt=0.1 s; "
            "masked multigrid V(2,2)-PCG to 1e-8")


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
        from oracle import oracle as O
        import numpy as np

        import __graft_entry__ as entry

        pkg = entry.package()
        self.np = np
        self.case = case
        self.threads = threads
        self.g = pkg.grid.Grid.build(case)
        self.pkg = pkg
        self.grids = [None] * threads
        self._each(lambda t: self.grids.__setitem__(t, O.Grid(case)))

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
        us = [self.pkg.synth.random_velocity(self.g, s) for s in seeds]

        def work(t):
            p = self.np.zeros(self.g.count)
            t0 = time.perf_counter()
            codes[t], _, _, _ = self.grids[t].project(us[t], p, DT, TOL, MAX_IT)
            times[t] = time.perf_counter() - t0

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


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import __graft_entry__ as entry

    pkg = entry.package()
    from oracle import oracle as O

    O.build()
    case = workload_case(pkg)
    threads = os.cpu_count() or 1
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
            "config": {"workload": WORKLOAD, "form": "CPU restatement of the reference (oracle), warm solves",
                       "threads": threads},
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

    def __init__(self, pkg, torch, dev, stream, form, cases, steps, rank):
        import numpy as np

        self.pkg, self.torch, self.form = pkg, torch, form
        self.ncases = cases
        case = workload_case(pkg)
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
        t = torch.tensor([total], device=flush.device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total = float(t.item())
    lat = sorted(a.elapsed_time(b) for a, b in marks)
    return total, lat, infos


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
    ncases = args.cases if args.form == "batched" else 1
    form = Form(pkg, torch, dev, stream, args.form, ncases, K + W, rank)
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
        t = torch.tensor([e2e_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())
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
                                  ("coarse_levels_cluster", 2, 20), ("vcycle_fp32", 3, 10)):
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
        pf = Form(pkg, torch, dev, stream, "plain", 1, 2 + 1, rank + 7)
        pms, plat, pinfos = timed_steps(pf, torch, stream, flush, 1, 2, dist)
        plain = {"value": round(world * 2 / (pms / 1e3), 4), "unit": UNIT, "ms_per_solve": round(pms / 2, 2),
                 "iterations_mean": round(statistics.mean(i.iterations for i in pinfos), 1), "steps": 2}
        pf.close()
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(workload_case(pkg))
    if rank == 0:
        its = [i.iterations for i in infos]
        outer = [i.work.get("refinement_steps", 0) for i in infos]
        line = {
            "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": round(total_ms / K, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.form == "plain" else "f32+f64",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "form": {"plain": "plain FP64 multigrid PCG (parity form)",
                                                       "mixed": "mixed FP32/FP64 multigrid PCG, one case",
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
    ap.add_argument("--form", default="batched", choices=["plain", "mixed", "batched"])
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
