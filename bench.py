"""Benchmark of the TCSEM_FDTD time-stepping hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--workload marine3d_256x256x160]

A "step" is one time step of the hot path (boundary pipeline, fused E/B
sweep, receiver sampling) over the workload's whole grid; the metric is
Gcell-steps/s = L*M*N*K / time / 1e9.  Default workload: the 3-D marine
survey at 256 x 256 x 160 cells (seeded synthetic model in the reference's
input formats).  With N > 1 (torchrun) every rank runs an independent replica
on its own GPU; the time is the maximum over ranks and the value the sum of
cells*steps over ranks.

--workload batch64 runs 64 generated surveys as one device batch and one at a
time (simulations per hour); --workload serve_poisson serves a seeded Poisson stream of
requests with continuous batching and one at a time (sims/hr, p50/p99).

--impl reference times the CPU implementation of the same path (the FP64 C
restatement in oracle/, all host threads) on the same workload, on a bounded
number of steps, rank 0 only.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

ALGO_BYTES_PER_CELL = {32: 52, 64: 104}  # 7 words read + 6 written per cell and step


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class Dist:
    """Barrier and max/sum reductions over ranks (gloo; no data-path collective)."""

    def __init__(self):
        self.rank, self.world, self.local = dist_env()
        self.pg = None
        if self.world > 1:
            import torch.distributed as td

            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def reduce(self, v, op):
        if self.world == 1:
            return v
        import torch

        t = torch.tensor([float(v)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX if op == "max" else self.td.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu, self.rows, self.proc = gpu, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                mx = float(r[1])
                for n, v in zip(names, r[4:8]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        j = json.load(open(p))
        return float(j["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(workload):
    """DRAM bytes per fused-sweep launch from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", f"fused_sweep_{workload}.json")
    if os.path.exists(p):
        try:
            return json.load(open(p)).get("dram_bytes_per_launch")
        except Exception:
            return None
    return None


def make_inputs(workload, rank):
    from tcsem_fdtd_gb300 import inputs

    d = tempfile.mkdtemp(prefix=f"tcsem_bench_{workload}_r{rank}_")
    inputs.write_case(inputs.case(workload), d)
    return d


def cpu_reference(args, d, cells):
    """The oracle (FP64 C, OpenMP) on a bounded number of steps of the same workload."""
    from oracle.oracle import Oracle, num_threads

    orc = Oracle(d)
    t0 = time.perf_counter()
    orc.run(0, max_steps=1)  # first touch of every array, and a per-step estimate
    per = time.perf_counter() - t0
    n = int(min(2000, max(2, 15.0 / max(per, 1e-6))))  # about 15 s of CPU work
    t0 = time.perf_counter()
    _, ran = orc.run(0, max_steps=n)
    dt = time.perf_counter() - t0
    out = {"value": cells * ran / dt / 1e9, "unit": "Gcell-steps/s", "cores": num_threads(), "kind": "port",
           "sample": f"{ran} time steps of the {args.workload} workload from a zero state (FP64 C restatement, "
                     f"{num_threads()} OpenMP threads), {dt:.2f} s"}
    remap = reference_cpu_remap(d)
    out["reference_remap"] = remap or {
        "unavailable": "the reference's CPU spline remap (SplineGridConvIR2R_cpu.cpp) is built from the reference's "
                       "sources by oracle/build_ref.py, and this host has neither the sources nor a binary built for it"}
    return out


def reference_cpu_remap(d, reps=20):
    """The reference's own CPU spline remap (SplineGridConvIR2R_cpu.cpp, built from its tree into
    oracle/_ref/ref_cpu_remap where the tree is present) timed on this host's cores; None where
    the binary is absent (it is built for the host it was compiled on)."""
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_cpu_remap")
    if not os.access(exe, os.X_OK):
        return None
    try:
        r = subprocess.run([exe, d, str(reps)], capture_output=True, text=True, timeout=120)
        l1, m1, thr, n, sec, _ = r.stdout.split()
    except Exception:
        return None
    return {"ms_per_call": float(sec) * 1e3, "plane": [int(l1), int(m1)], "cores": int(thr), "kind": "reference",
            "sample": f"{n} calls of SplineGridConvIR2R_cpu on a seeded top plane of the workload"}


def run_reference_arm(args, dist):
    if dist.rank != 0:
        return 0
    d = make_inputs(args.workload, 0)
    from tcsem_fdtd_gb300 import inputs

    c = inputs.case(args.workload)
    g = inputs.grid_axes(c)
    cells = g["L"] * g["M"] * g["N"]
    from oracle.oracle import Oracle, num_threads

    orc = Oracle(d)
    # bounded sample: W warm-up steps then up to K steps, capped at about a minute of CPU time
    t0 = time.perf_counter()
    orc.run(0, max_steps=max(1, min(args.warmup, 3)))
    per = (time.perf_counter() - t0) / max(1, min(args.warmup, 3))
    k = max(1, min(args.steps, int(60.0 / max(per, 1e-6))))
    t0 = time.perf_counter()
    _, ran = orc.run(0, max_steps=k)
    dt = time.perf_counter() - t0
    v = cells * ran / dt / 1e9
    line = {"metric": "Gcell-steps/s", "value": v, "unit": "Gcell-steps/s", "n_gpus": dist.world, "steps": ran,
            "warmup": min(args.warmup, 3), "ms_per_step": dt * 1e3 / ran, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": args.workload, "grid": [g["L"], g["M"], g["N"]], "cells": cells,
                       "plane": [orc.L1, orc.M1], "receivers": orc.NRx, "parallelism": "host cores",
                       "timed": f"{ran} time steps from a zero state on the host cores"},
            "cpu_baseline": {"value": v, "unit": "Gcell-steps/s", "cores": num_threads(), "kind": "port",
                             "sample": f"{ran} time steps from a zero state, FP64 C restatement of the reference "
                                       f"path (oracle/tcsem_oracle.c), {num_threads()} OpenMP threads"},
            "e2e": {"value": v, "unit": "Gcell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_batch_workloads(args, dist):
    """batch64: generated surveys advanced as one device batch vs one at a time (sims/hr).
    serve_poisson: a seeded Poisson stream of requests served with continuous batching (sims/hr, p50/p99)."""
    from tcsem_fdtd_gb300 import Batch, Simulation, build, inputs
    from tcsem_fdtd_gb300 import serve as sv

    build.build()
    if args.workload == "serve_poisson":
        reqs = sv.make_stream(args.surveys, args.rate, 5 + dist.rank, tn=(1.0, 10.0))
        srv = sv.Server(budget=64 << 30, block=64)
        try:
            batched = sv.summary(reqs, sv.serve(reqs, srv))
        finally:
            srv.close()
        plain_reqs = [sv.Request(r.rid, r.directory, r.arrival) for r in reqs]
        plain = sv.summary(plain_reqs, sv.run_plain(plain_reqs))
        line = {"metric": "sims/hr", "value": dist.reduce(batched["sims_per_hour"], "sum"), "unit": "sims/hr",
                "n_gpus": dist.world, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32", "data": "synthetic", "impl": "gb300",
                "config": {"workload": "serve_poisson", "requests": args.surveys, "rate_per_s": args.rate,
                           "sizes": "64x64x48 .. 256x256x160", "windows_s": [1.0, 10.0], "budget_gb": 64},
                "batched": batched, "plain": plain, "vs_plain": batched["sims_per_hour"] / plain["sims_per_hour"]}
        if dist.rank == 0:
            print(json.dumps(line), flush=True)
        return 0
    root = tempfile.mkdtemp(prefix="tcsem_bench_batch64_")
    dirs = []
    for q in range(args.surveys):
        d = os.path.join(root, f"s{q:03d}")
        inputs.write_case(inputs.batch_case(1000 * dist.rank + q), d)
        dirs.append(d)
    cells_steps = 0
    t0 = time.perf_counter()
    for d in dirs:  # one at a time: open, all steps, traces
        with Simulation(d, precision=args.precision, device=dist.local) as sim:
            sim.run(0)
            i = sim.info
            cells_steps += i["L"] * i["M"] * i["N"] * i["nsteps"]
    tp = time.perf_counter() - t0
    dist.barrier()
    t0 = time.perf_counter()
    with Batch(precision=args.precision, device=dist.local) as b:
        slots = [b.add(d) for d in dirs]
        while b.stats()["running"]:
            b.advance(256)
        b.poll()
        for s in slots:
            b.traces(s)
    tb = time.perf_counter() - t0
    tb_max = dist.reduce(tb, "max")
    n_all = dist.reduce(len(dirs), "sum")
    line = {"metric": "sims/hr", "value": 3600.0 * n_all / tb_max, "unit": "sims/hr", "n_gpus": dist.world,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if args.precision == 32 else "f64", "data": "synthetic", "impl": "gb300",
            "config": {"workload": "batch64", "surveys": len(dirs), "grids": "96..192 x 96..192 x 96..128",
                       "window_s": 1.0, "what": "tcsem_batch_add of every survey, all steps, traces to host"},
            "batched_s": tb, "plain_s": tp, "plain_sims_per_hour": 3600.0 * len(dirs) / tp,
            "vs_plain": tp / tb,
            "Gcell_steps_per_s": {"batched": cells_steps / tb / 1e9, "plain": cells_steps / tp / 1e9}}
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2048)
    ap.add_argument("--warmup", type=int, default=64)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="marine3d_256x256x160")
    ap.add_argument("--precision", type=int, default=32, choices=[32, 64])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-forms", action="store_true", help="leave out the batched and served sub-records")
    ap.add_argument("--surveys", type=int, default=64, help="batch64: surveys in the batch; serve_poisson: requests")
    ap.add_argument("--rate", type=float, default=8.0, help="serve_poisson: mean request arrivals per second")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    dist = Dist()
    try:
        if args.impl == "reference":
            return run_reference_arm(args, dist)
        if args.workload in ("batch64", "serve_poisson"):
            return run_batch_workloads(args, dist)
        return run_gb300(args, dist)
    finally:
        dist.close()


def timed_steps(d, precision, device, warmup, steps):
    """Device time of `steps` steps of the production loop: the handle captures blocks of
    `steps` steps (64 for longer runs) as one CUDA graph, so the timed region is graph
    replays; after `warmup` steps and one untimed replay (the graph's first launch uploads it)."""
    from tcsem_fdtd_gb300 import Simulation

    gsteps = steps - steps % 2 if steps < 64 else 64
    sim = Simulation(d, precision=precision, device=device, graph_steps=max(2, gsteps))
    sim.begin(0)
    sim.advance(warmup)
    sim.advance(steps)  # untimed replay
    sim.synchronize()
    return sim, gsteps


def batched_record(precision, device, surveys=16):
    """A compact batched-form record: `surveys` generated surveys of the batched workload
    (96..192 x 96..192 x 96..128 cells, 1 s window) as one device batch against the same
    surveys run one at a time, end to end (setup, all steps, traces to the host)."""
    from tcsem_fdtd_gb300 import Batch, Simulation, inputs

    root = tempfile.mkdtemp(prefix="tcsem_bench_batch_")
    dirs = []
    for q in range(surveys):
        dd = os.path.join(root, f"s{q:03d}")
        inputs.write_case(inputs.batch_case(q), dd)
        dirs.append(dd)
    cells_steps = 0
    t0 = time.perf_counter()
    for dd in dirs:
        with Simulation(dd, precision=precision, device=device) as sim:
            sim.run(0)
            i = sim.info
            cells_steps += i["L"] * i["M"] * i["N"] * i["nsteps"]
    tp = time.perf_counter() - t0
    t0 = time.perf_counter()
    with Batch(precision=precision, device=device) as b:
        slots = [b.add(dd) for dd in dirs]
        while b.stats()["running"]:
            b.advance(256)
        b.poll()
        for sl in slots:
            b.traces(sl)
    tb = time.perf_counter() - t0
    return {"surveys": surveys, "grids": "96..192 x 96..192 x 96..128", "window_s": 1.0,
            "sims_per_hour": 3600.0 * surveys / tb, "plain_sims_per_hour": 3600.0 * surveys / tp,
            "vs_plain": tp / tb, "batched_s": tb, "plain_s": tp,
            "Gcell_steps_per_s": {"batched": cells_steps / tb / 1e9, "plain": cells_steps / tp / 1e9}}


def served_record(precision, device, requests=24, rate=8.0):
    """A compact served-form record: a seeded Poisson stream of `requests` survey requests
    (64x64x48 .. 256x256x160 cells, 1 s or 10 s windows) at `rate` per second, served with
    continuous batching and one at a time (sims/hr, p50/p99 latency)."""
    from tcsem_fdtd_gb300 import serve as sv

    reqs = sv.make_stream(requests, rate, 5, tn=(1.0, 10.0))
    srv = sv.Server(precision=precision, device=device, budget=64 << 30, block=64)
    try:
        batched = sv.summary(reqs, sv.serve(reqs, srv))
    finally:
        srv.close()
    plain_reqs = [sv.Request(r.rid, r.directory, r.arrival) for r in reqs]
    plain = sv.summary(plain_reqs, sv.run_plain(plain_reqs, precision=precision, device=device))
    keys = ("sims_per_hour", "p50_latency_s", "p99_latency_s", "wall_s")
    return {"requests": requests, "rate_per_s": rate, "sizes": "64x64x48 .. 256x256x160", "windows_s": [1.0, 10.0],
            "batched": {k: batched[k] for k in keys}, "plain": {k: plain[k] for k in keys},
            "vs_plain": batched["sims_per_hour"] / plain["sims_per_hour"]}


def run_gb300(args, dist):
    from tcsem_fdtd_gb300 import Simulation, build, inputs

    build.build()
    d = make_inputs(args.workload, dist.rank)
    c = inputs.case(args.workload)
    g = inputs.grid_axes(c)
    cells = g["L"] * g["M"] * g["N"]
    nsteps_total = inputs.steps_estimate(c)
    K = max(2, min(args.steps, (nsteps_total - args.warmup) // 2 - 1))
    sim, gsteps = timed_steps(d, args.precision, dist.local, args.warmup, K)
    dist.barrier()
    with ClockSampler(dist.local) as clk:
        ms = sim.timed_advance(K)
    dist.barrier()
    ms_max = dist.reduce(ms, "max")
    work = dist.reduce(cells * K, "sum")
    value = work / (ms_max * 1e-3) / 1e9
    launches = K * sim.info["launches_per_step"] + math.ceil(K / gsteps)
    # per-kernel timings on the same stream (events around standalone launches)
    _, ms_sweep, ms_bnd = sim.time_steps(0, 64)
    sim.close()
    algo = ALGO_BYTES_PER_CELL[args.precision] * cells
    peak, peak_kind = measured_peak()
    achieved = algo / (ms_sweep * 1e-3) / 1e9
    # the same steps in the FP64 build (the reference's own precision)
    other = 64 if args.precision == 32 else 32
    sim2, _ = timed_steps(d, other, dist.local, args.warmup, K)
    ms2 = dist.reduce(sim2.timed_advance(K), "max")
    _, ms_sweep2, _ = sim2.time_steps(0, 64)
    sim2.close()
    other_rec = {"value": dist.reduce(cells * K, "sum") / (ms2 * 1e-3) / 1e9, "unit": "Gcell-steps/s",
                 "ms_per_step": ms2 / K, "sweep_ms_per_launch": ms_sweep2,
                 "sweep_frac": ALGO_BYTES_PER_CELL[other] * cells / (ms_sweep2 * 1e-3) / 1e9 / peak}
    # end to end through the C ABI with host buffers: tcsem_open of the model and survey held in
    # host memory (copied to the device inside), all steps, traces copied back to the host
    model, survey = inputs.memory_case(c)
    dist.barrier()
    t0 = time.perf_counter()
    with Simulation(precision=args.precision, device=dist.local, model=model, survey=survey) as s2:
        tr = s2.run(0)
        info2 = s2.info
    e2e_s = time.perf_counter() - t0
    e2e_s = dist.reduce(e2e_s, "max")
    e2e_val = dist.reduce(cells * info2["nsteps"], "sum") / e2e_s / 1e9
    line = {
        "metric": "Gcell-steps/s", "value": value, "unit": "Gcell-steps/s", "n_gpus": dist.world, "steps": K,
        "warmup": args.warmup, "ms_per_step": ms_max / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if args.precision == 32 else "f64", "data": "synthetic",
        "config": {"workload": args.workload, "grid": [g["L"], g["M"], g["N"]], "cells": cells,
                   "plane": [info2["L1"], info2["M1"]], "receivers": info2["NRx"],
                   "steps_per_run": info2["nsteps"], "parallelism": f"replicas{dist.world}",
                   "timed": "%d steps as replays of a captured %d-step CUDA graph" % (K, gsteps),
                   "l2": "working set 13 x %.0f MB volume arrays > 129 MB L2, no flush needed"
                         % (cells * 4 * 1.13 / 1e6)},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": "k_fused_sweep", "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": profiled_traffic(args.workload), "ms_per_launch": ms_sweep,
                     "algo_bytes_per_launch": algo, "boundary_ms_per_step": ms_bnd},
        "e2e": {"value": e2e_val, "unit": "Gcell-steps/s",
                "h2d_bytes_per_step": info2["uploaded_bytes"] / info2["nsteps"],
                "d2h_bytes_per_step": tr.nbytes / info2["nsteps"],
                "what": "tcsem_open of host buffers (conductivity, grid and survey; setup and uploads) + "
                        "tcsem_run of all %d steps + traces to the host" % info2["nsteps"], "seconds": e2e_s},
        "clocks": clk.summary(),
        ("fp64" if other == 64 else "fp32"): other_rec,
    }
    if not args.no_forms:
        line["batched"] = batched_record(args.precision, dist.local)
        line["served"] = served_record(args.precision, dist.local)
    if dist.rank == 0 and not args.no_cpu_baseline:
        try:
            line["cpu_baseline"] = cpu_reference(args, d, cells)
        except Exception as e:  # the baseline is reported, never required
            line["cpu_baseline"] = {"value": None, "error": str(e)}
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
