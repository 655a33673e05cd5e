"""Serving loop: simulation requests that arrive over time, run on one GPU with
continuous batching, and their latencies.

    python -m tcsem_fdtd_gb300.serve [--requests 48] [--rate 4.0] [--seed 5]
                                     [--budget-gb 64] [--plain] [--jsonl PATH]

A :class:`Server` owns one device batch (tcsem_batch_* of include/tcsem.h).
Each loop iteration (one graph block of the batch, `block` steps) it

1. moves the requests whose arrival time has passed into the queue,
2. enqueues one block of steps for every running request (asynchronous),
3. while the GPU runs that block, admits queued requests in arrival order
   while the batch accepts them -- a request is accepted when the estimate of
   its device footprint fits the remaining budget (the batch refuses it
   otherwise, nothing allocated), so admission is by HBM footprint and a large
   request waits until enough finished requests have left; reading its input
   files and setting up its device state overlap the running block,
4. collects finished requests (traces copied to the host, slot freed).

Requests join and leave only at block boundaries; each request's fields stay on
the device from admission to completion.  Latency = completion time - arrival
time.  :func:`run_plain` serves the same stream one request at a time with
:class:`~tcsem_fdtd_gb300.api.Simulation` for comparison.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import tempfile
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


class Request:
    def __init__(self, rid, directory, arrival, itx=0):
        self.rid, self.directory, self.arrival, self.itx = rid, directory, arrival, itx
        self.admitted = self.completed = None
        self.slot = None
        self.traces = None
        self.cells_steps = 0


class Server:
    """Continuous batching of survey requests on one GPU."""

    def __init__(self, precision=32, device=0, budget=64 << 30, block=64, zchunks=0, batch=None, persistent=False):
        """`batch`: an object with the methods of :class:`~tcsem_fdtd_gb300.api.Batch` used here
        (add, advance, poll, info, traces, remove, close); a device batch by default, with the
        persistent schedule (one launch per block) when `persistent`."""
        if batch is None:
            from .api import Batch

            batch = Batch(precision=precision, device=device, budget=budget, graph_steps=block, zchunks=zchunks,
                          persistent=persistent)
        self.batch = batch
        self.block = block
        self.queue, self.running, self.done = [], {}, []

    def submit(self, req):
        self.queue.append(req)

    def _admit(self, now):
        from .api import TcsemError

        while self.queue:
            req = self.queue[0]
            try:
                req.slot = self.batch.add(req.directory, req.itx)
            except TcsemError as e:
                if e.status == 5 and self.running:  # no room now: wait for running requests to leave
                    return
                raise
            self.queue.pop(0)
            req.admitted = now()
            info = self.batch.info(req.slot)
            req.cells_steps = info["L"] * info["M"] * info["N"] * info["nsteps"]
            self.running[req.slot] = req

    def step(self, now):
        """One loop iteration; returns the requests that finished in it."""
        if self.running:
            self.batch.advance(self.block)  # the new admissions below overlap this block
        self._admit(now)
        if not self.running:
            return []
        finished = []
        for slot in self.batch.poll():
            req = self.running.pop(slot)
            req.traces = self.batch.traces(slot)
            req.completed = now()
            self.batch.remove(slot)
            finished.append(req)
        self.done.extend(finished)
        return finished

    def close(self):
        self.batch.close()


def make_stream(n, rate, seed, size=((64, 256), (64, 256), (48, 160)), tn=(1.0, 10.0), root=None, pool=0):
    """Seeded Poisson stream of `n` survey requests (mean `rate` per second); writes their inputs.
    `pool` > 0: the requests draw their surveys (seeded) from that many distinct generated
    surveys, so a long stream does not need one input directory per request on disk; every
    request is still a simulation of its own."""
    from .inputs import batch_case, write_case

    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=n))
    arrivals -= arrivals[0]
    root = root or tempfile.mkdtemp(prefix="tcsem_serve_")
    ndirs = min(n, pool) if pool > 0 else n
    dirs = []
    for r in range(ndirs):
        d = os.path.join(root, f"req{r:04d}")
        write_case(batch_case(int(rng.integers(1 << 31)), size=size, tn=tn), d)
        dirs.append(d)
    pick = rng.integers(0, ndirs, size=n) if ndirs < n else np.arange(n)
    return [Request(r, dirs[int(pick[r])], float(arrivals[r])) for r in range(n)]


def request_record(req, mode="batched"):
    """One JSON-lines record of a finished request: its times, latency and work."""
    return {"request": req.rid, "mode": mode, "arrival_s": req.arrival, "admitted_s": req.admitted,
            "completed_s": req.completed, "latency_s": req.completed - req.arrival,
            "queued_s": req.admitted - req.arrival, "cell_steps": req.cells_steps,
            "Gcell_steps_per_s": req.cells_steps / max(req.completed - req.admitted, 1e-12) / 1e9}


def serve(reqs, server, speed=1.0, log=None):
    """Replay the arrivals in real time (scaled by `speed`); returns the wall time of the run.
    `log`: a text file that receives one JSON line per request as it finishes."""
    t0 = time.perf_counter()
    now = lambda: (time.perf_counter() - t0) * speed  # noqa: E731
    pending = sorted(reqs, key=lambda r: r.arrival)
    total = len(reqs)
    while len(server.done) < total:
        while pending and pending[0].arrival <= now():
            server.submit(pending.pop(0))
        if not server.running and not server.queue:
            if pending:  # idle until the next arrival
                time.sleep(max(0.0, (pending[0].arrival - now()) / speed))
            continue
        for req in server.step(now):
            if log is not None:
                log.write(json.dumps(request_record(req)) + "\n")
                log.flush()
    return now()


def run_plain(reqs, precision=32, device=0, speed=1.0):
    """The same stream served one request at a time, first come first served."""
    from .api import Simulation

    t0 = time.perf_counter()
    now = lambda: (time.perf_counter() - t0) * speed  # noqa: E731
    for req in sorted(reqs, key=lambda r: r.arrival):
        wait = req.arrival - now()
        if wait > 0:
            time.sleep(wait / speed)
        req.admitted = now()
        with Simulation(req.directory, precision=precision, device=device) as sim:
            req.traces = sim.run(req.itx)
            i = sim.info
            req.cells_steps = i["L"] * i["M"] * i["N"] * i["nsteps"]
        req.completed = now()
    return now()


def summary(reqs, wall):
    lat = np.array([r.completed - r.arrival for r in reqs])
    return {"requests": len(reqs), "wall_s": wall, "sims_per_hour": 3600.0 * len(reqs) / wall,
            "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
            "mean_latency_s": float(lat.mean()), "Gcell_steps_per_s": sum(r.cells_steps for r in reqs) / wall / 1e9}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--requests", type=int, default=48)
    ap.add_argument("--rate", type=float, default=4.0, help="mean arrivals per second")
    ap.add_argument("--seed", type=int, default=5)
    ap.add_argument("--budget-gb", type=float, default=64.0)
    ap.add_argument("--block", type=int, default=64)
    ap.add_argument("--tn", type=float, nargs="+", default=[1.0, 10.0])
    ap.add_argument("--plain", action="store_true", help="also serve the stream one request at a time")
    ap.add_argument("--jsonl", default=None, help="write one JSON line per finished request to this file")
    ap.add_argument("--pool", type=int, default=0, help="distinct surveys the requests draw from (0: one each)")
    ap.add_argument("--persistent", action="store_true", help="the batch's persistent schedule (one launch per block)")
    a = ap.parse_args(argv)
    from . import build

    build.build()
    reqs = make_stream(a.requests, a.rate, a.seed, tn=tuple(a.tn), pool=a.pool)
    srv = Server(budget=int(a.budget_gb * (1 << 30)), block=a.block, persistent=a.persistent)
    log = open(a.jsonl, "w") if a.jsonl else None
    try:
        out = {"batched": summary(reqs, serve(reqs, srv, log=log))}
    finally:
        srv.close()
        if log:
            log.close()
    if a.plain:
        plain = [Request(r.rid, r.directory, r.arrival) for r in reqs]
        out["plain"] = summary(plain, run_plain(plain))
    print(json.dumps(out), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
