"""The serving loop's scheduling on the CPU, without a GPU.

`Server` drives a stand-in batch with the methods of the device batch it uses:
slots advance one graph block per loop iteration, a slot whose footprint does
not fit the budget is refused with the batch's status 5 (TCSEM_ERR_NOMEM), as
tcsem_batch_add does.  Checked: every request completes once, admission is in
arrival order, the budget is never exceeded (requests wait in the queue
instead), a request that can never fit is reported, and latencies are
completion minus arrival.
"""
import numpy as np
import pytest

from tcsem_fdtd_gb300.api import TcsemError
from tcsem_fdtd_gb300.serve import Request, Server, request_record, serve, summary


class FakeBatch:
    """Slots with a footprint and a run length; `advance` moves every running slot on."""

    def __init__(self, budget, sizes, steps):
        self.budget, self.sizes, self.steps = budget, sizes, steps  # per directory
        self.slots, self.next_id, self.peak_used, self.adds = {}, 1, 0, []

    def used(self):
        return sum(s["bytes"] for s in self.slots.values())

    def add(self, d, itx=0):
        need = self.sizes[d]
        if self.used() + need > self.budget:
            raise TcsemError(5, "device budget")
        sid = self.next_id
        self.next_id += 1
        self.slots[sid] = {"dir": d, "bytes": need, "done": 0, "n": self.steps[d]}
        self.adds.append(d)
        self.peak_used = max(self.peak_used, self.used())
        return sid

    def advance(self, n):
        for s in self.slots.values():
            s["done"] = min(s["n"], s["done"] + n)

    def poll(self):
        return [sid for sid, s in self.slots.items() if s["done"] >= s["n"]]

    def info(self, sid):
        return {"L": 10, "M": 10, "N": 10, "nsteps": self.slots[sid]["n"]}

    def traces(self, sid):
        return np.full((2, 3, 4), float(sid))

    def remove(self, sid):
        del self.slots[sid]

    def close(self):
        pass


def stream(n, gap, sizes, steps):
    reqs = [Request(r, f"req{r}", r * gap) for r in range(n)]
    return reqs, {q.directory: sizes[q.rid % len(sizes)] for q in reqs}, {q.directory: steps[q.rid % len(steps)] for q in reqs}


def test_every_request_completes_in_arrival_order_within_the_budget():
    reqs, sizes, steps = stream(12, 0.002, sizes=[3, 5, 2, 4], steps=[64, 192, 128])
    fake = FakeBatch(budget=8, sizes=sizes, steps=steps)
    srv = Server(block=64, batch=fake)
    wall = serve(reqs, srv)
    assert sorted(r.rid for r in srv.done) == list(range(12))
    assert fake.adds == [f"req{r}" for r in range(12)]  # first come, first admitted
    assert fake.peak_used <= 8 and not fake.slots
    for r in reqs:
        assert r.arrival <= r.admitted <= r.completed <= wall
        assert r.traces.shape == (2, 3, 4)
    adm = [r.admitted for r in sorted(reqs, key=lambda q: q.arrival)]
    assert adm == sorted(adm)
    s = summary(reqs, wall)
    lat = sorted(r.completed - r.arrival for r in reqs)
    assert s["requests"] == 12 and s["p50_latency_s"] == pytest.approx(float(np.percentile(lat, 50)))


def test_requests_wait_in_the_queue_when_the_budget_is_full():
    reqs, sizes, steps = stream(6, 0.0, sizes=[5], steps=[256])
    fake = FakeBatch(budget=10, sizes=sizes, steps=steps)  # two at a time
    srv = Server(block=64, batch=fake)
    for r in reqs:
        srv.submit(r)
    t = [0.0]

    def now():
        t[0] += 1.0
        return t[0]

    seen = 0
    while len(srv.done) < 6:
        srv.step(now)
        seen = max(seen, len(srv.running))
        assert len(srv.running) <= 2
    assert seen == 2 and fake.peak_used == 10


def test_a_request_larger_than_the_whole_budget_is_reported():
    reqs, sizes, steps = stream(1, 0.0, sizes=[20], steps=[64])
    srv = Server(block=64, batch=FakeBatch(budget=10, sizes=sizes, steps=steps))
    srv.submit(reqs[0])
    with pytest.raises(TcsemError) as e:
        srv.step(lambda: 0.0)
    assert e.value.status == 5


def test_one_json_line_per_finished_request(tmp_path):
    import io
    import json

    reqs, sizes, steps = stream(5, 0.001, sizes=[2], steps=[64, 128])
    srv = Server(block=64, batch=FakeBatch(budget=10, sizes=sizes, steps=steps))
    log = io.StringIO()
    serve(reqs, srv, log=log)
    recs = [json.loads(x) for x in log.getvalue().splitlines()]
    assert sorted(r["request"] for r in recs) == list(range(5))
    for r in recs:
        q = reqs[r["request"]]
        assert r == json.loads(json.dumps(request_record(q)))
        assert r["latency_s"] == pytest.approx(q.completed - q.arrival) and r["queued_s"] >= 0


def test_a_request_stream_drawn_from_a_survey_pool(tmp_path):
    """make_stream with a pool: seeded Poisson arrivals from 0, one request per arrival, the
    surveys drawn from `pool` distinct generated input directories, the same stream again
    from the same seed."""
    import os

    from tcsem_fdtd_gb300.serve import make_stream

    size = ((64, 64), (64, 64), (48, 48))
    a = make_stream(12, 8.0, 3, size=size, tn=(1.0, 1.0), root=str(tmp_path / "a"), pool=3)
    b = make_stream(12, 8.0, 3, size=size, tn=(1.0, 1.0), root=str(tmp_path / "b"), pool=3)
    assert [r.rid for r in a] == list(range(12))
    t = [r.arrival for r in a]
    assert t[0] == 0.0 and all(x <= y for x, y in zip(t, t[1:]))
    assert [r.arrival for r in b] == t
    dirs = sorted({r.directory for r in a})
    assert len(dirs) <= 3 and len(os.listdir(tmp_path / "a")) == 3
    for d in dirs:
        assert {"FDTD_setup.in", "Cond.bin", "Receiver.in", "Transmitter.in"} <= set(os.listdir(d))
    # the same draw of surveys for the same seed
    assert [os.path.basename(r.directory) for r in a] == [os.path.basename(r.directory) for r in b]
