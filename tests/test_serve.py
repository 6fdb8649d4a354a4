"""Serving with continuous batching (sampo_gb300.serve): requests that arrive
while others run are admitted as memory and slots free up, share the batch's
day steps, and each result - stats rows of every step, age histogram and
status - is the same as the request run alone through the plain path."""
import numpy as np
import pytest

from sampo_gb300.serve import latency_summary, request_stream


def test_request_stream_follows_its_distributions():
    reqs = request_stream(2000, rate=100.0, seed=3, size_range=(1e2, 5e6), days_range=(30, 365))
    t = np.array([r.arrival for r in reqs])
    assert np.all(np.diff(t) >= 0)
    assert 0.8 < 1.0 / np.diff(t).mean() / 100.0 < 1.2          # Poisson rate
    sizes = np.log(np.array([r.spec.initial for r in reqs], dtype=np.float64))
    assert sizes.min() >= np.log(1e2) - 0.01 and sizes.max() <= np.log(5e6) + 0.01
    assert abs(sizes.mean() - 0.5 * (np.log(1e2) + np.log(5e6))) < 0.3   # log-uniform
    days = np.array([r.spec.days for r in reqs])
    assert days.min() >= 30 and days.max() <= 365
    assert len({r.spec.seed for r in reqs}) > 1990
    s = latency_summary([1.0, 2.0, 3.0, 4.0])
    assert s["p50"] == 2.5 and s["max"] == 4.0


@pytest.mark.gpu
def test_served_results_equal_solo_runs(gpu_ready):
    from sampo_gb300.serve import Server, plain_result
    reqs = request_stream(10, rate=400.0, seed=5, size_range=(100, 5000), days_range=(2, 5), growth=64.0)
    probe = Server(budget_bytes=1 << 40, max_days=5)
    biggest = max(probe.bytes_for(r.spec) for r in reqs)
    probe.close()
    budget = int(2.2 * biggest)  # room for about two requests: the rest must queue
    srv = Server(budget_bytes=budget, max_replicates=4, max_days=5)
    results = srv.serve(reqs)
    srv.close()
    assert len(results) == len(reqs)
    assert srv.peak_bytes <= budget and srv.peak_resident <= 4
    assert srv.peak_resident >= 2, "requests must overlap on the device"
    assert any(r.admitted > r.arrival for r in results), "some requests must wait for memory"
    by_id = {r.rid: r for r in reqs}
    for res in results:
        rows, hist, status = plain_result(by_id[res.rid].spec)
        assert res.rows.tobytes() == rows.tobytes(), f"request {res.rid}: rows differ from its solo run"
        assert np.array_equal(res.histogram, hist), f"request {res.rid}: histogram differs"
        assert res.status == status
        assert res.completed >= res.admitted >= res.arrival


@pytest.mark.gpu
@pytest.mark.parametrize("grow_at", [0, 2])
def test_served_pools_grow_and_match_solo_runs(gpu_ready, grow_at):
    """Requests admitted with pools far smaller than they grow to: the server
    moves them into larger ones, after a pause for capacity (grow_at = 0) or
    ahead of need, and every result still equals the request run alone in a
    fixed roomy pool."""
    from sampo_gb300.batch import ReplicateSpec
    from sampo_gb300.serve import Request, Server, plain_result
    # seed 21 outgrows 4096 slots at step 310 and reaches 18714 (oracle)
    specs = [ReplicateSpec(initial=2000, seed=21, mean_t=29.0, amplitude=2.0, rain_mean=3.0, days=16, capacity=4096),
             ReplicateSpec(initial=2000, seed=21, mean_t=29.0, amplitude=2.0, rain_mean=3.0, days=15, capacity=6000),
             ReplicateSpec(initial=300, seed=5, mean_t=26.0, amplitude=4.0, rain_mean=3.0, days=6, capacity=1024)]
    reqs = [Request(i, s, 0.0) for i, s in enumerate(specs)]
    srv = Server(budget_bytes=1 << 40, max_replicates=4, max_days=16, grow_at=grow_at)
    results = srv.serve(reqs)
    srv.close()
    assert srv.grows >= 2
    if grow_at == 0:
        assert srv.pauses >= 2
    for res in results:
        rows, hist, status = plain_result(specs[res.rid])
        assert res.rows.tobytes() == rows.tobytes(), f"request {res.rid}: rows differ from its solo run"
        assert np.array_equal(res.histogram, hist)
        assert res.status == status == 0


class _FakeBatch:
    """The two calls the growth policy makes, on fixed slot states."""

    def __init__(self, states):
        self.st = states
        self.grown = []

    def states(self):
        return self.st

    def grow(self, slot, capacity):
        self.grown.append((slot, capacity))
        self.st[slot]["capacity"] = capacity


def _policy_server(states, steps, budget, used_extra=0, grow_at=2, grow_to=3):
    """A Server whose batch is a fake: only the growth policy (_grow) runs."""
    from types import SimpleNamespace
    from sampo_gb300.batch import Batch
    from sampo_gb300.serve import Server
    srv = Server.__new__(Server)
    srv.grow_at, srv.grow_to, srv.ring = grow_at, grow_to, 25
    srv.batch = _FakeBatch(states)
    srv.resident = {}
    srv.used = used_extra
    for slot, st in states.items():
        nbytes = Batch.replicate_bytes(st["capacity"], srv.ring)
        srv.resident[slot] = (SimpleNamespace(spec=SimpleNamespace(steps=steps[slot])), None, nbytes)
        srv.used += nbytes
    srv.budget = budget
    srv.grows = srv.pauses = srv.over_budget = srv.peak_bytes = 0
    srv.held = False
    return srv


def _state(step, active, status, end, capacity):
    return {"step": step, "active": active, "status": status, "end": end, "capacity": capacity}


def test_growth_policy_without_gpu(sampo_lib):
    """Which pools the server grows between days, and when it holds
    admissions (host logic only: a fake batch stands for the GPU)."""
    from sampo_gb300.batch import Batch
    from sampo_gb300.serve import CAPACITY_BIT
    ring = 25
    cost = lambda cap: Batch.replicate_bytes(cap, ring)
    # a paused replicate, a running one past half its capacity, one below it,
    # one finished: the first two grow, paused first, to 3 x end + 65536
    states = {0: _state(40, 0, CAPACITY_BIT, 90000, 100000), 1: _state(40, 1, 0, 60000, 100000),
              2: _state(40, 1, 0, 40000, 100000), 3: _state(48, 0, 0, 99000, 100000)}
    srv = _policy_server(states, {0: 48, 1: 48, 2: 48, 3: 48}, budget=1 << 40)
    srv._grow()
    assert srv.batch.grown == [(0, 3 * 90000 + 65536), (1, 3 * 60000 + 65536)]
    assert (srv.grows, srv.pauses, srv.over_budget, srv.held) == (2, 1, 0, False)
    # grow_at = 0: only paused pools grow
    states = {0: _state(40, 0, CAPACITY_BIT, 90000, 100000), 1: _state(40, 1, 0, 60000, 100000)}
    srv = _policy_server(states, {0: 48, 1: 48}, budget=1 << 40, grow_at=0)
    srv._grow()
    assert srv.batch.grown == [(0, 3 * 90000 + 65536)]
    # a paused pool that does not fit while another runs: admissions are held
    states = {0: _state(40, 0, CAPACITY_BIT, 90000, 100000), 1: _state(40, 1, 0, 10000, 100000)}
    base = 2 * cost(100000)
    srv = _policy_server(states, {0: 48, 1: 48}, budget=base + 1000)
    srv._grow()
    assert srv.batch.grown == [] and srv.held
    # nothing runs: the smallest paused growth goes ahead over the budget
    states = {0: _state(40, 0, CAPACITY_BIT, 90000, 100000), 1: _state(40, 0, CAPACITY_BIT, 50000, 100000)}
    srv = _policy_server(states, {0: 48, 1: 48}, budget=base + 1000)
    srv._grow()
    assert srv.batch.grown == [(1, 3 * 50000 + 65536)]
    assert srv.over_budget == 1 and srv.used == base + cost(3 * 50000 + 65536) - cost(100000)
