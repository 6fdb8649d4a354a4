"""Serving SAMPO simulations with continuous batching on one GPU.

Requests (one simulation each: initial eggs, seed, weather, horizon in days)
arrive over time. The server keeps every admitted request's pool resident in
HBM as one replicate of a ``batch.Batch`` and steps all of them together one
simulated day (24 hourly steps, one CUDA graph) at a time. Between days it
retires the requests that reached their horizon (their stats rows, age
histogram and status are read back), grows the pools that need it and admits
waiting ones, first fit in arrival order, while the device bytes of the
resident requests stay within the HBM budget and a slot is free. A request
is admitted with a pool of twice its initial size (plus 65,536 slots) and
grows with it: a pool whose end passes half its capacity is moved into one
three times its end (sampo_batch_grow, slot indices kept), and a replicate
whose next layout does not fit pauses at that step until it has been grown
(the step then runs again). Residents' growth comes before admissions; when
every resident is paused and none fits the budget, the smallest growth is
made over the budget. A request's result is bit-identical to the same
simulation run alone (``plain_result``).

The reference has no server: it runs one simulation per process
(src/abms.c:557-686)."""
from __future__ import annotations

import collections
import time
from dataclasses import dataclass

import numpy as np

from .batch import Batch, ReplicateSpec
from ._lib import RandState
from .sim import Simulation, rand_state, seed_stream


@dataclass
class Request:
    rid: int
    spec: ReplicateSpec
    arrival: float                    # seconds after the stream starts


@dataclass
class Result:
    rid: int
    arrival: float
    admitted: float = 0.0
    completed: float = 0.0
    rows: np.ndarray | None = None    # stats rows of steps 0..horizon (row k = start of step k)
    histogram: np.ndarray | None = None
    status: int = 0                   # device error/warning bits (0 = clean)

    @property
    def latency(self) -> float:
        return self.completed - self.arrival


def request_stream(n: int, rate: float, seed: int, size_range=(1e2, 5e6), days_range=(30, 365),
                   growth: float = 2.0, slack: int = 65536) -> list[Request]:
    """Poisson arrivals at `rate` per second (all at time 0 for rate 0);
    initial sizes log-uniform in size_range; horizons uniform integers in
    days_range; each with its own seed and weather (mean temperature U[20,30]
    C, amplitude U[2,8] C, noise sd 0.5, rain mean U[2,8] mm). capacity (the
    pool a request is admitted with) = growth x initial + slack slots."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n)) if rate > 0 else np.zeros(n)
    lo, hi = np.log(size_range[0]), np.log(size_range[1])
    out = []
    for i in range(n):
        initial = int(round(float(np.exp(rng.uniform(lo, hi)))))
        days = int(rng.integers(days_range[0], days_range[1] + 1))
        spec = ReplicateSpec(initial=initial, seed=int(rng.integers(1, 2**31 - 1)),
                             mean_t=float(rng.uniform(20.0, 30.0)), amplitude=float(rng.uniform(2.0, 8.0)),
                             rain_mean=float(rng.uniform(2.0, 8.0)), days=days,
                             capacity=int(growth * initial) + slack)
        out.append(Request(i, spec, float(t[i])))
    return out


@dataclass
class _Prepared:
    T: np.ndarray
    env: np.ndarray
    init: np.ndarray
    stream: RandState  # srand(seed) after the initial draws; the device draws the rest


CAPACITY_BIT = 0x1       # SAMPO_DEV_ERR_CAPACITY: paused until its pool grows
GROW_AT = 2              # grow a running pool once its end passes capacity / GROW_AT
GROW_TO = 3              # ... into GROW_TO x its end (+ 65536 slots): room for a day of the fastest growth seen (2.75x)


class Server:
    def __init__(self, budget_bytes: int, max_replicates: int = 1024, max_days: int = 365, device: int = 0,
                 grow_at: int = GROW_AT, grow_to: int = GROW_TO):
        """grow_at = 0: pools grow only when their replicate pauses for capacity."""
        self.grow_at, self.grow_to = grow_at, grow_to
        self.ring = max_days * 24 + 1  # all of a request's inputs and rows stay on the device
        self.batch = Batch(max_replicates, self.ring, device)
        self.budget = int(budget_bytes)
        self.used = 0
        self.max_replicates = max_replicates
        self.resident: dict[int, tuple[Request, Result, int]] = {}  # slot -> (request, result, bytes)
        self.days_run = 0
        self.peak_bytes = 0
        self.peak_resident = 0
        self.grows = 0              # pools moved into larger ones
        self.pauses = 0             # growth after a replicate paused for capacity
        self.over_budget = 0        # growths made over the budget to keep the batch moving
        self.held = False           # a paused resident waits for memory: no admissions
        self.held_days = 0

    def close(self):
        self.batch.close()

    def bytes_for(self, spec: ReplicateSpec) -> int:
        return Batch.replicate_bytes(spec.capacity, self.ring)

    @staticmethod
    def _prepare(spec: ReplicateSpec) -> _Prepared:
        T, env = spec.inputs()
        init, stream = rand_state(spec.seed)
        return _Prepared(T, env, init, stream)

    def _grow(self):
        """Grow paused pools (first) and pools nearing their capacity, within
        the budget; sets `held` when a paused one does not fit."""
        st = self.batch.states()
        want = []
        for slot, (req, res, nbytes) in self.resident.items():
            o = st[slot]
            if o["step"] >= req.spec.steps:
                continue
            paused = bool(o["status"] & CAPACITY_BIT) and not o["active"]
            if paused or (self.grow_at and int(o["end"]) * self.grow_at > int(o["capacity"])):
                cap = self.grow_to * int(o["end"]) + 65536
                want.append((not paused, Batch.replicate_bytes(cap, self.ring) - nbytes, slot, cap))
        want.sort()  # paused first, the smallest growth first
        self.held = False
        # nothing runs: the smallest paused growth goes ahead even over the budget
        stalled = bool(want) and not any(st[k]["active"] for k in self.resident)
        for i, (ahead, extra, slot, cap) in enumerate(want):
            if self.used + extra > self.budget and not (stalled and i == 0):
                if not ahead:
                    self.held = True
                continue
            if self.used + extra > self.budget:
                self.over_budget += 1
            self.batch.grow(slot, cap)
            req, res, nbytes = self.resident[slot]
            self.resident[slot] = (req, res, nbytes + extra)
            self.used += extra
            self.grows += 1
            self.pauses += 0 if ahead else 1
            self.peak_bytes = max(self.peak_bytes, self.used)

    def _admit(self, req: Request, prep: _Prepared, res: Result, now: float):
        s = req.spec
        b = self.batch
        slot = b.add(s.capacity, s.cc, stop_step=s.steps)
        b.set_inputs(slot, prep.T, prep.env)
        b.init_population(slot, s.initial, prep.init, age_days_max=s.age_days_max, age_seed=s.seed)
        b.seed_stream(slot, prep.stream)
        nbytes = self.bytes_for(s)
        self.used += nbytes
        res.admitted = now
        self.resident[slot] = (req, res, nbytes)
        self.peak_bytes = max(self.peak_bytes, self.used)
        self.peak_resident = max(self.peak_resident, len(self.resident))

    def _retire(self, now: float, done: list[Result]):
        b = self.batch
        st = b.states()
        for slot in list(self.resident):
            req, res, nbytes = self.resident[slot]
            step, active, bits = int(st[slot]["step"]), bool(st[slot]["active"]), int(st[slot]["status"])
            if step < req.spec.steps and not bits & 0xFF & ~CAPACITY_BIT:
                continue  # running, or paused until its pool grows (errors retire the request early)
            res.rows = b.rows(slot, 0, step + 1)
            res.histogram = b.histogram(slot)
            res.status = bits
            res.completed = now
            b.remove(slot)
            self.used -= nbytes
            del self.resident[slot]
            done.append(res)

    def serve(self, requests: list[Request], clock=time.perf_counter) -> list[Result]:
        """Runs the stream in real time: request i becomes visible at
        requests[i].arrival seconds after the call starts."""
        pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        waiting: list[tuple[Request, Result]] = []
        prepared: dict[int, _Prepared] = {}
        done: list[Result] = []
        for r in requests:
            if self.bytes_for(r.spec) > self.budget:
                raise ValueError(f"request {r.rid} needs more than the whole HBM budget")
        t0 = clock()
        while pending or waiting or self.resident:
            now = clock() - t0
            while pending and pending[0].arrival <= now:
                r = pending.popleft()
                waiting.append((r, Result(r.rid, r.arrival)))
            # admission: first fit in arrival order, unless a paused resident waits for memory
            still = []
            for r, res in waiting:
                need = self.bytes_for(r.spec)
                if not self.held and len(self.resident) < self.max_replicates and self.used + need <= self.budget:
                    prep = prepared.pop(r.rid, None) or self._prepare(r.spec)
                    self._admit(r, prep, res, clock() - t0)
                else:
                    still.append((r, res))
            waiting = still
            if not self.resident:
                if pending:  # idle until the next arrival
                    time.sleep(max(0.0, pending[0].arrival - (clock() - t0)))
                continue
            self.batch.run(24, wait=False)
            # host work for the next admissions overlaps the day on the GPU
            for r, _ in waiting[:8]:
                if r.rid not in prepared:
                    prepared[r.rid] = self._prepare(r.spec)
            self.batch.sync()
            self.days_run += 1
            self._retire(clock() - t0, done)
            self._grow()
            self.held_days += int(self.held)
        return sorted(done, key=lambda r: r.rid)


def plain_capacity(spec: ReplicateSpec) -> int:
    """The fixed pool of the plain path: 96 x initial + 65536 slots (the
    largest growth over a year seen in these workloads is about 53x)."""
    return 96 * spec.initial + 65536


def plain_result(spec: ReplicateSpec, device: int = 0) -> tuple[np.ndarray, np.ndarray, int]:
    """The same simulation alone through the plain path, in a pool of
    plain_capacity(spec): (rows of steps 0..horizon, age histogram, status bits)."""
    steps = spec.steps
    T, env = spec.inputs()
    init, seeds = seed_stream(spec.seed, steps)
    with Simulation(capacity=plain_capacity(spec), carrying_capacity=spec.cc, max_steps=steps + 1, device=device) as sim:
        sim.set_inputs(T, env)
        sim.set_seeds(0, seeds)
        sim.init_population(spec.initial, init, age_days_max=spec.age_days_max, age_seed=spec.seed)
        status = 0
        try:
            rows = sim.run(steps)
            rows = np.concatenate([rows, [sim.current_row()]])
        except Exception:
            rows = None
        status = sim.device_status()
        hist = sim.histogram() if rows is not None else None
        return rows, hist, status


def one_at_a_time(requests: list[Request], device: int = 0, clock=time.perf_counter):
    """Serves the stream with the plain path, one request at a time in
    arrival order: each request's service time is measured by running it
    alone; completion = max(arrival, previous completion) + service."""
    out = []
    prev = 0.0
    for r in sorted(requests, key=lambda r: r.arrival):
        t0 = clock()
        rows, hist, status = plain_result(r.spec, device)
        service = clock() - t0
        start = max(r.arrival, prev)
        prev = start + service
        out.append(dict(rid=r.rid, arrival=r.arrival, completed=prev, service=service, rows=rows, hist=hist,
                        status=status))
    return out


def latency_summary(latencies) -> dict:
    a = np.asarray(latencies, dtype=np.float64)
    return {"p50": float(np.percentile(a, 50)), "p95": float(np.percentile(a, 95)), "p99": float(np.percentile(a, 99)),
            "mean": float(a.mean()), "max": float(a.max())}
