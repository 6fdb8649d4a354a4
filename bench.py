#!/usr/bin/env python
"""Throughput of SAMPO's simulated day on GB300, in agent-days per second.

A bench step is one simulated day: 24 hourly steps of the hot path (count
pass + update/scatter pass each), replayed as one CUDA graph. The default
workload is the bandwidth-roofline run: 5e7 preloaded agents uniform over
the egg / larva / pupa / adult stages (50/50 gender), a 1e8-slot pool, a
constant 28 C for 90 days, seed 3; W warm-up days, then K timed days.
agent-days = sum over hourly steps of the live agents at the step's start
/ 24.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--workload roofline|plain-large|plain-small|ensemble|served]

--workload ensemble: 512 replicates (sizes log-uniform in [1e3, 1e6] eggs, each
with its own seed and weather) stepped as one batch for W + K days against
the same replicates run one at a time through the plain path; every
replicate's rows are compared bit for bit.
--workload served: Poisson request streams (--rates) served with continuous
batching under an HBM budget against one-at-a-time plain service; reports
p50/p95/p99 latency and sims/s per rate.

--impl reference times the reference's own per-step algorithm on the host
cores (the CPU restatement in oracle/, pinned to the reference's code by the
golden traces) over the same simulated days: W untimed warm-up days, then
K timed days, with the same `config`.
Under torchrun (N > 1) every rank runs its own replicate (replicas only:
a simulation does not shard), rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

from sampo_gb300.workloads import WORKLOADS, build_workload  # noqa: E402

# algorithmic bytes per live agent read by the count pass, by state of its range
# (the fields that decide survival, the next state and eggs laid)
COUNT_BYTES = np.array([8, 12, 8, 12, 13, 12, 12, 12], dtype=np.float64)
RECORD_BYTES = 37.0   # 9 x 4-byte fields + 1 flag byte


def peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def oracle_seed_stream(seed: int, nsteps: int):
    """srand(seed) + generateSeeds draws from the oracle's glibc restatement
    (the reference arm never loads the CUDA library)."""
    import oracle
    v = oracle.glibc_rand(seed, 16 * (nsteps + 1))
    return v[:16].reshape(4, 4), v[16:].reshape(nsteps, 4, 4)


def start_pool(sim, wl, init, pool):
    if pool is not None:
        sim.load_pool(*pool)
    else:
        sim.init_population(wl["eggs"], init, 3, wl["seed"])


def live_counts(rows) -> np.ndarray:
    r = rows["ranges"].astype(np.int64)
    return (r[:, :, 1] - r[:, :, 0])


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons), "samples": len(sm)}


def traffic_from_profile():
    """dram bytes per live agent of the update/scatter kernel from the
    committed ncu summary (profiles/k_scatter_dram.json), or None."""
    p = os.path.join(REPO, "profiles", "k_scatter_dram.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        return json.load(f)


def gpu_arm(args, wl, rank, world, device):
    from sampo_gb300.sim import PinnedArray, Simulation
    days = max(wl["days"], args.warmup + args.steps)
    T, env, init, seeds, pool = build_workload(wl, days)
    if rank > 0:  # independent replicate per rank
        from sampo_gb300.sim import seed_stream
        init, seeds = seed_stream(rank_seed(wl["seed"], rank), days * 24)
    nsteps = days * 24
    sim = Simulation(capacity=wl["capacity"], carrying_capacity=wl["cc"], max_steps=nsteps + 1, device=device)
    sim.set_inputs(T, env)
    sim.set_seeds(0, seeds)

    def fresh():
        start_pool(sim, wl, init, pool)
        if args.warmup:
            sim.run(24 * args.warmup, want_rows=False)

    # the autotuner picks the step kernels' grid sizes on the first timed day's
    # state (it leaves the run unchanged); they stay for every phase below.
    # --ctas-per-sm fixes them instead (profiling runs, where timings under
    # the profiler would mislead the tuner)
    fresh()
    sim.set_small_step(None if args.small_step == "auto" else 0 if args.small_step == "off" else int(args.small_step))
    sim.set_small_step_items(args.small_items)
    if args.ctas_per_sm:
        tuned = tuple(int(x) for x in args.ctas_per_sm.split(","))
        sim.set_grids(*tuned)
    else:
        tuned = sim.autotune()
    items = sim.items_per_thread()
    # ---- value: device-resident inputs, day graphs, L2 flushed between days ----
    fresh()
    sim.flush_l2()
    rows, ms = [], 0.0
    launches0 = sim.kernel_times()[1]
    small0 = sim.small_step_info()
    sync_barrier(world)
    t0 = time.perf_counter()
    with ClockSampler(device) as clk:
        for _ in range(args.steps):
            rows.append(sim.run(24))
            ms += sim.last_run_ms()
            sim.flush_l2()
    wall = time.perf_counter() - t0
    sync_barrier(world)
    rows = np.concatenate(rows)
    live = live_counts(rows)
    agent_days = float(live.sum()) / 24.0
    # kernels the library launched in the timed region (its own count: the
    # kernel nodes of each replayed day graph plus the launches outside graphs)
    gpu_launches = sim.kernel_times()[1] - launches0
    small = sim.small_step_info()

    # ---- roofline: the same days again, each kernel between CUDA events ----
    fresh()
    sim.set_timing(True)
    rows2 = sim.run(24 * args.steps)
    times, launches = sim.kernel_times()
    sim.set_timing(False)
    live2 = live_counts(rows2)
    if not np.array_equal(live2, live):
        raise RuntimeError("timing-mode rerun diverged from the graph run")
    tot = live2.sum(axis=1).astype(np.float64)
    nxt = np.append(tot[1:], tot[-1])  # agents written = pool size at the next step's start
    scatter_bytes = RECORD_BYTES * (tot + nxt)
    count_bytes = (live2 * COUNT_BYTES).sum(axis=1)
    n_launch = len(tot)
    scatter_ms, count_ms = times[1] / n_launch, times[0] / n_launch
    # the step in timing mode minus the two passes: k_publish and the gaps between the launches
    publish_ms = (times[2] - times[0] - times[1]) / n_launch
    peak, peak_kind = peaks()
    achieved = scatter_bytes.mean() / (scatter_ms * 1e-3) / 1e9
    prof = traffic_from_profile()
    traffic = None
    if prof:
        traffic = float(prof["dram_bytes_per_live_agent"] * tot.mean())

    # ---- e2e: through the C ABI with page-locked host buffers, per day ----
    from sampo_gb300._lib import ENV_DTYPE, ROW_DTYPE
    fresh()
    hT = PinnedArray((24,), np.float32)
    hE = PinnedArray((24,), ENV_DTYPE)
    hS = PinnedArray((24, 4, 4), np.uint32)
    hR = PinnedArray((24,), ROW_DTYPE)
    lib = sim.lib
    first = 24 * args.warmup
    sync_barrier(world)
    t0 = time.perf_counter()
    e2e_live = 0
    for d in range(args.steps):
        s0 = first + 24 * d
        hT.a[:] = T[s0:s0 + 24]
        hE.a[:] = env[s0:s0 + 24]
        hS.a[:] = seeds[s0:s0 + 24]
        sim._check(lib.sampo_set_inputs(sim.h, s0, hT.p, hE.p, 24))
        sim._check(lib.sampo_set_seeds(sim.h, s0, hS.p, 24))
        sim.run_into(24, hR.p)
        r = hR.a["ranges"].astype(np.int64)
        e2e_live += int((r[:, :, 1] - r[:, :, 0]).sum())
    e2e_wall = time.perf_counter() - t0
    sync_barrier(world)
    for h in (hT, hE, hS, hR):
        h.free()
    sim.close()
    # each pass against the peak, and the whole step as the day graphs run it
    step_ms_graph = ms / (24 * args.steps)
    step_bytes = float(count_bytes.mean() + scatter_bytes.mean())

    def pass_line(nbytes, t_ms):
        gbs = nbytes / (t_ms * 1e-3) / 1e9
        return {"bytes_per_launch": nbytes, "ms_per_launch": t_ms, "gbs": gbs, "frac": gbs / peak}
    passes = {
        "k_count: decisions + in-tile scan (8-13 B read per live agent)": pass_line(float(count_bytes.mean()), count_ms),
        "k_scatter: update + cross-tile scan + compaction (37 B read + 37 B written per agent)": pass_line(float(scatter_bytes.mean()), scatter_ms),
        "hourly step in the day graphs (both passes + k_publish)": pass_line(step_bytes, step_ms_graph),
    }
    return dict(agent_days=agent_days, ms=ms, wall=wall, live=live, rows=rows, clocks=clk.summary(), passes=passes,
                gpu_launches=gpu_launches, scatter_ms=scatter_ms, count_ms=count_ms, publish_ms=publish_ms, achieved=achieved, peak=peak,
                peak_kind=peak_kind, traffic=traffic, e2e_agent_days=e2e_live / 24.0, e2e_wall=e2e_wall,
                count_gbs=count_bytes.mean() / (count_ms * 1e-3) / 1e9, days=days, tuned=tuned, items=items, small=small, small0=small0)


def cpu_reference(wl, seconds: float, first_steps: int | None = None, warmup: int = 0):
    """The oracle port on all host threads over a bounded sample (hourly
    steps from the workload's start, after `warmup` untimed steps) of about
    `seconds` of CPU work, or exactly `first_steps` timed steps."""
    from oracle import OracleSim
    days = wl["days"]
    T, env, init, seeds, pool = build_workload(wl, days, seed_fn=oracle_seed_stream)
    threads = os.cpu_count() or 1
    o = OracleSim(wl["capacity"], threads)
    if pool is not None:
        o.load_pool(*pool)
    else:
        o.init_eggs(wl["eggs"], T[0], init, 3, wl["seed"])
    for i in range(warmup):
        o.step(env[i], T[i], i % 24, seeds[i])
    live_sum, steps, t0 = 0, warmup, time.perf_counter()
    limit = warmup + first_steps if first_steps else len(T)
    while steps < limit:
        r = o.step(env[steps], T[steps], steps % 24, seeds[steps])
        rr = r["ranges"].astype(np.int64)
        live_sum += int((rr[:, 1] - rr[:, 0]).sum())
        steps += 1
        if first_steps is None and time.perf_counter() - t0 > seconds:
            break
    dt = time.perf_counter() - t0
    o.close()
    return dict(value=live_sum / 24.0 / dt, steps=steps - warmup, seconds=dt, threads=threads, agent_steps=live_sum)


# ---------------- distributed plumbing (replicas only) ----------------
_PG = None


def rank_seed(seed: int, rank: int) -> int:
    """The glibc seed of rank's replicate (rank 0 runs the workload's own seed)."""
    return seed if rank == 0 else seed * 1000 + rank


def job_rate(units: float, seconds: float) -> float:
    """Whole-job throughput of replicas: units summed over ranks / the slowest rank's time."""
    return units / seconds


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def dist_init(world):
    global _PG
    if world > 1 and _PG is None:
        import torch.distributed as dist
        dist.init_process_group(backend="gloo")
        _PG = dist
    return _PG


def sync_barrier(world):
    if world > 1:
        _PG.barrier()


def all_reduce(vals, op):
    if _PG is None:
        return vals
    import torch
    t = torch.tensor(vals, dtype=torch.float64)
    _PG.all_reduce(t, op=_PG.ReduceOp.MAX if op == "max" else _PG.ReduceOp.SUM)
    return t.tolist()


def ensemble_arm(args):
    """The 512-replicate ensemble over a window of days: batched vs one at a time."""
    from sampo_gb300.batch import Batch, ensemble_specs
    from sampo_gb300.sim import Simulation, rand_state, seed_stream
    days = args.warmup + args.steps
    n = args.replicates
    # the hottest replicates reach 12x their initial size by day 15 (oracle)
    specs = ensemble_specs(n, seed=4, days=days, growth=20.0)
    prep = []
    for s in specs:
        T, env = s.inputs()
        init, seeds = seed_stream(s.seed, s.steps)
        prep.append((T, env, init, seeds))
    ring = days * 24 + 1
    # ---- batched (each replicate draws its seeds on the device) ----
    # e2e: the whole batched run through the public API, timed on the host:
    # slots taken, every replicate's inputs for all its days up from
    # page-locked buffers, initial populations, warm-up days, grid tuning, the
    # timed days, and every replicate's stats rows back. value: the device time
    # of the timed days alone (CUDA events)
    from sampo_gb300._lib import ENV_DTYPE, ROW_DTYPE
    from sampo_gb300.sim import PinnedArray
    nsteps = 24 * days
    hT, hE = PinnedArray((nsteps,), np.float32), PinnedArray((nsteps,), ENV_DTYPE)
    hR = PinnedArray((nsteps + 1,), ROW_DTYPE)
    t_all = time.perf_counter()
    b = Batch(n, ring)
    slots = []
    for s, (T, env, init, seeds) in zip(specs, prep):
        slot = b.add(s.capacity, s.cc, stop_step=s.steps)
        hT.a[:] = T
        hE.a[:] = env
        b._check(b.lib.sampo_batch_set_inputs(b.h, slot, 0, hT.p, hE.p, nsteps))
        init, stream = rand_state(s.seed)
        b.init_population(slot, s.initial, init, age_days_max=s.age_days_max, age_seed=s.seed)
        b.seed_stream(slot, stream)
        slots.append(slot)
    b.sync()
    setup_batch = time.perf_counter() - t_all
    b.run(24 * args.warmup)
    tuned = b.autotune()
    batch_items = b.items_per_thread()
    launches0 = b.launches()
    with ClockSampler(0) as clk:
        b.run(24 * args.steps)
    dev_batch = b.last_run_ms() / 1e3
    gpu_launches = b.launches() - launches0
    rows_b, bits_b = [], []
    for slot in slots:
        b._check(b.lib.sampo_batch_rows(b.h, slot, 0, nsteps + 1, hR.p))
        rows_b.append(hR.a.copy())
        bits_b.append(b.state(slot)[2])
    wall_e2e = time.perf_counter() - t_all
    for h in (hT, hE, hR):
        h.free()
    b.close()
    # ---- one at a time through the plain path ----
    from sampo_gb300._lib import SampoError
    plain_run_s, plain_total_s, exact, live_sum, overflow = 0.0, 0.0, 0, 0, 0
    for i, (s, (T, env, init, seeds)) in enumerate(zip(specs, prep)):
        t0 = time.perf_counter()
        with Simulation(capacity=s.capacity, carrying_capacity=s.cc, max_steps=s.steps + 1) as sim:
            sim.set_inputs(T, env)
            sim.set_seeds(0, seeds)
            sim.init_population(s.initial, init, age_days_max=s.age_days_max, age_seed=s.seed)
            try:
                r0 = sim.run(24 * args.warmup)
                sim.autotune()  # each replicate tuned on its own (outside the timed run)
                t1 = time.perf_counter()
                r1 = sim.run(24 * args.steps)
                plain_run_s += time.perf_counter() - t1
                rows = np.concatenate([r0, r1, [sim.current_row()]])
                live_sum += int(live_counts(r1).sum())
            except SampoError:  # outgrew its pool: compare the status bits only
                rows, overflow = None, overflow + 1
            bits = sim.device_status()
        plain_total_s += time.perf_counter() - t0
        exact += int((rows is None or rows.tobytes() == rows_b[i].tobytes()) and bits == bits_b[i])
    sizes = np.array([s.initial for s in specs])
    value = n * args.steps / dev_batch
    return {
        "metric": "replicate-days/s", "value": value, "unit": "replicate-days/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_batch * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+u32", "data": "synthetic",
        "config": {"workload": f"ensemble: {n} replicates, initial eggs log-uniform in [1e3, 1e6] aged U{{0..3}} days, "
                               "own seed and weather each (mean T U[20,30] C, amplitude U[2,8] C, sd 0.5), "
                               f"days {args.warmup}..{days} of a 365-day run; capacity 20 x initial + 65536",
                   "step": "one simulated day of every replicate (24 hourly steps, one CUDA graph)",
                   "seeds": "batched: drawn on the device per replicate (sampo_batch_seed_stream); "
                            "one at a time: uploaded",
                   "initial_agents_total": int(sizes.sum()), "agent_days_timed": live_sum / 24.0,
                   "ctas_per_sm": {"count": tuned[0], "scatter": tuned[1], "picked_by": "sampo_batch_autotune"},
                   "slots_per_thread": batch_items,
                   "l2": "pools far larger than L2"},
        "batched": {"replicate_days_per_s": value, "sims_per_s_365d_equiv": value / 365.0,
                    "agent_days_per_s": live_sum / 24.0 / dev_batch, "device_s": dev_batch,
                    "setup_s": setup_batch},
        "one_at_a_time": {"replicate_days_per_s": n * args.steps / plain_run_s, "run_s": plain_run_s,
                          "with_setup_s": plain_total_s},
        "speedup_vs_one_at_a_time": plain_run_s / dev_batch,
        "speedup_incl_setup": plain_total_s / (dev_batch + setup_batch),
        "bit_exact_replicates": f"{exact}/{n}",
        "replicates_out_of_capacity": overflow,
        "e2e": {"value": n * days / wall_e2e, "unit": "replicate-days/s",
                "h2d_bytes_per_step": n * 24 * (4 + 24 + 4), "d2h_bytes_per_step": n * 24 * 92,
                "window": f"the whole batched run: setup, days 0..{days}, grid tuning, rows read back"},
        "gpu_launches": gpu_launches,
        "clocks": clk.summary(),
    }


def ensemble_year_arm(args):
    """The ensemble at its stated horizon: every replicate runs its 365 days,
    admitted in waves under the HBM budget by the server (all arrive at time
    0; pools start at 2 x initial and grow). Against the plain path one
    replicate at a time, timed on a sample (every `--plain-every`-th replicate,
    scaled to all) and compared bit for bit on that sample."""
    from sampo_gb300.batch import ensemble_specs
    from sampo_gb300.serve import Request, Server, plain_result
    n, days = args.replicates, 365
    specs = ensemble_specs(n, seed=4, days=days, growth=2.0)
    reqs = [Request(i, s, 0.0) for i, s in enumerate(specs)]
    srv = Server(budget_bytes=int(args.budget_gb * 1e9), max_replicates=min(n, 1024), max_days=days)
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()
        res = srv.serve(reqs)
        wall = time.perf_counter() - t0
    gpu_launches = srv.batch.launches()
    srv.close()
    agent_days = sum(float(live_counts(r.rows[:-1]).sum()) for r in res) / 24.0
    sample = list(range(0, n, args.plain_every))
    plain_s, exact = 0.0, 0
    by_id = {r.rid: r for r in res}
    for i in sample:
        t1 = time.perf_counter()
        rows, hist, status = plain_result(specs[i])
        plain_s += time.perf_counter() - t1
        r = by_id[i]
        exact += int(rows is not None and r.rows.tobytes() == rows.tobytes() and np.array_equal(r.histogram, hist)
                     and r.status == status)
    plain_all = plain_s * n / len(sample)
    value = n * days / wall
    return {
        "metric": "replicate-days/s", "value": value, "unit": "replicate-days/s", "n_gpus": 1, "steps": days,
        "warmup": 0, "ms_per_step": wall * 1e3 / days, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+u32", "data": "synthetic",
        "config": {"workload": f"ensemble at its horizon: {n} replicates x 365 days, initial eggs log-uniform in "
                               "[1e3, 1e6] aged U{0..3} days, own seed and weather each (mean T U[20,30] C, amplitude "
                               f"U[2,8] C, sd 0.5); admitted in waves under a {args.budget_gb:g} GB HBM budget, pools "
                               "start at 2 x initial + 65536 slots and grow",
                   "step": "one simulated day of every resident replicate (24 hourly steps, one CUDA graph)",
                   "seeds": "batched: drawn on the device per replicate; one at a time: uploaded",
                   "initial_agents_total": int(sum(s.initial for s in specs))},
        "batched": {"wall_s": wall, "replicate_days_per_s": value, "sims_per_s": n / wall,
                    "agent_days_per_s": agent_days / wall, "agent_days": agent_days,
                    "days_stepped": srv.days_run, "peak_resident": srv.peak_resident,
                    "peak_hbm_gb": srv.peak_bytes / 1e9, "pool_growths": srv.grows,
                    "growths_after_a_pause": srv.pauses, "growths_over_budget": srv.over_budget},
        "one_at_a_time": {"sample": f"{len(sample)} of {n} replicates (every {args.plain_every}th)",
                          "sample_s": plain_s, "scaled_s": plain_all, "sims_per_s": n / plain_all},
        "speedup_vs_one_at_a_time": plain_all / wall,
        "bit_exact_sample": f"{exact}/{len(sample)}",
        "e2e": {"value": value, "unit": "replicate-days/s", "h2d_bytes_per_step": n * 24 * (4 + 24 + 4),
                "d2h_bytes_per_step": n * 24 * 92,
                "note": "value is already end to end: wall clock through sampo_gb300.serve.Server, inputs up and rows down"},
        "gpu_launches": gpu_launches,
        "gpu_launches_counts": "step kernels (day graphs' kernel nodes + one constants refresh per run call); "
                               "pool set-up and growth copies not counted",
        "clocks": clk.summary(),
    }


def served_arm(args):
    """The served request stream, a bounded number of requests per rate."""
    from sampo_gb300.serve import Server, latency_summary, one_at_a_time, request_stream
    rates = [float(x) for x in args.rates.split(",")]
    out = {"metric": "sims/s", "unit": "sims/s", "n_gpus": 1, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32+u32", "data": "synthetic", "steps": args.requests, "warmup": 0}
    per_rate = {}
    plain = None
    for rate in rates:
        reqs = request_stream(args.requests, rate, seed=7, days_range=(args.min_days, args.max_days))
        srv = Server(budget_bytes=int(args.budget_gb * 1e9), max_days=args.max_days)
        t0 = time.perf_counter()
        res = srv.serve(reqs)
        makespan = max(r.completed for r in res) - min(r.arrival for r in res)
        launches = srv.batch.launches()
        srv.close()
        if plain is None:  # service times do not depend on the arrival rate
            plain = {p["rid"]: p for p in one_at_a_time(reqs)}
        prev, lat_plain = 0.0, []
        for r in sorted(reqs, key=lambda r: r.arrival):
            prev = max(r.arrival, prev) + plain[r.rid]["service"]
            lat_plain.append(prev - r.arrival)
        plain_makespan = prev - min(r.arrival for r in reqs)
        def same(x):
            p = plain[x.rid]
            if x.status != p["status"]:
                return False
            if p["rows"] is None:  # both outgrew their pools at the same step
                return True
            return x.rows is not None and x.rows.tobytes() == p["rows"].tobytes()
        exact = sum(int(same(x)) for x in res)
        # the stream's work, and how fast each path does it: batching cannot
        # beat the rate at which the HBM-bound large requests already run alone
        agent_days = sum(float(live_counts(x.rows[:-1]).sum()) for x in res if x.rows is not None) / 24.0
        service = sum(p["service"] for p in plain.values())
        per_rate[str(rate)] = {
            "agent_days": agent_days, "batched_agent_days_per_s": agent_days / makespan,
            "one_at_a_time_agent_days_per_s": agent_days / service,
            "sims_per_s": len(res) / makespan, "latency_s": latency_summary([r.latency for r in res]),
            "one_at_a_time": {"sims_per_s": len(reqs) / plain_makespan, "latency_s": latency_summary(lat_plain)},
            "speedup_sims_per_s": (len(res) / makespan) / (len(reqs) / plain_makespan),
            "bit_exact": f"{exact}/{len(res)}", "peak_resident": srv.peak_resident,
            "peak_hbm_gb": srv.peak_bytes / 1e9, "days_stepped": srv.days_run, "pool_growths": srv.grows,
            "growths_after_a_pause": srv.pauses, "growths_over_budget": srv.over_budget,
            "days_admission_held": srv.held_days, "gpu_launches": launches, "wall_s": time.perf_counter() - t0}
    first = per_rate[str(rates[0])]
    # host traffic per request (the line's step): its inputs up at admission
    # (temperature, environment row, world time per hourly step) and its stats
    # rows and histogram down at completion
    hours = np.array([r.spec.steps for r in request_stream(args.requests, rates[0], seed=7,
                                                          days_range=(args.min_days, args.max_days))], dtype=np.float64)
    out.update({"value": first["sims_per_s"], "ms_per_step": None,
                "config": {"workload": f"served stream: {args.requests} requests per rate, Poisson arrivals, initial eggs "
                                       f"log-uniform in [1e2, 5e6], horizons U{{{args.min_days}..{args.max_days}}} days, "
                                       f"own seed and weather each, {args.budget_gb:g} GB HBM budget; pools admitted at 2 x initial + "
                                       "65536 slots and grown (one at a time: a fixed pool of 96 x initial + 65536)",
                           "rates_per_s": rates},
                "per_rate": per_rate,
                "e2e": {"value": first["sims_per_s"], "unit": "sims/s", "h2d_bytes_per_step": float(hours.mean() * (4 + 24 + 4)),
                        "d2h_bytes_per_step": float((hours.mean() + 1) * 92 + 400),
                        "note": "value is already end to end: wall clock through sampo_gb300.serve.Server"},
                "gpu_launches": first["gpu_launches"]})
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="roofline", choices=list(WORKLOADS) + ["ensemble", "ensemble-year", "served"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--ctas-per-sm", default="",
                    help="COUNT,SCATTER: fixed grid sizes of the plain-path workloads instead of the autotuner")
    ap.add_argument("--small-step", default="auto",
                    help="plain-path workloads: 'auto' (one-launch step for pools of up to one tile per CTA of its "
                         "grid), 'off' (the three-kernel step every hour) or a largest pool in 1024-slot tiles")
    ap.add_argument("--small-items", type=int, default=0, choices=(0, 1, 2, 4),
                    help="plain-path workloads: slots per thread of the one-launch step (0: by pool size)")
    ap.add_argument("--replicates", type=int, default=512, help="ensemble: replicates")
    ap.add_argument("--requests", type=int, default=200, help="served: requests per rate")
    ap.add_argument("--plain-every", type=int, default=8, help="ensemble-year: the one-at-a-time arm's sample stride")
    ap.add_argument("--batched-sample", type=int, default=64,
                    help="plain workloads: replicates of the compact batched-vs-one-at-a-time figure (0: none)")
    ap.add_argument("--rates", default="10,100,1000", help="served: arrival rates per second")
    ap.add_argument("--budget-gb", type=float, default=150.0, help="served: HBM budget")
    ap.add_argument("--min-days", type=int, default=30)
    ap.add_argument("--max-days", type=int, default=365)
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("at least 3 warm-up steps")
    if args.workload in ("ensemble", "ensemble-year", "served"):
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference runs one simulation per process; "
                              "its arm is the plain workloads"}))
            return
        if args.workload == "ensemble":
            if "--steps" not in sys.argv:
                args.steps = 12
            print(json.dumps(ensemble_arm(args)))
        elif args.workload == "ensemble-year":
            print(json.dumps(ensemble_year_arm(args)))
        else:
            print(json.dumps(served_arm(args)))
        return
    wl = WORKLOADS[args.workload]
    rank, world, local = dist_env()
    dist_init(world)
    # both arms print this same config: the workload and the simulated days they time
    cfg = {"workload": wl["name"], "step": "one simulated day = 24 hourly steps",
           "days_warmup": args.warmup, "days_timed": args.steps, "window": f"days {args.warmup}..{args.warmup + args.steps}",
           "capacity_slots": wl["capacity"], "carrying_capacity": wl["cc"],
           "l2": "GPU arm: flushed between timed days (write of a buffer > 2x L2)"}

    if args.impl == "reference":
        if rank != 0:
            return
        # the reference's per-step algorithm on the host cores over the same
        # days: warm-up days untimed, then the timed days
        ref = cpu_reference(wl, 0, first_steps=24 * args.steps, warmup=24 * args.warmup)
        line = {"impl": "reference", "metric": "agent-days/s", "value": ref["value"], "unit": "agent-days/s",
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": ref["seconds"] * 1e3 / max(args.steps, 1), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32+u32", "data": "synthetic", "config": cfg,
                "cpu_baseline": {"value": ref["value"], "unit": "agent-days/s", "cores": ref["threads"], "kind": "port",
                                 "sample": f"hourly steps {24 * args.warmup}..{24 * (args.warmup + args.steps)} of the workload "
                                           f"(the timed days; {ref['seconds']:.1f} s), all host threads (OpenMP)"},
                "e2e": {"value": ref["value"], "unit": "agent-days/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    r = gpu_arm(args, wl, rank, world, local if world > 1 else 0)
    dev_s = r["ms"] / 1e3
    tmax, = all_reduce([dev_s], "max")
    e2e_max, = all_reduce([r["e2e_wall"]], "max")
    tot_days, e2e_days = all_reduce([r["agent_days"], r["e2e_agent_days"]], "sum")
    if rank != 0:
        return
    cpu = cpu_reference(wl, args.cpu_seconds) if world == 1 else None
    live_tot = r["live"].sum(axis=1)
    pool_bytes = live_tot * RECORD_BYTES
    details = {"live_agents_min": int(live_tot.min()), "live_agents_max": int(live_tot.max()),
               "pool_bytes": [float(pool_bytes.min()), float(pool_bytes.max())], "parallelism": f"replicas x{world}",
               "ctas_per_sm": {"count": r["tuned"][0], "scatter": r["tuned"][1],
                               "picked_by": "--ctas-per-sm" if args.ctas_per_sm else "sampo_autotune"},
               "slots_per_thread": r["items"],
               "small_step": {"largest_grid_ctas": r["small"]["grid"], "max_tiles": r["small"]["max_tiles"],
                              "timed_days_one_launch": r["small"]["days_one_launch"] - r["small0"]["days_one_launch"],
                              "timed_days_three_kernel": r["small"]["days_three_kernel"] - r["small0"]["days_three_kernel"],
                              "one_launch_kind": {0: "-", 1: "-", 2: "cooperative launch", 3: "plain launch of a co-resident grid"}[r["small"]["last_day"]],
                              "slots_per_thread": args.small_items or "by pool size (the smallest tiles, of 256, 512 or 1024 slots, that fit two per CTA of the largest grid)"}}
    line = {
        "metric": "agent-days/s", "value": job_rate(tot_days, tmax), "unit": "agent-days/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": tmax * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+u32 (f64 where the reference promotes)",
        "data": "synthetic", "config": cfg, "details": details,
        "roofline": {"bound": "hbm", "achieved": r["achieved"], "peak": r["peak"], "unit": "GB/s",
                     "frac": r["achieved"] / r["peak"], "traffic": r["traffic"], "kernel": "k_scatter (update + stable scatter)",
                     "traffic_from": "scaled: DRAM bytes per live agent of a single-pass ncu capture of k_scatter on the "
                                     "roofline workload at 5.7e7 live agents (profiles/k_scatter_dram.json: 0.998 of the "
                                     "algorithmic bytes) x this run's mean live pool",
                     "peak_kind": r["peak_kind"], "scatter_ms_per_launch": r["scatter_ms"], "count_ms_per_launch": r["count_ms"],
                     "publish_and_gaps_ms_per_step": r["publish_ms"],
                     "count_pass_gbs": r["count_gbs"],
                     "algorithmic_bytes": "k_scatter: 37 B read per live agent + 37 B written per agent of the next pool",
                     "passes": r["passes"]},
        "e2e": {"value": e2e_days / e2e_max, "unit": "agent-days/s", "h2d_bytes_per_step": 24 * (4 + 24 + 4 + 64),
                "d2h_bytes_per_step": 24 * 92},
        "gpu_launches": r["gpu_launches"] * world,
        "clocks": r["clocks"],
        "wall_s_timed": r["wall"],
    }
    if args.batched_sample and world == 1:
        # a compact record of batching: the ensemble workload's replicates,
        # fewer of them, over days 3..6, batched against one at a time
        import copy
        a2 = copy.copy(args)
        a2.replicates, a2.warmup, a2.steps = args.batched_sample, 3, 3
        e = ensemble_arm(a2)
        line["batched_vs_one_at_a_time"] = {
            "workload": f"{a2.replicates} replicates of the ensemble workload (initial eggs log-uniform in [1e3, 1e6]), "
                        "days 3..6, device time of the timed days",
            "batched_replicate_days_per_s": e["value"],
            "one_at_a_time_replicate_days_per_s": e["one_at_a_time"]["replicate_days_per_s"],
            "speedup": e["speedup_vs_one_at_a_time"], "bit_exact_replicates": e["bit_exact_replicates"]}
    if cpu:
        line["cpu_baseline"] = {"value": cpu["value"], "unit": "agent-days/s", "cores": cpu["threads"], "kind": "port",
                                "sample": f"first {cpu['steps']} hourly steps of the same workload ({cpu['seconds']:.1f} s), oracle port, OpenMP"}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
