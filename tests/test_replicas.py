"""Multi-GPU is replicas only: every rank runs its own simulation with its
own seed stream and no data-path collective; bench.py combines the ranks with
a barrier, the max of the device times and the sum of the work. This runs
that aggregation with two gloo ranks on the CPU."""
import multiprocessing as mp
import os
import socket


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import bench
    r, w, _ = bench.dist_env()
    bench.dist_init(w)
    seconds = 1.5 + rank                 # this rank's device time
    agent_days = 1000.0 * (rank + 1)     # this rank's work
    bench.sync_barrier(w)
    tmax, = bench.all_reduce([seconds], "max")
    total, = bench.all_reduce([agent_days], "sum")
    from sampo_gb300.sim import seed_stream
    init, seeds = seed_stream(bench.rank_seed(2, r), 48)
    q.put((r, tmax, total, bench.job_rate(total, tmax), int(seeds[0, 0, 0]), int(init[0, 0])))
    bench._PG.destroy_process_group()


def test_two_gloo_ranks_aggregate_like_bench(sampo_lib):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, t0, s0, v0, a0, i0), (r1, t1, s1, v1, a1, i1) = out
    assert (r0, r1) == (0, 1)
    assert t0 == t1 == 2.5            # the slowest rank's time
    assert s0 == s1 == 3000.0         # work summed over ranks
    assert v0 == v1 == 3000.0 / 2.5   # weak scaling: the whole job's rate
    assert (a0, i0) != (a1, i1)       # independent seed streams
    import bench
    from sampo_gb300.sim import seed_stream
    init, seeds = seed_stream(2, 48)
    assert (int(seeds[0, 0, 0]), int(init[0, 0])) == (a0, i0)  # rank 0 runs the workload's own seed
