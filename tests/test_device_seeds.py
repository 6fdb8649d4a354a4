"""Device-side seed streams (sampo_batch_seed_stream): a replicate that draws
the generateSeeds values of every step (src/abms.c:145-150) on the GPU, from
its own copy of the glibc rand() stream, must run bit for bit like the same
simulation fed host-drawn seeds, and its stream must stay on the platform's
glibc sequence (the host restatement is pinned to libc's rand() in
test_math_rand.py)."""
import ctypes as C

import numpy as np
import pytest

from tests.test_batch import SPECS, compare, plain_run


def _host_stream(seed: int, draws: int):
    """srand(seed) followed by `draws` rand() calls."""
    from sampo_gb300 import _lib
    from sampo_gb300._lib import RandState
    lib = _lib.load()
    st = RandState()
    lib.sampo_rand_seed(C.byref(st), seed)
    for _ in range(draws):
        lib.sampo_rand_next(C.byref(st))
    return st


def _draws(st, n: int) -> list[int]:
    from sampo_gb300 import _lib
    lib = _lib.load()
    return [lib.sampo_rand_next(C.byref(st)) for _ in range(n)]


def _check_stream(b, slot, seed: int, next_step: int):
    """The device stream has drawn the 16 initial values and 16 per step
    before next_step, and continues like the host stream from there."""
    st, nxt = b.seed_state(slot)
    assert nxt == next_step
    assert st.i % 31 == 0
    assert _draws(st, 200) == _draws(_host_stream(seed, 16 * (1 + next_step)), 200)


@pytest.mark.gpu
def test_device_seeds_equal_host_seeds(gpu_ready):
    from sampo_gb300.batch import Batch, admit
    steps = [72, 50, 72, 31, 72]
    on_device = [True, True, False, True, False]
    with Batch(max_replicates=8, ring_steps=80) as b:
        slots = [admit(b, s, st, device_seeds=d) for s, st, d in zip(SPECS, steps, on_device)]
        b.run(30)
        # the publish after step 29 drew the seeds of step 30
        _check_stream(b, slots[0], SPECS[0].seed, 31)
        _check_stream(b, slots[3], SPECS[3].seed, 31)   # stops at 31: step 31 is never drawn
        b.run(48)
        for s, spec, st, d in zip(slots, SPECS, steps, on_device):
            compare(b, s, spec, st, f"replicate {spec.seed} ({'device' if d else 'host'} seeds)")
        _check_stream(b, slots[0], SPECS[0].seed, 72)
        _check_stream(b, slots[1], SPECS[1].seed, 50)
        _check_stream(b, slots[3], SPECS[3].seed, 31)


@pytest.mark.gpu
def test_device_seeds_across_ring_wrap(gpu_ready):
    """Inputs fed a day at a time through a 30-step ring: the device writes
    each step's seeds into the step's ring slot like an upload would."""
    from sampo_gb300.batch import Batch
    from sampo_gb300.sim import rand_state
    spec, steps = SPECS[1], 72
    rows, pop, arrays, hist, status = plain_run(spec, steps)
    T, env = spec.inputs()
    with Batch(max_replicates=2, ring_steps=30) as b:
        slot = b.add(spec.capacity, spec.cc, stop_step=steps)
        b.set_inputs(slot, T[:24], env[:24])
        init, st = rand_state(spec.seed)
        b.init_population(slot, spec.initial, init, age_days_max=spec.age_days_max, age_seed=spec.seed)
        b.seed_stream(slot, st)
        got = []
        for day in range(3):
            if day:
                b.set_inputs(slot, T[24 * day:24 * day + 24], env[24 * day:24 * day + 24], first=24 * day)
            b.run(24)
            got.append(b.rows(slot, 24 * day, 24))
        got.append(b.rows(slot, steps, 1))
        assert np.concatenate(got).tobytes() == rows.tobytes()
        bpop, barrays = b.read_pool(slot)
        assert np.array_equal(bpop["ranges"], pop["ranges"])
        assert np.array_equal(b.histogram(slot), hist)
        _check_stream(b, slot, spec.seed, steps)


@pytest.mark.gpu
def test_seed_source_is_exclusive(gpu_ready):
    """Uploading seeds to a slot that draws its own fails, and so does
    reading the device stream of a slot fed from the host."""
    from sampo_gb300._lib import SampoError
    from sampo_gb300.batch import Batch, admit
    from sampo_gb300.sim import seed_stream
    with Batch(max_replicates=2, ring_steps=40) as b:
        dev = admit(b, SPECS[2], 24, device_seeds=True)
        host = admit(b, SPECS[0], 24)
        _, seeds = seed_stream(SPECS[2].seed, 24)
        with pytest.raises(SampoError):
            b.set_seeds(dev, 0, seeds)
        with pytest.raises(SampoError):
            b.seed_state(host)
        b.remove(dev)                    # a new occupant of the slot starts on host seeds again
        again = admit(b, SPECS[2], 24)
        assert again == dev
        b.run(24)
        compare(b, again, SPECS[2], 24, "host-seeded occupant of a device-seeded slot")
