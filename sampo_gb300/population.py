"""Mixed-stage initial populations (an extension of the reference, whose
only initial population is age-0 eggs, src/abms.c:185-228).

make_pool(counts, ...) builds a pool in the layout a compaction produces
(kernel/oldToNewAgents.cl:57-95: eggs at [0, n_egg), every next range at
((previous end + 64) / 64) * 64). Field values are drawn from a seeded
numpy PCG64 generator; they follow the reference's meaning of each field so
the first steps behave like a population in progress:

  egg      ageInHours = hoursInState = U{0..71}; delay = eggsIncubation(T0)
           + eggsHatching(U[0,1)) as initAgents draws it.
  larva    hoursInState = U{0..(24*larva_days-1)}, ageInHours = 24 + that;
           delay = max(N(1, 0.1), 0.05) (larvaDelay);
           cumulativeLarvalDelay = hoursInState * larvaDevelopment(T0), capped
           below delay.
  pupa     hoursInState = U{0..pupaDelay(T0)-1}; ageInHours = 24*(1+larva_days)
           + hoursInState; delay = pupaDelay(T0).
  adult    ageInHours = U{0..24*adult_days-1}. Females are spread over
           IMMATURE, MATESEEKING, BMS, BMD, GRAVID with female_split; males
           are IMMATURE or MATESEEKING (males never leave MATESEEKING,
           kernel/updateAgents.cl:146). State fields are set as the
           reference sets them on entering each state; bitten states carry
           humanBloodmealCount >= 1, cumulativeSporogonicDevelopment ~
           U[0, 1.5), numEggBatches >= 1; gravids carry availableEggs
           U{1..170} and ovipositionAttemps U{0..2}.
  isFemale is Bernoulli(female_frac) for every agent.

All float fields are float32 values computed with float32 arithmetic.
"""
from __future__ import annotations

import numpy as np

from ._lib import POOL_COLUMNS

LAYOUT_ALIGN = 64
F = np.float32


def padded_ranges(counts) -> np.ndarray:
    r = np.zeros((8, 2), dtype=np.int64)
    r[0] = (0, counts[0])
    for k in range(1, 8):
        s = ((r[k - 1][1] + LAYOUT_ALIGN) // LAYOUT_ALIGN) * LAYOUT_ALIGN
        r[k] = (s, s + counts[k])
    return r


def eggs_incubation(T):
    return F(F(F(-0.923) * F(T)) + F(60.923))


def eggs_hatching(p: np.ndarray) -> np.ndarray:
    p = p.astype(np.float32)
    m = np.select([p < F(0.5), p < F(0.85), p < F(0.90), p < F(0.94)], [F(48.0), F(68.5714), F(480.0), F(600.0)], F(2400.0)).astype(np.float32)
    b = np.select([p < F(0.5), p < F(0.85), p < F(0.90), p < F(0.94)], [F(0.0), F(-10.2857), F(-360.0), F(-468.0)], F(-2160.0)).astype(np.float32)
    v = ((m * p).astype(np.float32) + b).astype(np.float32) + F(0.5)
    return np.floor(np.maximum(v, F(0))).astype(np.uint32).astype(np.float32)


DEV_RATES = np.array([0.000175044, 0.000549094, 0.00109031, 0.001494158, 0.001752487, 0.001962866, 0.002171238,
                      0.002392989, 0.002633689, 0.00289619, 0.003182685, 0.003495287, 0.003836204, 0.004207789,
                      0.004612566, 0.005053243, 0.005532729, 0.006054144, 0.006620836, 0.007236393, 0.007904657,
                      0.008629745, 0.009416051, 0.010267388, 0.011113704, 0.011960019, 0.012806335, 0.010401163,
                      0.007995991, 0.00033845, 0.00000533086, 0.0000000840986]).astype(np.float32)


def larva_stage_hours(T0: float) -> int:
    """Hours of development until a mean larva (delay 1.0) pupates at T0."""
    Ti = int(np.clip(np.float32(T0), F(12.0), F(48.0))) - 12
    return max(24, int(1.0 / float(DEV_RATES[min(Ti, 31)])))


# Adult sub-state split near the end of a year-long run of the CPU-runnable
# workload: females over IMMATURE, MATESEEKING, BMS, BMD, GRAVID; males over
# IMMATURE, MATESEEKING.
FEMALE_SPLIT = (0.26, 0.10, 0.04, 0.26, 0.34)
MALE_SPLIT = (0.26, 0.74)


def make_pool(counts_by_stage, T0: float, seed: int, female_frac: float = 0.5, larva_days: int | None = None,
              adult_days: int = 20, female_split=FEMALE_SPLIT, male_split=MALE_SPLIT):
    """counts_by_stage = (eggs, larvae, pupae, adults). Returns (ranges, arrays).
    larva_days=None spreads larval development uniformly over the stage
    length at T0 (larva_stage_hours)."""
    if larva_days is None:
        larva_days = max(1, larva_stage_hours(T0) // 24)
    rng = np.random.default_rng(seed)
    n_egg, n_lar, n_pup, n_ad = (int(c) for c in counts_by_stage)
    female_ad = rng.uniform(size=n_ad) < female_frac
    nf = int(female_ad.sum())
    nm = n_ad - nf
    fs = np.asarray(female_split, dtype=np.float64) / sum(female_split)
    ms = np.asarray(male_split, dtype=np.float64) / sum(male_split)
    fcnt = np.floor(fs * nf).astype(np.int64)
    fcnt[0] += nf - fcnt.sum()
    mcnt = np.floor(ms * nm).astype(np.int64)
    mcnt[0] += nm - mcnt.sum()
    counts = [n_egg, n_lar, n_pup, fcnt[0] + mcnt[0], fcnt[1] + mcnt[1], fcnt[2], fcnt[3], fcnt[4]]
    ranges = padded_ranges(counts)
    n = int(ranges[7][1])
    a = {name: np.zeros(n, dtype=dt) for name, dt in POOL_COLUMNS}
    T0 = F(T0)
    Ti = int(np.clip(T0, F(12.0), F(48.0))) - 12
    dev = DEV_RATES[min(Ti, 31)]
    pupa_delay = F(np.float64(-0.923) * np.float64(T0) + np.float64(60.923))
    imm_delay = F(F(F(-2.667) * T0) + F(120.0))
    bmd_delay = F(F(F(-1.231) * T0) + F(77.231))

    def sl(k):
        return slice(int(ranges[k][0]), int(ranges[k][1]))

    # eggs
    s = sl(0)
    h = rng.integers(0, 72, n_egg).astype(np.float32)
    a["ageInHours"][s] = h
    a["hoursInState"][s] = h
    a["delay"][s] = (eggs_incubation(T0) + eggs_hatching(rng.uniform(size=n_egg))).astype(np.float32)
    a["state"][s] = 0
    a["isFemale"][s] = rng.uniform(size=n_egg) < female_frac
    # larvae
    s = sl(1)
    his = rng.integers(0, min(24 * larva_days, larva_stage_hours(T0)), n_lar).astype(np.float32)
    a["hoursInState"][s] = his
    a["ageInHours"][s] = (his + F(24.0)).astype(np.float32)
    dl = np.maximum(rng.normal(1.0, 0.1, n_lar), 0.05).astype(np.float32)
    a["delay"][s] = dl
    cld = np.minimum((his * dev).astype(np.float32), (dl * F(0.99)).astype(np.float32)).astype(np.float32)
    a["larvalDelayOrOviAttempts"][s] = cld.view(np.uint32)
    a["state"][s] = 1
    a["isFemale"][s] = rng.uniform(size=n_lar) < female_frac
    # pupae
    s = sl(2)
    his = rng.integers(0, max(int(pupa_delay), 1), n_pup).astype(np.float32)
    a["hoursInState"][s] = his
    a["ageInHours"][s] = (his + F(24.0 * (1 + larva_days))).astype(np.float32)
    a["delay"][s] = pupa_delay
    a["state"][s] = 2
    a["isFemale"][s] = rng.uniform(size=n_pup) < female_frac
    # adults: females first within IMMATURE and MATESEEKING, then males
    for k in range(3, 8):
        s = sl(k)
        m = int(ranges[k][1] - ranges[k][0])
        if m == 0:
            continue
        nfk = int(fcnt[k - 3])
        fem = np.zeros(m, dtype=np.uint8)
        fem[:nfk] = 1
        a["isFemale"][s] = fem
        a["state"][s] = k
        age = rng.integers(0, 24 * adult_days, m).astype(np.float32)
        a["ageInHours"][s] = age
        if k == 3:
            a["hoursInState"][s] = np.minimum(age, imm_delay - F(1.0)).astype(np.float32)
            a["delay"][s] = imm_delay
        elif k == 4:
            a["hoursInState"][s] = np.floor(age * F(0.5)).astype(np.float32)
            a["delay"][s] = F(1.0)
        else:
            bitten = k >= 6
            a["humanBloodmealCount"][s] = rng.integers(1 if bitten else 0, 4, m)
            a["cumulativeSporogonicDevelopment"][s] = np.where(a["humanBloodmealCount"][s] > 0,
                                                               rng.uniform(0.0, 1.5, m), 0.0).astype(np.float32)
            a["cycleLength"][s] = rng.integers(0, 72, m)
            a["numEggBatches"][s] = rng.integers(1 if bitten else 0, 4, m)
            if k == 5:
                a["hoursInState"][s] = rng.integers(0, 24, m).astype(np.float32)
                a["delay"][s] = F(0.0)
            elif k == 6:
                a["hoursInState"][s] = rng.integers(0, max(int(bmd_delay), 1), m).astype(np.float32)
                a["delay"][s] = bmd_delay
            else:
                a["hoursInState"][s] = rng.integers(0, 24, m).astype(np.float32)
                a["availableEggs"][s] = rng.integers(1, 171, m)
                a["larvalDelayOrOviAttempts"][s] = rng.integers(0, 3, m)
    return ranges, a
