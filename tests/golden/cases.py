"""Golden cases: parameters and deterministic inputs (shared by the fixture
generator and the tests; nothing here reads the reference tree)."""
from __future__ import annotations

import os
import sys

REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

import numpy as np  # noqa: E402

from sampo_gb300 import inputs  # noqa: E402

CASES = {
    # The CPU-runnable benchmark workload: 10,000 eggs aged U{0..3} days,
    # seasonal weather (26 +- 4 C, noise 0.5), 365 days, seed 1, cc = 5 x 10,000.
    "eggs_1e4_year": dict(seed=1, initial=10000, cc=50000.0, steps=8760, age_days=3, age_seed=1,
                          weather=("seasonal", 365, 1, 26.0, 4.0, 0.5), interventions=None),
    # All four interventions switched on and off every 10 days.
    "interventions": dict(seed=3, initial=2000, cc=10000.0, steps=1440, age_days=3, age_seed=3,
                          weather=("seasonal", 60, 5, 27.0, 3.0, 0.5), interventions="alternating"),
    # The reference's own defaults: age-0 eggs, shipped constant 30 C and
    # no-intervention files (regenerated byte for byte), its initial layout.
    "reference_default": dict(seed=11, initial=32000, cc=160000.0, steps=1200, age_days=-1, age_seed=0,
                              weather=("constant30", 50), interventions=None),
    # Constant-temperature segments across the species functions' edges, after
    # a warm start that brings bitten adults: 16.0 C (sporogonic development
    # off, the test is T > 16), 16.5 C, 8.0 C (below the devRates clamp at
    # 12 C), exactly 12.0 C, 43.9 C (the last devRates entry), then 30 C.
    "temperature_edges": dict(seed=21, initial=2000, cc=10000.0, steps=960, age_days=3, age_seed=6,
                              weather=("segments", ((18, 28.0), (4, 16.0), (4, 16.5), (4, 8.0), (2, 12.0),
                                                    (3, 43.9), (5, 30.0))), interventions=None),
    # A mixed-stage start: every one of the eight states populated
    # (sampo_gb300.population.make_pool at the first hour's temperature),
    # loaded in place of the initial eggs; interventions on from day 10.
    "mixed_pool": dict(seed=31, initial=0, cc=27500.0, steps=480, age_days=-1, age_seed=0,
                       pool=dict(counts=(1500, 1200, 400, 2400), seed=17),
                       weather=("seasonal", 20, 9, 27.0, 3.0, 0.5), interventions="alternating"),
    # Small, quick cases for the CPU suite.
    "small_a": dict(seed=7, initial=600, cc=3000.0, steps=720, age_days=3, age_seed=9,
                    weather=("seasonal", 30, 2, 25.0, 5.0, 0.5), interventions=None),
    "small_b": dict(seed=123456789, initial=1500, cc=7500.0, steps=960, age_days=2, age_seed=4,
                    weather=("seasonal", 40, 3, 29.0, 2.0, 0.5), interventions="alternating"),
}

# Cases run with another species header (tests/golden/species/) in place of
# the shipped properties.h: the reference's kernels compiled against it
# (oracle/ref_build, target species) give the fixtures.
SPECIES_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "species")
SPECIES_CASES = {
    # every species hook differs; interventions on and off so that the
    # *_PROBABILITY factors matter too
    "hot_species": dict(seed=99, initial=2000, cc=10000.0, steps=1440, age_days=3, age_seed=5,
                        weather=("seasonal", 60, 8, 26.0, 4.0, 0.5), interventions="alternating",
                        species="hot_species.h"),
}


def make_case_inputs(name: str, directory: str):
    c = CASES[name] if name in CASES else SPECIES_CASES[name]
    w = c["weather"]
    if w[0] == "seasonal":
        _, days, wseed, mean, amp, sd = w
        weather = inputs.seasonal_weather(days, wseed, mean, amp, sd)
        tp, ep = inputs.write_inputs(directory, weather,
                                     inputs.alternating_interventions() if c["interventions"] == "alternating" else None)
    elif w[0] == "segments":
        temps = [t for days, t in w[1] for _ in range(days)]
        weather = inputs.DailyWeather(np.array(temps, dtype=np.float64), np.full(len(temps), 75.0),
                                      np.full(len(temps), 4.0))
        tp, ep = inputs.write_inputs(directory, weather,
                                     inputs.alternating_interventions() if c["interventions"] == "alternating" else None)
    elif w[0] == "constant30":
        days = w[1]
        tp = os.path.join(directory, "temp.txt")
        ep = os.path.join(directory, "environment.txt")
        with open(tp, "w") as f:
            f.writelines(["30 \n"] * (days * 24))
        with open(ep, "w") as f:
            f.writelines(["0, 0, 0, 0, 0, 0, 0, 0, 0.25 \n"] * (days * 24))
    else:
        raise ValueError(w)
    meta = {"temp_sha256": inputs.file_sha256(tp), "env_sha256": inputs.file_sha256(ep)}
    return tp, ep, meta


def case_pool(name: str, T0: float):
    """The initial pool of a case with a "pool" entry: (ranges, arrays)."""
    from sampo_gb300.population import make_pool
    p = CASES[name]["pool"]
    return make_pool(p["counts"], T0, seed=p["seed"])


def write_ref_pool(path: str, ranges, arrays) -> None:
    """A pool in the file format of ref-as-C's --pool option: "SAMPOPL1", the
    ranges, n, then the slots as the reference's device records (struct Agent,
    struct AgentAge, struct AgentState, include/agent.h:66-102)."""
    r = np.asarray(ranges, dtype=np.uint32).reshape(8, 2)
    n = int(r[7][1])
    agent = np.zeros(n, dtype=[("availableEggs", "<u4"), ("cycleLength", "<u4"), ("hbc", "<u4"), ("delay", "<f4"),
                               ("numEggBatches", "<u4"), ("uni", "<u4")])
    age = np.zeros(n, dtype=[("age", "<f4"), ("his", "<f4"), ("isFemale", "<i4"), ("sporo", "<f4")])
    st = np.zeros(n, dtype=[("dead", "<i4"), ("state", "<i4")])
    agent["availableEggs"] = arrays["availableEggs"][:n]
    agent["cycleLength"] = arrays["cycleLength"][:n]
    agent["hbc"] = arrays["humanBloodmealCount"][:n]
    agent["delay"] = arrays["delay"][:n]
    agent["numEggBatches"] = arrays["numEggBatches"][:n]
    agent["uni"] = arrays["larvalDelayOrOviAttempts"][:n]
    age["age"] = arrays["ageInHours"][:n]
    age["his"] = arrays["hoursInState"][:n]
    age["isFemale"] = arrays["isFemale"][:n].astype(np.int32)
    age["sporo"] = arrays["cumulativeSporogonicDevelopment"][:n]
    st["state"] = (1 << arrays["state"][:n].astype(np.int64)).astype(np.int32)
    with open(path, "wb") as f:
        f.write(b"SAMPOPL1")
        f.write(r.astype("<u4").tobytes())
        f.write(np.uint32(n).astype("<u4").tobytes())
        f.write(agent.tobytes())
        f.write(age.tobytes())
        f.write(st.tobytes())
