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
