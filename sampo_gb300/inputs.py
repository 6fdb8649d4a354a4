"""Synthetic inputs in the reference's file formats.

The reference reads one temperature per hourly step from ``temp.txt``
(src/abms.c:94-108, ``fscanf("%f")``) and one intervention row per step from
``environment.txt`` (src/abms.c:110-137: four ``coverage, effectiveness``
pairs for IRS, ITN, larvicide and ovitrap, then ``bloodmealSuccess``). The
shipped files hold a constant 30 C and ``0, 0, 0, 0, 0, 0, 0, 0, 0.25``.

The benchmark workloads describe weather per day. ``write_inputs`` expands a
daily temperature series to 24 identical hourly rows per day. Relative
humidity and rainfall have no consumer in the reference (the larval
rainfall coefficient is the constant 1.0f, kernel/killAgents.cl:118, and
``struct Environment`` has no humidity field), so they are drawn and
returned for the record but never reach the model.
"""
from __future__ import annotations

import hashlib
import os
from dataclasses import dataclass

import numpy as np

NO_INTERVENTIONS = (0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.25)


@dataclass
class DailyWeather:
    temperature_c: np.ndarray   # float64, one value per day
    humidity_pct: np.ndarray    # recorded only
    rainfall_mm: np.ndarray     # recorded only


def seasonal_weather(days: int, seed: int, mean: float = 26.0, amplitude: float = 4.0,
                     noise_sd: float = 0.5, rain_mean: float = 5.0) -> DailyWeather:
    """temperature = mean + amplitude*sin(2*pi*d/365) + N(0, noise_sd^2);
    humidity ~ U(60, 80) %; rainfall = 0 with p = 0.6 else Exponential(rain_mean)."""
    rng = np.random.default_rng(seed)
    d = np.arange(days, dtype=np.float64)
    temp = mean + amplitude * np.sin(2.0 * np.pi * d / 365.0) + rng.normal(0.0, noise_sd, days)
    hum = rng.uniform(60.0, 80.0, days)
    wet = rng.uniform(0.0, 1.0, days) >= 0.6
    rain = np.where(wet, rng.exponential(rain_mean, days), 0.0)
    return DailyWeather(temp, hum, rain)


def constant_weather(days: int, temperature: float, humidity: float = 75.0, rainfall: float = 4.0) -> DailyWeather:
    return DailyWeather(np.full(days, temperature), np.full(days, humidity), np.full(days, rainfall))


def hourly_temperature(weather: DailyWeather) -> list[str]:
    """Text rows of temp.txt: each day's value repeated for its 24 steps."""
    rows = []
    for t in weather.temperature_c:
        s = "%.4f \n" % float(t)
        rows.extend([s] * 24)
    return rows


def write_inputs(directory: str, weather: DailyWeather, intervention_rows=None,
                 temp_name: str = "temp.txt", env_name: str = "environment.txt") -> tuple[str, str]:
    """Write temp.txt and environment.txt for len(weather)*24 steps.

    intervention_rows: None for the reference's no-intervention row, or a
    callable step -> 9 floats (IRS cov, eff, ITN cov, eff, larvicide cov,
    eff, ovitrap cov, eff, bloodmealSuccess)."""
    os.makedirs(directory, exist_ok=True)
    tp = os.path.join(directory, temp_name)
    ep = os.path.join(directory, env_name)
    rows = hourly_temperature(weather)
    with open(tp, "w") as f:
        f.writelines(rows)
    n = len(rows)
    with open(ep, "w") as f:
        if intervention_rows is None:
            line = "0, 0, 0, 0, 0, 0, 0, 0, 0.25 \n"
            f.writelines([line] * n)
        else:
            for i in range(n):
                f.write(", ".join("%.4f" % float(x) for x in intervention_rows(i)) + " \n")
    return tp, ep


def alternating_interventions(period_steps: int = 240):
    """Every other block of period_steps steps turns all four interventions on."""
    on = (0.6, 0.05, 0.5, 0.1, 0.4, 0.2, 0.5, 0.3, 0.5)
    off = (0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.3)
    return lambda i: on if (i // period_steps) % 2 else off


def file_sha256(path: str) -> str:
    h = hashlib.sha256()
    with open(path, "rb") as f:
        h.update(f.read())
    return h.hexdigest()


def read_temperature(path: str, nsteps: int) -> np.ndarray:
    """As src/abms.c:94-108: nsteps whitespace-separated floats."""
    vals = np.loadtxt(path, dtype=np.float64, max_rows=nsteps, ndmin=1)
    if vals.size < nsteps:
        raise ValueError(f"{path}: {vals.size} temperatures, {nsteps} steps requested")
    return vals.astype(np.float32)


ENV_DTYPE = np.dtype([("bloodmealSuccess", "<f4"), ("ITNValue", "<f4"), ("IRSValue", "<f4"),
                      ("carryingCapacity", "<f4"), ("larvacideValue", "<f4"), ("oviTrapValue", "<f4")])


def read_environment(path: str, nsteps: int, carrying_capacity: float) -> np.ndarray:
    """As src/abms.c:110-137: value = coverage*effectiveness in float32."""
    raw = np.loadtxt(path, dtype=np.float64, delimiter=",", max_rows=nsteps, ndmin=2)
    if raw.shape[0] < nsteps:
        raise ValueError(f"{path}: {raw.shape[0]} rows, {nsteps} steps requested")
    r = raw.astype(np.float32)
    env = np.zeros(nsteps, dtype=ENV_DTYPE)
    env["IRSValue"] = r[:, 0] * r[:, 1]
    env["ITNValue"] = r[:, 2] * r[:, 3]
    env["larvacideValue"] = r[:, 4] * r[:, 5]
    env["oviTrapValue"] = r[:, 6] * r[:, 7]
    env["bloodmealSuccess"] = r[:, 8]
    env["carryingCapacity"] = np.float32(carrying_capacity)
    return env
