"""Synthetic workloads with the shapes of the benchmark configurations (no datasets exist).

ensemble_params(): 256 replicates with populations log-uniform in [10k, 500k], grid side
ceil(sqrt(N / 0.16)), regular transmission rate uniform in [0.02, 0.10] (the other disease
fields of small pox), exposed = ceil(0.05% of N), 2,400 hours, no interventions, and one seed
per replicate -- all drawn from seed 11.
"""
from __future__ import annotations

import json
import math
import os

import numpy as np

from ._lib import EpiParams
from .engine import Config

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

SMALL_POX = {
    "regular_transmission_start_day": 10, "high_transmission_start_day": 16, "last_day": 22,
    "asymptomatic_last_day": 22, "mild_infected_last_day": 22,
    "regular_transmission_rate": 0.05, "high_transmission_rate": 0.5, "death_rate": 0.2,
    "percentage_asymptomatic_population": 0.0, "percentage_severe_infected_population": 1.0,
    "exposed_duration": 0, "pre_symptomatic_duration": 0,
}


def config_dict(n: int, grid: int, hours: int, seed: int, disease: dict | None = None, exposed: int = 1,
                interventions: list | None = None, **extra) -> dict:
    cfg = {
        "population": {"Auto": {"number_of_agents": n, "public_transport_percentage": 0.2, "working_percentage": 0.7}},
        "disease": dict(disease or SMALL_POX),
        "geography_parameters": {"grid_size": grid, "hospital_beds_percentage": 0.003},
        "hours": hours,
        "interventions": interventions or [],
        "starting_infections": {"infected_mild_asymptomatic": 0, "infected_mild_symptomatic": 0,
                                "infected_severe": 0, "exposed": exposed},
        "seed": seed,
    }
    cfg.update(extra)
    return cfg


def params_of(cfg: dict) -> EpiParams:
    return Config(json.dumps(cfg)).params


def ensemble_configs(replicates: int = 256, seed: int = 11, hours: int = 2400, n_min: float = 1e4,
                     n_max: float = 5e5) -> list[dict]:
    rng = np.random.default_rng(seed)
    out = []
    for r in range(replicates):
        n = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        grid = int(math.ceil(math.sqrt(n / 0.16)))
        disease = dict(SMALL_POX)
        disease["regular_transmission_rate"] = float(rng.uniform(0.02, 0.10))
        rep_seed = int(rng.integers(1, 2 ** 63 - 1))
        out.append(config_dict(n, grid, hours, rep_seed, disease, exposed=int(math.ceil(0.0005 * n))))
    return out


def ensemble_params(**kw) -> list[EpiParams]:
    return [params_of(c) for c in ensemble_configs(**kw)]
