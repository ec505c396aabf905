"""Config builders and comparison helpers shared by the tests."""
from __future__ import annotations

import copy
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

SMALL_POX = {
    "regular_transmission_start_day": 10, "high_transmission_start_day": 16, "last_day": 22,
    "asymptomatic_last_day": 22, "mild_infected_last_day": 22,
    "regular_transmission_rate": 0.05, "high_transmission_rate": 0.5, "death_rate": 0.2,
    "percentage_asymptomatic_population": 0.0, "percentage_severe_infected_population": 1.0,
    "exposed_duration": 0, "pre_symptomatic_duration": 0,
}

# a faster, messier disease: every branch of the state machine fires within a few days
COVID_FAST = {
    "regular_transmission_start_day": 1, "high_transmission_start_day": 3, "last_day": 6,
    "asymptomatic_last_day": 9, "mild_infected_last_day": 12,
    "regular_transmission_rate": 0.3, "high_transmission_rate": 0.6, "death_rate": 0.3,
    "percentage_asymptomatic_population": 0.3, "percentage_severe_infected_population": 0.4,
    "exposed_duration": 12, "pre_symptomatic_duration": 10,
}


def golden(name: str) -> dict:
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def make_config(n=500, grid=60, hours=240, disease=None, interventions=None, seed=1,
                starting=(0, 0, 0, 5), pt=0.2, working=0.7, beds=0.003, occupancy=None) -> dict:
    cfg = {
        "population": {"Auto": {"number_of_agents": n, "public_transport_percentage": pt,
                                "working_percentage": working}},
        "disease": copy.deepcopy(disease or SMALL_POX),
        "geography_parameters": {"grid_size": grid, "hospital_beds_percentage": beds},
        "hours": hours,
        "interventions": interventions or [],
        "starting_infections": {"infected_mild_asymptomatic": starting[0], "infected_mild_symptomatic": starting[1],
                                "infected_severe": starting[2], "exposed": starting[3]},
        "seed": seed,
    }
    if occupancy is not None:
        cfg["hospital_occupancy_trigger"] = occupancy
    return cfg


def rows_to_array(rows) -> np.ndarray:
    """(n, 7) uint32 from a structured counts array."""
    return np.stack([rows[k] for k in rows.dtype.names], axis=1).astype(np.int64)


def diff_records(a: np.ndarray, b: np.ndarray, limit: int = 5) -> str:
    """Human-readable first differences between two agent-record arrays."""
    out = []
    for name in a.dtype.names:
        bad = np.nonzero(a[name] != b[name])[0]
        if len(bad):
            out.append(f"{name}: {len(bad)} differ, e.g. agent {bad[0]}: {a[name][bad[0]]} vs {b[name][bad[0]]}")
    if out:
        i = int(np.nonzero(np.any([a[k] != b[k] for k in a.dtype.names], axis=0))[0][0])
        out.append(f"first differing agent {i}: {a[i]} vs {b[i]}")
    return "; ".join(out[:limit + 1])


def hospital_world(oracle_mod, occupy_hospital: bool):
    """A 50-grid world whose hospital is the row (40,0)-(44,0) after the resize, with one
    severe agent on day 19 (day 20 after the hour-0 increment: rate(20 + 0) is the high rate,
    so it is to be hospitalized).  With occupy_hospital, agents 1..5 fill the five cells."""
    cfg = make_config(n=10, grid=50, starting=(0, 0, 0, 0))
    p = oracle_mod.params_from_config(cfg)
    sim = oracle_mod.O1(p)
    recs = sim.export()
    assert sim.geography().hospital.tuple() == (40, 0, 44, 0)
    recs["immunity"][0] = 0
    recs["state"][0] = 5  # Infected-Severe
    recs["infection_day"][0] = 19
    if occupy_hospital:
        for k, (x, y) in enumerate([(40, 0), (41, 0), (42, 0), (43, 0), (44, 0)], start=1):
            recs["x"][k], recs["y"][k] = x, y
    return p, recs
