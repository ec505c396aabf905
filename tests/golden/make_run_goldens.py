"""Generate the end-to-end golden files of the benchmarked workloads with the CPU oracle O1.

TEST INFRASTRUCTURE ONLY: this script runs the scalar oracle (oracle/o1.c) and writes what
the GPU tests compare the engine with.  It never touches a GPU.

    python tests/golden/make_run_goldens.py run1m     # about 15 CPU-minutes
    python tests/golden/make_run_goldens.py fast1m    # about 4 CPU-minutes
    python tests/golden/make_run_goldens.py ensemble  # 8 replicates of the 256, in parallel

run_small_pox_1m_2500.json.gz
    The 1,000,000-agent / 2,500-grid run of small_pox_1m_2500.json (4,800 hours, lockdown at
    1,000 infections, vaccination of 20 % of the susceptible at hour 2,400, hospital build at
    70 % occupancy) through run_single_engine
    (engine/src/epidemiology_simulation.rs:211-274): every hourly counts row, the
    intervention reports (hour, name, data; engine/src/interventions/intervention_reporter.rs:28-63)
    and the SHA-256 of the full agent records (the engine's snapshot layout) every
    CHECKPOINT hours and at the end.  (Small pox spreads slowly on this world: at most 129
    agents are infected at once, so of its interventions only the vaccination fires.)
run_fast_1m_2500.json.gz
    The same world and interventions with a fast disease (fast_1m_2500.json, 1,200 hours,
    vaccination at hour 600), on which the lockdown, the occupancy-triggered hospital build
    and the lockdown's lifting fire too; the same contents.
ensemble_sample_256.json.gz
    Eight replicates of the 256-replicate batched workload (epirust_gb300.workloads.
    ensemble_configs: populations log-uniform in [10k, 500k], 2,400 hours, no interventions):
    the largest, the smallest and six spread between them by population.  For each: its
    index, its config, every counts row and the SHA-256 of its final agent records.
"""
from __future__ import annotations

import gzip
import hashlib
import json
import multiprocessing as mp
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

RUNS = {"run1m": ("small_pox_1m_2500.json", os.path.join(HERE, "run_small_pox_1m_2500.json.gz"), 480),
        "fast1m": ("fast_1m_2500.json", os.path.join(HERE, "run_fast_1m_2500.json.gz"), 120)}
ENS_OUT = os.path.join(HERE, "ensemble_sample_256.json.gz")


def records_sha256(records) -> str:
    return hashlib.sha256(records.tobytes()).hexdigest()


def rows_list(rows) -> list[list[int]]:
    return [[int(r[k]) for k in rows.dtype.names] for r in rows]


def run_with_checkpoints(oracle, cfg: dict, checkpoint: int) -> dict:
    """run_single_engine in segments of `checkpoint` hours (the oracle's run loop keeps its
    intervention state across calls), hashing the agent records after each segment."""
    import numpy as np

    sim = oracle.O1(oracle.params_from_config(cfg))
    hours = int(cfg["hours"])
    rows, hashes = [], {}
    first = 1
    while first < hours:
        last = min(first + checkpoint, hours)
        part = sim.run(first, last, interventions=True, stop=True)
        rows.append(part)
        if len(part) < last - first:  # the stop rule ended the run
            break
        hashes[str(last - 1)] = records_sha256(sim.export())
        first = last
    allrows = np.concatenate(rows) if rows else np.zeros(0, dtype=oracle.ROW_DTYPE)
    return {"rows": rows_list(allrows), "checkpoint_sha256": hashes, "final_sha256": records_sha256(sim.export()),
            "reports": [list(r) for r in sim.reports()]}


def make_run(which: str) -> None:
    from oracle import oracle

    oracle.build()
    config, path, checkpoint = RUNS[which]
    with open(os.path.join(HERE, config)) as f:
        cfg = json.load(f)
    t0 = time.time()
    out = run_with_checkpoints(oracle, cfg, checkpoint)
    out["config"] = config
    out["generator"] = f"tests/golden/make_run_goldens.py {which} (oracle O1)"
    out["oracle_s"] = round(time.time() - t0, 1)
    with gzip.open(path, "wt") as f:
        json.dump(out, f, separators=(",", ":"))
    print(f"wrote {path}: {len(out['rows'])} rows, {len(out['reports'])} reports, {out['oracle_s']} s")


def sample_indices(configs: list[dict], k: int = 8) -> list[int]:
    """The largest and smallest replicate and k - 2 spread between them by population."""
    order = sorted(range(len(configs)), key=lambda r: configs[r]["population"]["Auto"]["number_of_agents"])
    picks = [order[round(q * (len(order) - 1) / (k - 1))] for q in range(k)]
    return sorted(set(picks))


def _one_replicate(args) -> dict:
    r, cfg = args
    from oracle import oracle

    t0 = time.time()
    sim = oracle.O1(oracle.params_from_config(cfg))
    rows = sim.run(1, int(cfg["hours"]), interventions=True, stop=True)
    return {"index": r, "config": cfg, "rows": rows_list(rows), "final_sha256": records_sha256(sim.export()),
            "oracle_s": round(time.time() - t0, 1)}


def make_ensemble() -> None:
    from epirust_gb300.workloads import ensemble_configs
    from oracle import oracle

    oracle.build()
    configs = ensemble_configs()
    picks = sample_indices(configs)
    with mp.get_context("spawn").Pool(min(len(picks), os.cpu_count() or 1)) as pool:
        reps = pool.map(_one_replicate, [(r, configs[r]) for r in picks])
    out = {"replicates": len(configs), "sample": reps,
           "generator": "tests/golden/make_run_goldens.py ensemble (oracle O1)"}
    with gzip.open(ENS_OUT, "wt") as f:
        json.dump(out, f, separators=(",", ":"))
    print(f"wrote {ENS_OUT}: replicates {picks}")


if __name__ == "__main__":
    what = sys.argv[1] if len(sys.argv) > 1 else "all"
    for which in RUNS:
        if what in (which, "all"):
            make_run(which)
    if what in ("ensemble", "all"):
        make_ensemble()
