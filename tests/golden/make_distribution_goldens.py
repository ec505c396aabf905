"""Generate the reference-order-semantics sample for the distributional test of the default world.

TEST INFRASTRUCTURE ONLY: runs O2 (oracle/o2.c: FNV hash map keyed by cell, map phase over
the map, serial first-come resolve in hash order, swap -- the data flow of
engine/src/allocation_map.rs:67-129) on the CPU.  It never touches a GPU.

    python tests/golden/make_distribution_goldens.py   # ~5 CPU-minutes on 8 cores

o2_small_pox_10k_250_200.json
    The 10,000-agent / 250-grid small-pox run of small_pox_10k_250.json (2,400 hours, 5
    exposed, no interventions) under 200 seeds (5000 .. 5199): per seed the peak of active
    cases (exposed + infected + hospitalized), the day of that peak, the final attack rate
    and the number of rows before the stop rule ended the run.
"""
from __future__ import annotations

import json
import multiprocessing as mp
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

OUT = os.path.join(HERE, "o2_small_pox_10k_250_200.json")
SEEDS = range(5000, 5200)


def summary(rows, n: int) -> list:
    """[peak active cases, day of the peak, final attack rate, rows]."""
    import numpy as np

    active = rows["exposed"].astype(np.int64) + rows["infected"] + rows["hospitalized"]
    k = int(np.argmax(active))
    last = rows[-1]
    attack = (int(last["recovered"]) + int(last["deceased"]) + int(active[-1])) / n
    return [int(active[k]), int(rows["hour"][k]) // 24, attack, len(rows)]


def config_with_seed(seed: int) -> dict:
    with open(os.path.join(HERE, "small_pox_10k_250.json")) as f:
        cfg = json.load(f)
    cfg["seed"] = seed
    return cfg


def _o2_run(seed: int) -> list:
    from oracle import oracle

    cfg = config_with_seed(seed)
    params = oracle.params_from_config(cfg)
    records = oracle.O1(params).export()  # the world build (equal to the engine's, tested)
    sim = oracle.O2(params, records, threads=1)
    return summary(sim.run(1, int(cfg["hours"]), interventions=True, stop=True), len(records))


def main() -> None:
    from oracle import oracle

    oracle.build()
    t0 = time.time()
    with mp.get_context("spawn").Pool(os.cpu_count() or 1) as pool:
        runs = pool.map(_o2_run, list(SEEDS))
    out = {"config": "small_pox_10k_250.json", "seeds": [SEEDS.start, SEEDS.stop],
           "fields": ["peak_active", "peak_day", "attack_rate", "rows"], "runs": runs,
           "generator": "tests/golden/make_distribution_goldens.py (oracle O2)", "oracle_s": round(time.time() - t0, 1)}
    with open(OUT, "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print(f"wrote {OUT}: {len(runs)} runs in {out['oracle_s']} s")


if __name__ == "__main__":
    main()
