"""The benchmarked workloads end to end against golden files that the CPU oracle O1 wrote
(tests/golden/make_run_goldens.py): bit for bit.

* The 1,000,000-agent / 2,500-grid run of small_pox_1m_2500.json through the run loop
  (run_single_engine, engine/src/epidemiology_simulation.rs:211-274; interventions of
  engine/src/allocation_map.rs:306-387): every one of its 4,799 hourly counts rows, the hours
  and kinds of the interventions that fired, and the SHA-256 of all agent records every 480
  hours and at the end.  Small pox stays small on this world (at most 129 agents infected at
  once), so of its interventions only the vaccination at hour 2,400 fires.
* The same world with a fast disease (fast_1m_2500.json, 1,200 hours), on which the lockdown
  at 1,000 infections, the occupancy-triggered hospital build, the vaccination and the
  lockdown's lifting all fire at 1M-agent scale; records hashed every 120 hours.
* Eight replicates of the 256-replicate batched workload, run inside the full ensemble (30.6M
  agents, 2,400 hours): every counts row and the SHA-256 of the final records of each.

The CPU side of these files takes minutes of oracle time, so it is generated once and
committed; the non-GPU tests below check that the files are complete and consistent.
"""
import gzip
import hashlib
import json
import os

import numpy as np
import pytest

from helpers import GOLDEN, golden, rows_to_array

RUNS = {"small_pox_1m": os.path.join(GOLDEN, "run_small_pox_1m_2500.json.gz"),
        "fast_1m": os.path.join(GOLDEN, "run_fast_1m_2500.json.gz")}
# the interventions each pinned run must exercise (kind -> hours, None = any)
EXPECTED = {"small_pox_1m": {"vaccination": [2400]},
            "fast_1m": {"vaccination": [600], "lockdown": None, "build_new_hospital": None}}
ENS = os.path.join(GOLDEN, "ensemble_sample_256.json.gz")


def _load(path):
    with gzip.open(path, "rt") as f:
        return json.load(f)


def _sha(records) -> str:
    return hashlib.sha256(records.tobytes()).hexdigest()


@pytest.mark.parametrize("name", sorted(RUNS))
def test_run_golden_is_complete(name):
    g = _load(RUNS[name])
    cfg = golden(g["config"])
    rows = np.array(g["rows"], dtype=np.int64)
    assert list(rows[:, 0]) == list(range(1, len(rows) + 1))
    assert (rows[:, 1:].sum(axis=1) == cfg["population"]["Auto"]["number_of_agents"]).all()
    for kind, hours in EXPECTED[name].items():
        fired = [r[0] for r in g["reports"] if r[1] == kind]
        assert fired and (hours is None or fired == hours), (kind, fired)
    assert len(g["checkpoint_sha256"]) >= 5


def test_ensemble_golden_is_complete():
    from epirust_gb300.workloads import ensemble_configs

    g = _load(ENS)
    configs = ensemble_configs()
    assert g["replicates"] == len(configs) == 256
    sizes = [c["population"]["Auto"]["number_of_agents"] for c in configs]
    picked = [s["index"] for s in g["sample"]]
    assert len(picked) == 8 and sizes.index(max(sizes)) in picked and sizes.index(min(sizes)) in picked
    for s in g["sample"]:
        assert s["config"] == configs[s["index"]]  # the generator saw today's workload
        rows = np.array(s["rows"], dtype=np.int64)
        assert (rows[:, 1:].sum(axis=1) == sizes[s["index"]]).all()


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(RUNS))
def test_run_equals_oracle_golden(gpu, name):
    """epi_engine_run over a 1M-agent world == O1: every row, every intervention, the agent
    records at every checkpoint and at the end."""
    import tempfile

    from epirust_gb300 import Config, Epidemiology

    g = _load(RUNS[name])
    cfg = golden(g["config"])
    want = np.array(g["rows"], dtype=np.int64)
    eng = Epidemiology(Config(json.dumps(cfg)))
    last = int(cfg["hours"]) - 1
    for hour in sorted(g["checkpoint_sha256"], key=int):
        rows, nxt = eng.run_until(int(hour))
        assert nxt == (int(hour) + 1 if int(hour) < last else 0)  # 0: the run has ended
        got = rows_to_array(rows)
        assert (got == want[: len(got)]).all(), f"rows differ before hour {hour}"
        assert _sha(eng.snapshot()) == g["checkpoint_sha256"][hour], f"agent records differ at hour {hour}"
    if nxt:  # the run continues past the last checkpoint (after it ends, run() would start over)
        rows = eng.run()
    got = rows_to_array(rows)
    assert got.shape == want.shape, (got.shape, want.shape)
    bad = np.nonzero((got != want).any(axis=1))[0]
    assert len(bad) == 0, f"first differing hour {bad[0] + 1}: {got[bad[0]]} vs {want[bad[0]]}"
    assert _sha(eng.snapshot()) == g["final_sha256"]
    with tempfile.TemporaryDirectory() as d:
        eng.write_outputs(d, "1m")
        out = os.path.join(d, "output")
        fname = [f for f in os.listdir(out) if f.endswith("_interventions.json")][0]
        with open(os.path.join(out, fname)) as f:
            reports = json.load(f)
    assert [(r["hour"], r["intervention"], json.dumps(r["data"], separators=(",", ":"))) for r in reports] == \
        [tuple(r) for r in g["reports"]]
    eng.check_invariants()
    eng.close()


@pytest.mark.gpu
def test_ensemble_sample_equals_oracle_golden(gpu):
    """The full 256-replicate ensemble (one launch per kernel and hour for all replicates):
    the eight sampled replicates equal O1 row for row and record for record."""
    from epirust_gb300 import Ensemble
    from epirust_gb300.workloads import ensemble_params

    g = _load(ENS)
    ens = Ensemble(ensemble_params())
    rows = ens.run()
    for s in g["sample"]:
        r = s["index"]
        got = rows_to_array(rows[r])
        want = np.array(s["rows"], dtype=np.int64)
        assert got.shape == want.shape and (got == want).all(), f"replicate {r}"
        assert _sha(ens.snapshot(r)) == s["final_sha256"], f"replicate {r} final records"
    ens.check_invariants()
    ens.close()
