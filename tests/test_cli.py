"""The standalone binary `epirust-gb300`, the drop-in for the reference's engine-app
(engine-app/src/main.rs:60-87): its flags, its refusals, and on a GPU its output files --
the hourly CSV of CsvListener (engine/src/listeners/csv_service.rs:44-71) equal to the CPU
oracle's rows, the interventions JSON, and the citizen-state stream when the config asks for
it (enable_citizen_state_messages, common/src/config/mod.rs:55)."""
import glob
import json
import os
import subprocess

import numpy as np
import pytest

from helpers import COVID_FAST, golden, make_config, rows_to_array


def _cli(engine_built):
    path = os.path.join(os.path.dirname(engine_built), "epirust-gb300")
    assert os.path.exists(path), path
    return path


def _run(cli, *args, timeout=600):
    return subprocess.run([cli, *args], capture_output=True, text=True, timeout=timeout)


def test_flags_and_refusals(engine_built, tmp_path):
    """Help, the multi-region modes that are out of scope, a missing or malformed config:
    each ends with a message and a non-zero status, before any device work."""
    cli = _cli(engine_built)
    r = _run(cli, "--help")
    assert r.returncode == 0 and "usage" in r.stderr
    for mode in ("kafka", "mpi"):
        r = _run(cli, "-m", mode)
        assert r.returncode == 2 and "not supported" in r.stderr
    r = _run(cli, "-c", str(tmp_path / "absent.json"))
    assert r.returncode == 1 and "Failed to read config file" in r.stderr
    bad = tmp_path / "bad.json"
    bad.write_text('{"population": 3}')
    r = _run(cli, "-c", str(bad))
    assert r.returncode == 1 and "Failed to read config file" in r.stderr
    r = _run(cli, "--bogus")
    assert r.returncode == 2


def _outputs(out_dir):
    files = sorted(glob.glob(os.path.join(out_dir, "output", "simulation_0_*")))
    csv = [f for f in files if f.endswith(".csv")]
    js = [f for f in files if f.endswith("_interventions.json")]
    assert len(csv) == 1 and len(js) == 1, files
    lines = open(csv[0]).read().splitlines()
    assert lines[0] == "hour,susceptible,exposed,infected,hospitalized,recovered,deceased"
    rows = np.array([[int(v) for v in ln.split(",")] for ln in lines[1:]], dtype=np.int64)
    with open(js[0]) as f:
        reports = json.load(f)
    return rows, reports


@pytest.mark.gpu
def test_default_world_run_equals_oracle(gpu, engine_built, oracle_mod, tmp_path):
    """The reference's default world (10,000 agents, 250 grid, small pox,
    2,400 hours) through the binary: every CSV row equals the oracle's."""
    cfg = golden("small_pox_10k_250.json")
    path = tmp_path / "config.json"
    path.write_text(json.dumps(cfg))
    r = _run(_cli(engine_built), "-c", str(path), "-o", str(tmp_path), "-t", "4")
    assert r.returncode == 0, r.stderr
    assert "Number of iterations" in r.stdout
    rows, reports = _outputs(str(tmp_path))
    sim = oracle_mod.O1(oracle_mod.params_from_config(cfg))
    want = rows_to_array(sim.run(1, cfg["hours"], interventions=True, stop=True))
    assert rows.shape == want.shape and (rows == want).all()
    assert reports == []


@pytest.mark.gpu
def test_interventions_and_citizen_states(gpu, engine_built, oracle_mod, tmp_path):
    """A run with a lockdown and a vaccination and the citizen-state messages switched on:
    the CSV and the interventions JSON equal the oracle's, and the stream's last record holds
    the oracle's final cells and state letters."""
    from epirust_gb300.state_stream import read_state_stream

    cfg = make_config(n=3000, grid=110, hours=24 * 8, seed=61, disease=COVID_FAST, starting=(0, 0, 5, 20),
                      interventions=[{"Lockdown": {"at_number_of_infections": 20, "essential_workers_population": 0.1}},
                                     {"Vaccinate": {"at_hour": 100, "percent": 0.3}}])
    cfg["enable_citizen_state_messages"] = True
    path = tmp_path / "config.json"
    path.write_text(json.dumps(cfg))
    r = _run(_cli(engine_built), "-c", str(path), "-o", str(tmp_path), "--seed", "61")
    assert r.returncode == 0, r.stderr
    rows, reports = _outputs(str(tmp_path))
    sim = oracle_mod.O1(oracle_mod.params_from_config(cfg))
    want = rows_to_array(sim.run(1, cfg["hours"], interventions=True, stop=True))
    assert rows.shape == want.shape and (rows == want).all()
    assert [(r["hour"], r["intervention"]) for r in reports] == [(h, k) for h, k, _ in sim.reports()]
    assert any(r["intervention"] == "lockdown" for r in reports)
    decoded = list(read_state_stream(str(tmp_path / "output" / "citizen_states_0.bin")))
    assert [h for h, *_ in decoded][1:] == [int(v) for v in rows[:, 0]]
    _, x, y, letters = decoded[-1]
    ref = sim.export()
    s = ref["state"].astype(np.int64)
    want_letters = np.select([s == 0, s == 1, s == 6, s == 7], [0, 1, 3, 4], default=2)
    assert (x == ref["x"]).all() and (y == ref["y"]).all() and (letters == want_letters).all()
