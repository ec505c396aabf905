"""The engine's own intervention triggers (process_interventions: lockdown, vaccination, hospital
build; engine/src/allocation_map.rs:306-337) on the host, without a device: the reference's
known-answer tests for engine/src/interventions/{lockdown,hospital,vaccination}.rs, the
oracle's triggers on random count sequences, and the run loop's device guard, which must mark
exactly the day-boundary rows at which a lockdown or a hospital build fires.  Also the
listeners' output files (CsvListener, InterventionReporter) for a run's rows."""
import json

import numpy as np
import pytest

from helpers import golden, make_config

LOCK, REVOKED, VACC, HOSP = 2, 4, 1, 8


def _params(cfg):
    from epirust_gb300 import Config

    return Config(json.dumps(cfg)).params


def _rows(*rows):
    """(hour, S, E, I, H, R, D) tuples as a counts array."""
    from epirust_gb300 import COUNTS_DTYPE

    return np.array([tuple(r) for r in rows], dtype=COUNTS_DTYPE)


def _replay(cfg, rows):
    from epirust_gb300.engine import interventions_replay

    return interventions_replay(_params(cfg), rows)


def _lockdown(threshold=20, essential=0.1, **kw):
    return make_config(n=100, grid=50, interventions=[{"Lockdown": {"at_number_of_infections": threshold,
                                                                    "essential_workers_population": essential}}], **kw)


def test_lockdown_applies_at_a_day_boundary_above_threshold(engine_built):
    # lockdown.rs:126-137 should_apply_lockdown_at_threshold; 140-148 not when locked down
    applied, guard = _replay(_lockdown(), _rows((0, 99, 0, 1, 0, 0, 0), (22, 80, 0, 20, 0, 0, 0),
                                                (28, 79, 0, 21, 0, 0, 0), (48, 79, 0, 21, 0, 0, 0),
                                                (72, 75, 0, 25, 0, 0, 0)))
    assert list(applied) == [0, 0, 0, LOCK, 0]
    assert list(guard) == [0, 0, 0, 1, 0]


def test_standalone_lockdown_lifts_at_hour_504(engine_built):
    # lockdown.rs:150-181: the lockdown lifts 21 days after zero_infection_hour, which a
    # standalone engine never sets (0): at hour 504 exactly, whatever the counts are
    rows = [(48, 79, 0, 21, 0, 0, 0)] + [(h, 79, 0, 21, 0, 0, 0) for h in (100, 480, 503)]
    rows += [(504, 79, 0, 21, 0, 0, 0), (505, 79, 0, 21, 0, 0, 0)]
    applied, guard = _replay(_lockdown(), _rows(*rows))
    assert list(applied) == [LOCK, 0, 0, 0, REVOKED, 0]
    assert list(guard) == [1, 0, 0, 0, 0, 0]  # the lift is a fixed event (chains end there), not a guard mark


def test_lockdown_after_the_lift(engine_built):
    # unapply (lockdown.rs:87-90) clears is_locked_down, so a later day boundary above the
    # threshold locks the city again; zero_infection_hour is 0 again, so that lockdown never lifts
    rows = [(24, 79, 0, 21, 0, 0, 0), (504, 80, 0, 20, 0, 0, 0), (528, 70, 0, 30, 0, 0, 0),
            (1032, 70, 0, 30, 0, 0, 0), (1056, 70, 0, 30, 0, 0, 0)]
    applied, guard = _replay(_lockdown(), _rows(*rows))
    assert list(applied) == [LOCK, REVOKED, LOCK, 0, 0]
    assert list(guard) == [1, 0, 1, 0, 0]


def test_hospital_build_at_threshold(engine_built):
    # hospital.rs:96-127: the day's new infections (infected minus the previous figure,
    # floored at 0) reach spread_rate_threshold at a day boundary
    cfg = make_config(n=100, grid=50, interventions=[{"BuildNewHospital": {"spread_rate_threshold": 10}}])
    applied, guard = _replay(cfg, _rows((0, 99, 1, 0, 0, 0, 0), (24, 80, 0, 20, 0, 0, 0), (48, 70, 0, 30, 0, 0, 0)))
    assert list(applied) == [0, HOSP, 0]  # built once
    assert list(guard) == [0, 1, 0]
    applied, guard = _replay(cfg, _rows((0, 99, 1, 0, 0, 0, 0), (24, 95, 0, 5, 0, 0, 0)))
    assert list(applied) == [0, 0] and list(guard) == [0, 0]
    applied, _ = _replay(make_config(n=100, grid=50), _rows((0, 99, 1, 0, 0, 0, 0), (24, 80, 0, 20, 0, 0, 0)))
    assert list(applied) == [0, 0]  # absent


def test_vaccination_only_at_its_hour(engine_built):
    # vaccination.rs:77-98 on the reference's auto_pop fixture: 20 % at hour 5000
    cfg = golden("auto_pop_config.json")
    applied, guard = _replay(cfg, _rows((4999, 10, 0, 10, 10, 10, 10), (5000, 10, 0, 10, 10, 10, 10),
                                        (5001, 10, 0, 10, 10, 10, 10)))
    assert list(applied & VACC) == [0, VACC, 0]
    assert not guard.any()


def _random_rows(rng, n_days, agents):
    """Hourly counts over n_days whose infected / hospitalized figures wander."""
    rows = []
    inf, hosp = int(rng.integers(0, agents // 50)), 0
    for h in range(1, 24 * n_days):
        inf = int(np.clip(inf + rng.integers(-3, 5), 0, agents // 2))
        hosp = int(np.clip(hosp + rng.integers(-1, 2), 0, inf))
        rows.append((h, agents - inf, 0, inf - hosp, hosp, 0, 0))
    return _rows(*rows)


@pytest.mark.parametrize("seed", range(6))
def test_engine_triggers_equal_the_oracle_and_the_guard(engine_built, oracle_mod, seed):
    """Random count sequences: the engine's host triggers fire at the same rows with the same
    bits as the oracle's, and the device guard marks a day-boundary row exactly when a
    lockdown or a hospital build fires there."""
    rng = np.random.default_rng(seed)
    n = 2000
    cfg = make_config(n=n, grid=110, occupancy=0.05 if seed % 2 else None, interventions=[
        {"Lockdown": {"at_number_of_infections": int(rng.integers(5, 60)), "essential_workers_population": 0.1}},
        {"BuildNewHospital": {"spread_rate_threshold": int(rng.integers(3, 40))}},
        {"Vaccinate": {"at_hour": int(rng.integers(1, 24 * 30)), "percent": 0.2}}])
    rows = _random_rows(rng, 40, n)
    applied, guard = _replay(cfg, rows)
    sim = oracle_mod.O1(oracle_mod.params_from_config(cfg))
    want = np.array([sim.process_interventions(int(r["hour"]), [int(r[k]) for k in rows.dtype.names[1:]])
                     for r in rows], dtype=np.uint32)
    assert (applied == want).all(), np.nonzero(applied != want)[0][:5]
    boundary = rows["hour"] % 24 == 0
    assert ((guard != 0) == (boundary & ((applied & (LOCK | HOSP)) != 0))).all()
    assert (applied & (LOCK | HOSP)).any()  # the sequences do exercise the triggers


def test_listener_files_for_a_run(engine_built, tmp_path):
    """CsvListener and InterventionReporter output for given rows: the file names of
    output_file_format (util.rs:36-43), the csv header and one line per row, and the report
    list serde writes (hour, intervention, data; compact JSON)."""
    import glob
    import os
    import re

    from epirust_gb300.engine import write_outputs_for_rows

    cfg = _lockdown(threshold=20)
    cfg["interventions"].append({"Vaccinate": {"at_hour": 30, "percent": 0.2}})
    rows = _rows(*[(h, 100 - min(h, 30), 0, min(h, 30), 0, 0, 0) for h in range(1, 50)])
    write_outputs_for_rows(str(tmp_path), "7", _params(cfg), rows)
    files = sorted(os.path.basename(f) for f in glob.glob(str(tmp_path / "output" / "*")))
    assert len(files) == 2
    stamp = r"\d{4}-\d\d-\d\dT\d\d:\d\d:\d\d"
    assert re.fullmatch(rf"simulation_7_{stamp}\.csv", files[0]), files
    assert re.fullmatch(rf"simulation_7_{stamp}_interventions\.json", files[1]), files
    lines = (tmp_path / "output" / files[0]).read_text().splitlines()
    assert lines[0] == "hour,susceptible,exposed,infected,hospitalized,recovered,deceased"
    assert lines[1:] == [",".join(str(int(v)) for v in r) for r in rows]
    reports = json.loads((tmp_path / "output" / files[1]).read_text())
    assert reports == [{"hour": 24, "intervention": "lockdown", "data": {"status": "locked_down"}},
                       {"hour": 30, "intervention": "vaccination", "data": {}}]
    text = (tmp_path / "output" / files[1]).read_text()
    assert text == json.dumps(reports, separators=(",", ":"))
