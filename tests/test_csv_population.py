"""Population::Csv (engine/src/geography/grid.rs:194-231, citizen/population_record.rs): rows of
ind, age, working, pub_transport with True/False values; houses and offices are handed out
in cyclic order, working and public transport come from the row, the rest as in the Auto
build.  The device build equals the host build, and the engine runs it like any world."""
import json

import numpy as np
import pytest

from helpers import COVID_FAST, make_config


def _write_csv(path, n, seed=0, bad=None):
    rng = np.random.default_rng(seed)
    working = rng.random(n) < 0.6
    pt = rng.random(n) < 0.3
    lines = ["ind,age,working,pub_transport"]
    for i in range(n):
        lines.append(f"{i},{rng.integers(1, 90)},{'True' if working[i] else 'False'},{'True' if pt[i] else 'False'}")
    if bad is not None:
        lines[bad] = f"{bad},30,yes,False"
    path.write_text("\n".join(lines) + "\n")
    return working, pt


def _config(path, n_hours=24 * 5, **kw):
    cfg = make_config(n=1, grid=120, hours=n_hours, seed=21, disease=COVID_FAST, starting=(0, 0, 2, 10), **kw)
    cfg["population"] = {"Csv": {"file": str(path), "cols": ["ind", "age", "working", "pub_transport"]}}
    return cfg


def test_csv_rows_become_flags_and_records(engine_built, tmp_path):
    from epirust_gb300 import Config
    from epirust_gb300.engine import read_population_csv, world_build

    path = tmp_path / "pop.csv"
    working, pt = _write_csv(path, 3000, seed=1)
    flags = read_population_csv(str(path))
    assert len(flags) == 3000
    assert ((flags & 1) != 0).tolist() == working.tolist() and ((flags & 2) != 0).tolist() == pt.tolist()
    cfg = Config(json.dumps(_config(path)))
    assert cfg.params.population_source == 1 and cfg.number_of_agents == 3000
    recs, geo = world_build(cfg.params)
    ws = recs["work_status"]
    assert ((ws != 3) == working).all()                       # WS_NA = 3 exactly for non-workers
    assert (((recs["flags"] & 16) != 0) == pt).all()           # public transport as given
    houses = geo.houses_x * geo.houses_y
    hx = geo.housing.x0 + 2 * (np.arange(3000) % houses % geo.houses_x)
    assert (recs["home_x"] == hx).all()                        # houses cycled in order
    offices = geo.offices_x * geo.offices_y
    ox = geo.work.x0 + 10 * (np.arange(3000) % offices % geo.offices_x)
    assert (recs["work_x"] == ox).all()                        # offices cycled, also for non-workers
    assert ((recs["state"] != 0).sum()) == 12                  # starting infections


def test_csv_errors(engine_built, tmp_path):
    from epirust_gb300 import Config, EpiError

    path = tmp_path / "bad.csv"
    _write_csv(path, 50, bad=7)
    with pytest.raises(EpiError, match="True or False"):
        Config(json.dumps(_config(path)))
    nohead = tmp_path / "nohead.csv"
    nohead.write_text("ind,age\n0,4\n")
    with pytest.raises(EpiError, match="pub_transport"):
        Config(json.dumps(_config(nohead)))
    big = tmp_path / "big.csv"
    _write_csv(big, 4 * 3025 + 1)  # grid 120: more citizens than house cells
    cfg = _config(big)
    from epirust_gb300.engine import world_build

    with pytest.raises(EpiError, match="accommodate"):
        world_build(Config(json.dumps(cfg)).params)


@pytest.mark.gpu
def test_csv_world_on_the_device_and_run_parity(gpu, oracle_mod, tmp_path):
    from epirust_gb300 import Config, Epidemiology
    from epirust_gb300.engine import world_build
    from helpers import rows_to_array

    path = tmp_path / "pop.csv"
    _write_csv(path, 4000, seed=2)
    cfg = _config(path, interventions=[{"Lockdown": {"at_number_of_infections": 15,
                                                      "essential_workers_population": 0.2}}])
    config = Config(json.dumps(cfg))
    host, _ = world_build(config.params)
    eng = Epidemiology(config)
    assert (eng.snapshot().view(np.uint8) == host.view(np.uint8)).all()
    rows = eng.run()
    sim = oracle_mod.O1(oracle_mod.params_from_config(cfg | {"population": {"Auto": {
        "number_of_agents": 4000, "public_transport_percentage": 0.0, "working_percentage": 0.0}}}), host)
    want = rows_to_array(sim.run(1, cfg["hours"], interventions=True, stop=True))
    got = np.stack([rows[k] for k in rows.dtype.names], axis=1).astype(np.int64)
    assert got.shape == want.shape and (got == want).all()
    assert (eng.snapshot().view(np.uint8) == sim.export().view(np.uint8)).all()
    eng.close()
