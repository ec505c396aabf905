"""GPU parity: the sm_103a engine tick against the CPU oracle (O1), bit for bit.

Every test drives the engine through the C ABI (include/epi_engine.h via ctypes) and the
oracle from the same world, and compares the hourly counts and the full agent snapshots
(positions, states, timers, flags, current areas).  Integer work: the bar is exact equality.
"""
import json

import numpy as np
import pytest

from helpers import COVID_FAST, diff_records, golden, hospital_world, make_config, rows_to_array

pytestmark = pytest.mark.gpu

S, E, I_PRE, I_ASYM, I_MILD, I_SEVERE, R, D = range(8)


def _engine(cfg, records=None):
    from epirust_gb300 import Config, Epidemiology

    return Epidemiology(Config(json.dumps(cfg)), records=records)


def _oracle(oracle_mod, cfg, records=None):
    return oracle_mod.O1(oracle_mod.params_from_config(cfg), records)


def _assert_same_agents(eng, sim, where=""):
    a, b = eng.snapshot(), sim.export()
    assert (a.view(np.uint8) == b.view(np.uint8)).all(), f"{where}: " + diff_records(a, b)


def _engine_rows(rows):
    return np.stack([rows[k] for k in rows.dtype.names], axis=1).astype(np.int64)


TICK_CASES = {
    "small_pox": make_config(n=3000, grid=120, hours=24 * 30, seed=1, starting=(0, 0, 0, 20)),
    "covid_fast": make_config(n=3000, grid=120, hours=24 * 20, seed=2, disease=COVID_FAST, starting=(5, 5, 5, 20)),
    "dense": make_config(n=5500, grid=120, hours=24 * 12, seed=3, disease=COVID_FAST, starting=(0, 0, 10, 30),
                         pt=0.6, working=0.9),
}


@pytest.mark.parametrize("name", sorted(TICK_CASES))
def test_tick_parity_hour_by_hour(gpu, oracle_mod, name):
    """Many days of ticks without interventions: counts every hour, agents every day."""
    cfg = TICK_CASES[name]
    eng, sim = _engine(cfg), _oracle(oracle_mod, cfg)
    _assert_same_agents(eng, sim, "world")
    hour, peak = 1, 0
    while hour < cfg["hours"]:
        end = min(((hour - 1) // 24 + 1) * 24, cfg["hours"] - 1)  # day segments 1..24, 25..48, ...
        n = end - hour + 1
        got = _engine_rows(eng.simulate_hours(hour, n))
        want = rows_to_array(sim.run(hour, hour + n, interventions=False, stop=False))
        assert (got == want).all(), f"hours {hour}..{hour + n - 1}: first diff row " \
            f"{np.nonzero((got != want).any(axis=1))[0][:1]}: {got[(got != want).any(axis=1)][:1]} vs " \
            f"{want[(got != want).any(axis=1)][:1]}"
        _assert_same_agents(eng, sim, f"after hour {hour + n - 1}")
        peak = max(peak, int(want[:, 3].max()))
        hour += n
    eng.check_invariants()
    assert peak > 0  # the epidemic actually ran through the state machine


def test_single_hour_api(gpu, oracle_mod):
    """epi_engine_simulate (one hour per call) == oracle, across a day boundary."""
    cfg = make_config(n=2000, grid=100, seed=9, disease=COVID_FAST, starting=(2, 2, 2, 10))
    eng, sim = _engine(cfg), _oracle(oracle_mod, cfg)
    for hour in range(1, 60):
        c = eng.simulate(hour)
        want = sim.simulate(hour)
        got = np.array([c.susceptible, c.exposed, c.infected, c.hospitalized, c.recovered, c.deceased])
        assert c.hour == hour and (got == want).all(), hour
    _assert_same_agents(eng, sim)


def test_claim_windows_and_rewinds(gpu, oracle_mod):
    """Claim keys carry the hour mod 128: segments that straddle window starts (hours 128, 256,
    384), single hours, a restore to an earlier hour and an hour run out of order all equal the
    oracle."""
    cfg = make_config(n=4000, grid=110, seed=21, disease=COVID_FAST, starting=(3, 3, 3, 25))
    eng, sim = _engine(cfg), _oracle(oracle_mod, cfg)

    def step(first, n):
        got = _engine_rows(eng.simulate_hours(first, n))
        want = rows_to_array(sim.run(first, first + n, False, False))
        assert (got == want).all(), f"hours {first}..{first + n - 1}"

    step(1, 100)
    step(101, 57)                  # crosses 128
    for hour in range(158, 262):   # single hours across 256
        step(hour, 1)
    eng.save_state()
    ref = sim.export()
    step(262, 300)                 # crosses 384 and 512
    eng.restore_state()            # rewind to hour 262 with claims of hour 561 left behind
    sim = oracle_mod.O1(oracle_mod.params_from_config(cfg), ref)
    step(262, 140)
    step(395, 30)                  # overlaps hours 395..401 already run
    step(390, 20)                  # back 35 hours, into the window of the stale keys
    _assert_same_agents(eng, sim, "after rewinds")
    eng.check_invariants()


def test_interventions_bulk_ops(gpu, oracle_mod):
    """lock / unlock / vaccinate / grow hospital as bulk device ops == oracle."""
    cfg = make_config(n=4000, grid=120, seed=4, disease=COVID_FAST, starting=(0, 0, 0, 40),
                      interventions=[{"Lockdown": {"at_number_of_infections": 10, "essential_workers_population": 0.2}}])
    eng, sim = _engine(cfg), _oracle(oracle_mod, cfg)
    eng.simulate_hours(1, 30)
    sim.run(1, 31, False, False)
    eng.lock_city(); sim.lock_city()
    _assert_same_agents(eng, sim, "locked")
    eng.simulate_hours(31, 40)
    sim.run(31, 71, False, False)
    _assert_same_agents(eng, sim, "locked run")
    eng.vaccinate(71, 0.35); sim.vaccinate(71, 0.35)
    _assert_same_agents(eng, sim, "vaccinated")
    eng.unlock_city(); sim.unlock_city()
    eng.increase_hospital_size(); sim.increase_hospital_size()
    assert eng.geography().hospital.tuple() == sim.geography().hospital.tuple()
    got = _engine_rows(eng.simulate_hours(71, 100))
    want = rows_to_array(sim.run(71, 171, False, False))
    assert (got == want).all()
    _assert_same_agents(eng, sim, "after growth")
    eng.check_invariants()


RUN_CASES = {
    "lockdown_vaccinate": make_config(
        n=5000, grid=120, hours=24 * 40, seed=5, disease=COVID_FAST, starting=(0, 0, 0, 30),
        interventions=[{"Lockdown": {"at_number_of_infections": 20, "essential_workers_population": 0.1}},
                       {"Vaccinate": {"at_hour": 100, "percent": 0.3}},
                       {"Vaccinate": {"at_hour": 333, "percent": 0.5}}]),
    "spread_hospital": make_config(
        n=5000, grid=120, hours=24 * 40, seed=6, disease=COVID_FAST, starting=(0, 0, 10, 30),
        interventions=[{"BuildNewHospital": {"spread_rate_threshold": 5}}]),
    "occupancy_hospital": make_config(
        n=5500, grid=120, hours=24 * 40, seed=7, starting=(0, 0, 30, 30), occupancy=0.7,
        interventions=[{"Lockdown": {"at_number_of_infections": 100, "essential_workers_population": 0.1}}]),
    "stop_early": make_config(n=800, grid=100, hours=24 * 60, seed=8, starting=(0, 0, 0, 1)),
}


@pytest.mark.parametrize("name", sorted(RUN_CASES))
def test_run_loop_parity(gpu, oracle_mod, name):
    """epi_engine_run (segments, interventions, stop rule) == oracle's run_single_engine."""
    cfg = RUN_CASES[name]
    eng, sim = _engine(cfg), _oracle(oracle_mod, cfg)
    got = _engine_rows(eng.run())
    want = rows_to_array(sim.run(1, cfg["hours"], interventions=True, stop=True))
    assert got.shape == want.shape, (got.shape, want.shape)
    assert (got == want).all(), np.nonzero((got != want).any(axis=1))[0][:3]
    # the final state matches too, also after an early stop (hours after it change nothing)
    _assert_same_agents(eng, sim, "end of run")
    eng.check_invariants()


def test_small_pox_10k_full_run_parity(gpu, oracle_mod):
    """The 10k-agent / 250-grid small-pox run (2,400 h): every hourly row equal."""
    cfg = golden("small_pox_10k_250.json")
    eng, sim = _engine(cfg), _oracle(oracle_mod, cfg)
    got = _engine_rows(eng.run())
    want = rows_to_array(sim.run(1, cfg["hours"], interventions=True, stop=True))
    assert got.shape == want.shape and (got == want).all()
    assert want[:, 3].max() > 0  # the epidemic took off


def test_hospital_known_answers_on_gpu(gpu, oracle_mod):
    """allocation_map.rs:444-495 on the device: first vacant hospital cell / full -> home."""
    for occupied in (False, True):
        p, recs = hospital_world(oracle_mod, occupy_hospital=occupied)
        cfg = make_config(n=10, grid=50, starting=(0, 0, 0, 0))
        eng = _engine(cfg, records=recs)
        sim = oracle_mod.O1(p, recs)
        eng.simulate(24)
        sim.simulate(24)
        _assert_same_agents(eng, sim)
        r = eng.snapshot()[0]
        if occupied:
            assert not (r["flags"] & 1)
        else:
            assert (r["x"], r["y"]) == (40, 0) and r["flags"] & 1


def test_contested_hospital_cell_losers_stay_hospitalized(gpu, oracle_mod):
    """Several severe agents on one hour 0 target the same first vacant cell: the lowest index
    moves in, the others stay put but are flagged hospitalized (citizen/mod.rs:359-363)."""
    cfg = make_config(n=30, grid=50, starting=(0, 0, 0, 0))
    p = oracle_mod.params_from_config(cfg)
    recs = oracle_mod.O1(p).export()
    for k in (3, 7, 11):
        recs["state"][k], recs["infection_day"][k], recs["immunity"][k] = I_SEVERE, 19, 0
    eng, sim = _engine(cfg, records=recs), oracle_mod.O1(p, recs)
    eng.simulate(48)
    sim.simulate(48)
    _assert_same_agents(eng, sim)
    out = eng.snapshot()
    assert (out["x"][3], out["y"][3]) == (40, 0)
    assert all(out["flags"][k] & 1 for k in (3, 7, 11))
    assert (out["x"][7], out["y"][7]) == (recs["x"][7], recs["y"][7])


def test_records_roundtrip(gpu, oracle_mod):
    """A mid-epidemic oracle state loaded into the engine continues identically."""
    cfg = make_config(n=3000, grid=120, seed=12, disease=COVID_FAST, starting=(10, 10, 10, 30),
                      interventions=[{"Lockdown": {"at_number_of_infections": 0, "essential_workers_population": 0.3}}])
    sim = _oracle(oracle_mod, cfg)
    sim.run(1, 200, interventions=False, stop=False)
    sim.lock_city()
    mid = sim.export()
    eng = _engine(cfg, records=mid)
    _assert_same_agents(eng, sim, "loaded")
    sim2 = oracle_mod.O1(oracle_mod.params_from_config(cfg), mid)
    got = _engine_rows(eng.simulate_hours(200, 50))
    want = rows_to_array(sim2.run(200, 250, False, False))
    assert (got == want).all()
    _assert_same_agents(eng, sim2, "continued")


def test_bad_records_are_refused(gpu, oracle_mod):
    """Records are checked where they are packed, on the device: a field out of range or a
    current area that is none of the agent's areas refuses the engine with EPI_ERR_ARG, and
    the message names the first bad record in index order.  Good records still load."""
    from epirust_gb300 import _lib

    cfg = make_config(n=3000, grid=120, seed=12, disease=COVID_FAST, starting=(10, 10, 10, 30))
    good = _oracle(oracle_mod, cfg).export()
    G = cfg["geography_parameters"]["grid_size"]
    worker = int(np.flatnonzero(good["work_status"] != 3)[0])

    def refused(edit):
        recs = good.copy()
        edit(recs)
        with pytest.raises(_lib.EpiError) as e:
            _engine(cfg, records=recs)
        assert e.value.code == 6
        return str(e.value)

    def set_(field, k, v):
        return lambda r: r[field].__setitem__(k, v)

    assert "agent record 17 out of range" in refused(set_("x", 17, G + 1))
    assert "agent record 3 out of range" in refused(set_("immunity", 3, 3))
    assert "agent record 40 out of range" in refused(set_("state", 40, 8))
    assert "agent record 2999 out of range" in refused(set_("home_y", 2999, G))
    assert f"agent record {worker} out of range" in refused(set_("work_x", worker, G - 5))

    def shift_area(k):
        def edit(r):
            r["area_x0"][k] += 1
            r["area_x1"][k] += 1
        return edit

    msg = refused(shift_area(5))
    assert "replicate 0: agent record 5: current area is not one of its areas" in msg

    def two(r):  # the lower index is reported, whatever its kind
        shift_area(9)(r)
        r["y"][30] = -1
    assert "agent record 9: current area" in refused(two)

    def two_b(r):
        shift_area(31)(r)
        r["y"][30] = -1
    assert "agent record 30 out of range" in refused(two_b)

    eng = _engine(cfg, records=good)
    _assert_same_agents(eng, _oracle(oracle_mod, cfg), "loaded")


def test_full_size_world_first_day_parity(gpu, oracle_mod):
    """The 1M-agent / 2,500-grid world: the first 30 hours equal the oracle."""
    cfg = golden("small_pox_1m_2500.json")
    eng, sim = _engine(cfg), _oracle(oracle_mod, cfg)
    got = _engine_rows(eng.simulate_hours(1, 30))
    want = rows_to_array(sim.run(1, 31, interventions=False, stop=False))
    assert (got == want).all()
    _assert_same_agents(eng, sim, "1M after 30 h")
    eng.check_invariants()


def test_full_size_run_properties(gpu):
    """The 1M-agent / 2,500-grid run end to end: invariants that hold whatever the trajectory."""
    cfg = golden("small_pox_1m_2500.json")
    eng = _engine(cfg)
    rows = eng.run()
    arr = _engine_rows(rows)
    assert (arr[:, 1:].sum(axis=1) == 1_000_000).all()         # every row accounts for everyone
    assert list(arr[:, 0]) == list(range(1, len(arr) + 1))      # consecutive hours from 1
    assert (np.diff(arr[:, 6]) >= 0).all()                      # deaths never decrease
    assert (np.diff(arr[:, 5] + arr[:, 6]) >= 0).all()          # removed never decreases
    eng.check_invariants()
    snap = eng.snapshot()
    cells = snap["x"].astype(np.int64) * 4096 + snap["y"]
    assert len(np.unique(cells)) == len(snap)                   # one agent per cell


def test_create_errors(gpu):
    from epirust_gb300 import EpiError

    with pytest.raises(EpiError, match="CAPACITY"):
        _engine(make_config(n=5000, grid=50))
    with pytest.raises(EpiError, match="CONFIG"):
        _engine(make_config(n=10, grid=30))


def test_profiling_counts_kernels(gpu):
    cfg = make_config(n=2000, grid=100, seed=3)
    eng = _engine(cfg)
    eng.set_profiling(True)
    before = eng.kernels_launched()  # the world build's kernels
    eng.simulate_hours(1, 24)
    stats = eng.kernel_stats()
    # hours 2..6 repeat hour 1 within a segment: one sleep launch per day
    assert stats["k_sleep"][0] == 1 and stats["k_decide"][0] == 18 and stats["k_commit"][0] == 18
    assert eng.kernels_launched() - before == 1 + 2 * 18 + 1  # and the piece end (k_piece_end)
    assert all(ms > 0 for launches, ms in stats.values() if launches)
