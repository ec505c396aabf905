"""The CPU oracle pinned against the reference's own known-answer unit tests.

Every expectation below is the assertion of a reference test (cited file:line in the
thoughtworks/epirust tree); the reference RNG is unseeded, so no reference test pins a
stochastic trajectory and these are all the fixed points there are.  Philox is pinned to the
published Random123 known-answer vectors.
"""
import numpy as np
import pytest

from helpers import SMALL_POX, golden, hospital_world, make_config

S, E, I_PRE, I_ASYM, I_MILD, I_SEVERE, R, D = range(8)


def test_philox2x32_known_answers(oracle_mod):
    # Salmon et al. SC'11 / Random123 kat_vectors, philox2x32 with 10 rounds
    assert oracle_mod.philox2x32([0, 0], 0) == [0xFF1DAE59, 0x6CD10DF2]
    assert oracle_mod.philox2x32([0xFFFFFFFF, 0xFFFFFFFF], 0xFFFFFFFF) == [0x2C3F628B, 0xAB4FD7AD]
    assert oracle_mod.philox2x32([0x243F6A88, 0x85A308D3], 0x13198A2E) == [0xDD7CE038, 0xF62A4C12]


def test_philox_known_answers(oracle_mod):
    # Salmon et al. SC'11 / Random123 kat_vectors, philox4x32 with 10 rounds
    assert oracle_mod.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert oracle_mod.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert oracle_mod.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_define_geography_grid_10(oracle_mod):
    # engine/src/geography/mod.rs:76-90
    g = oracle_mod.define_geography(10)
    assert g.housing.tuple() == (0, 0, 3, 10)
    assert g.transport.tuple() == (4, 0, 5, 10)
    assert g.work.tuple() == (6, 0, 7, 10)
    assert g.hospital.tuple() == (8, 0, 8, 10)


def test_increase_hospital_size(oracle_mod):
    # engine/src/geography/grid.rs:377-385
    g = oracle_mod.define_geography(100)
    oracle_mod.increase_hospital_size(g, 120)
    assert g.hospital.tuple() == (80, 0, 120, 120)


def test_resize_hospital(oracle_mod):
    # engine/src/geography/grid.rs:405-421
    g = oracle_mod.resize_hospital(oracle_mod.define_geography(100), 1000, 0.02, 0.01)
    assert g.hospital.tuple() == (80, 0, 89, 3)
    g = oracle_mod.resize_hospital(oracle_mod.define_geography(100), 50000, 0.02, 0.01)
    assert g.hospital.tuple() == (80, 0, 89, 100)


def test_small_pox_rates(oracle_mod):
    # common/src/disease/mod.rs:145-163
    p = oracle_mod.params_from_config(make_config(disease=SMALL_POX))
    assert oracle_mod.transmission_rate(p, 12) == 0.05
    assert oracle_mod.transmission_rate(p, 22) == 0.5
    assert not oracle_mod.is_to_be_hospitalized(p, 12)
    assert oracle_mod.is_to_be_hospitalized(p, 22)
    # the piecewise bounds: (10, 16] regular, (16, 22] high, else 0
    assert [oracle_mod.transmission_rate(p, d) for d in (10, 11, 16, 17, 22, 23)] == [0.0, 0.05, 0.05, 0.5, 0.5, 0.0]
    # (day + immunity) as u32 wraps for negative values: rate 0 (citizen/mod.rs:184)
    assert oracle_mod.transmission_rate(p, 0xFFFFFFFF) == 0.0


def test_area_neighbors_and_moore_order(oracle_mod):
    # engine/src/geography/area.rs:227-234
    nb = oracle_mod.area_neighbors((0, 0, 5, 5), (4, 5))
    assert len(nb) == 5 and (4, 4) in nb and (4, 6) not in nb
    # engine/src/geography/point.rs:84-101 (offset order)
    assert oracle_mod.area_neighbors((-10, -10, 10, 10), (1, 1)) == \
        [(0, 0), (1, 0), (2, 0), (0, 1), (2, 1), (0, 2), (1, 2), (2, 2)]


def test_area_iteration_order(oracle_mod):
    # engine/src/geography/area.rs:164-186
    assert oracle_mod.area_cells((0, 0, 2, 2)) == [(0, 0), (1, 0), (2, 0), (0, 1), (1, 1), (2, 1), (0, 2), (1, 2), (2, 2)]
    assert oracle_mod.area_cells((1, 1, 2, 2)) == [(1, 1), (2, 1), (1, 2), (2, 2)]


def test_area_factory(oracle_mod):
    # engine/src/geography/area.rs:198-225
    b = oracle_mod.area_factory((10, 0), (21, 10), 3)
    assert len(b) == 12
    assert b[0] == (10, 0, 12, 2)
    assert b[5] == (13, 3, 15, 5)
    assert b[-1] == (19, 6, 21, 8)


def test_starting_infection_split(oracle_mod):
    # engine/src/citizen/citizen_factory.rs:189-215: (asym, mild, severe, exposed) = (2, 3, 4, 5)
    cfg = make_config(n=20, grid=50, starting=(2, 3, 4, 5))
    recs = oracle_mod.O1(oracle_mod.params_from_config(cfg)).export()
    st = recs["state"]
    assert (st == I_ASYM).sum() == 2 and (st == I_MILD).sum() == 3
    assert (st == I_SEVERE).sum() == 4 and (st == E).sum() == 5
    # starting infected agents are on day 1, exposed at hour 0 (citizen_factory.rs:122-133, disease_state_machine.rs:109-121)
    assert set(recs["infection_day"][(st >= I_PRE) & (st <= I_SEVERE)]) == {1}
    assert set(recs["at_hour"][st == E]) == {0}


def test_generate_population_invariants(oracle_mod):
    # engine/src/geography/grid.rs:350-375 (10 agents on a 100 grid) and
    # citizen_factory.rs:172-187 (one exposed agent)
    cfg = make_config(n=10, grid=100, pt=0.2, working=0.2, starting=(0, 0, 0, 1))
    sim = oracle_mod.O1(oracle_mod.params_from_config(cfg))
    g = sim.geography()
    recs = sim.export()
    assert len(recs) == 10 and (recs["state"] == E).sum() == 1
    hx0, hy0, hx1, hy1 = g.housing.tuple()
    wx0, wy0, wx1, wy1 = g.work.tuple()
    for r in recs:
        assert hx0 <= r["home_x"] <= hx1 and hy0 <= r["home_y"] <= hy1
        working = r["work_status"] != 3
        if working:
            assert wx0 <= r["work_x"] + 9 <= wx1 and wy0 <= r["work_y"] + 9 <= wy1
        # every agent starts inside its own house
        assert r["home_x"] <= r["x"] <= r["home_x"] + 1 and r["home_y"] <= r["y"] <= r["home_y"] + 1


def test_config_parse_fixture(oracle_mod):
    # common/src/config/mod.rs:164-189 (config/test/auto_pop.json)
    p = oracle_mod.params_from_config(golden("auto_pop_config.json"))
    assert (p.number_of_agents, p.public_transport_percentage, p.working_percentage) == (10000, 0.2, 0.7)
    assert (p.regular_transmission_start_day, p.high_transmission_start_day, p.last_day) == (5, 20, 40)
    assert (p.regular_transmission_rate, p.high_transmission_rate, p.death_rate) == (0.025, 0.25, 0.035)
    assert (p.exposed_duration, p.pre_symptomatic_duration) == (48, 48)
    assert (p.grid_size, p.hospital_beds_percentage, p.hours) == (250, 0.003, 10000)
    assert (p.n_vaccinations, p.vaccination_at_hour[0], p.vaccination_percent[0]) == (1, 5000, 0.2)
    assert (p.infected_mild_asymptomatic, p.infected_mild_symptomatic, p.infected_severe, p.exposed) == (2, 3, 4, 5)


def _counts(hour, s, e, i, h, r, d):
    return [s, e, i, h, r, d]


def test_lockdown_triggers(oracle_mod):
    # engine/src/interventions/lockdown.rs:126-191 (at_number_of_infections 20)
    cfg = make_config(n=100, grid=50, interventions=[{"Lockdown": {"at_number_of_infections": 20,
                                                                   "essential_workers_population": 0.1}}])
    sim = oracle_mod.O1(oracle_mod.params_from_config(cfg))
    assert sim.process_interventions(0, _counts(0, 99, 0, 1, 0, 0, 0)) == 0
    assert sim.process_interventions(22, _counts(22, 80, 0, 20, 0, 0, 0)) == 0
    assert sim.process_interventions(28, _counts(28, 79, 0, 21, 0, 0, 0)) == 0
    assert sim.process_interventions(48, _counts(48, 79, 0, 21, 0, 0, 0)) == 2      # locked down
    assert sim.process_interventions(72, _counts(72, 75, 0, 25, 0, 0, 0)) == 0      # not re-applied
    for hr in (100, 480, 503):
        assert sim.process_interventions(hr, _counts(hr, 80, 0, 20, 0, 0, 0)) == 0
    # standalone: zero_infection_hour stays 0, so it lifts at 0 + 21 * 24
    assert sim.process_interventions(504, _counts(504, 80, 0, 20, 0, 0, 0)) == 4
    recs = sim.export()
    assert not (recs["flags"] & 2).any()  # nobody isolated after the unlock
    names = [r[1] for r in sim.reports()]
    assert names == ["lockdown", "lockdown"]


def test_lockdown_isolates_non_essential(oracle_mod):
    # allocation_map.rs:349-356: every non-essential agent is isolated
    cfg = make_config(n=400, grid=60, interventions=[{"Lockdown": {"at_number_of_infections": 0,
                                                                   "essential_workers_population": 0.5}}])
    sim = oracle_mod.O1(oracle_mod.params_from_config(cfg))
    sim.process_interventions(24, _counts(24, 399, 0, 1, 0, 0, 0))
    recs = sim.export()
    iso = (recs["flags"] & 2) != 0
    assert (iso == (recs["work_status"] != 1)).all()
    assert (recs["work_status"] == 1).sum() > 50  # ~half of the Normal workers became essential


def test_hospital_trigger(oracle_mod):
    # engine/src/interventions/hospital.rs:96-128 (spread_rate_threshold 10)
    cfg = make_config(n=100, grid=50, interventions=[{"BuildNewHospital": {"spread_rate_threshold": 10}}])
    sim = oracle_mod.O1(oracle_mod.params_from_config(cfg))
    assert sim.process_interventions(0, _counts(0, 99, 1, 0, 0, 0, 0)) == 0
    assert sim.process_interventions(24, _counts(24, 80, 0, 20, 0, 0, 0)) == 8
    assert sim.geography().hospital.tuple()[2:] == (50, 50)
    # already applied: never again (hospital.rs:153-160)
    assert sim.process_interventions(48, _counts(48, 50, 0, 50, 0, 0, 0)) == 0
    sim2 = oracle_mod.O1(oracle_mod.params_from_config(cfg))
    sim2.process_interventions(0, _counts(0, 99, 1, 0, 0, 0, 0))
    assert sim2.process_interventions(24, _counts(24, 95, 0, 5, 0, 0, 0)) == 0  # below threshold


def test_vaccination_only_at_its_hour(oracle_mod):
    # engine/src/interventions/vaccination.rs:88-98; allocation_map.rs:381-387
    cfg = make_config(n=2000, grid=100, interventions=[{"Vaccinate": {"at_hour": 5000, "percent": 0.2}}])
    sim = oracle_mod.O1(oracle_mod.params_from_config(cfg))
    assert sim.process_interventions(5001, _counts(5001, 1995, 5, 0, 0, 0, 0)) == 0
    assert sim.process_interventions(5000, _counts(5000, 1995, 5, 0, 0, 0, 0)) == 1
    recs = sim.export()
    vac = (recs["flags"] & 4) != 0
    assert not vac[recs["state"] != S].any()          # only susceptible agents
    frac = vac.sum() / (recs["state"] == S).sum()
    assert 0.17 < frac < 0.23


def test_goto_first_vacant_hospital_cell(oracle_mod):
    # allocation_map.rs:444-471: the first vacant cell in area order
    p, recs = hospital_world(oracle_mod, occupy_hospital=False)
    sim = oracle_mod.O1(p, recs)
    sim.simulate(24)
    out = sim.export()
    assert (out["x"][0], out["y"][0]) == (40, 0) and out["flags"][0] & 1


def test_full_hospital_sends_home(oracle_mod):
    # allocation_map.rs:473-495: hospital full -> a point of the home area, not hospitalized
    p, recs = hospital_world(oracle_mod, occupy_hospital=True)
    sim = oracle_mod.O1(p, recs)
    sim.simulate(24)
    out = sim.export()
    r = out[0]
    assert not (r["flags"] & 1)
    assert r["home_x"] <= r["x"] <= r["home_x"] + 1 and r["home_y"] <= r["y"] <= r["home_y"] + 1


def test_counts_total_and_stop_rule(oracle_mod):
    # allocation_map.rs:128 (total == population) and epidemiology_simulation.rs:564-575
    cfg = make_config(n=300, grid=50, hours=2000, starting=(0, 0, 0, 2))
    sim = oracle_mod.O1(oracle_mod.params_from_config(cfg))
    rows = sim.run(1, 2000)
    tot = rows["susceptible"].astype(int) + rows["exposed"] + rows["infected"] + rows["hospitalized"] + \
        rows["recovered"] + rows["deceased"]
    assert (tot == 300).all()
    assert list(rows["hour"]) == list(range(1, len(rows) + 1))
    last = rows[-1]
    if len(rows) < 1999:
        assert last["exposed"] == last["infected"] == last["hospitalized"] == 0
    active = rows["exposed"].astype(int) + rows["infected"] + rows["hospitalized"]
    assert (active[:-1] > 0).all()


def test_oracle_world_is_deterministic(oracle_mod):
    cfg = make_config(n=1000, grid=80, seed=5)
    a = oracle_mod.O1(oracle_mod.params_from_config(cfg)).export()
    b = oracle_mod.O1(oracle_mod.params_from_config(cfg)).export()
    assert (a == b).all()
    c = oracle_mod.O1(oracle_mod.params_from_config(make_config(n=1000, grid=80, seed=6))).export()
    assert not (a == c).all()


def test_capacity_errors(oracle_mod):
    # grid.rs:140-142 (more than 4 agents per house) and citizen_factory.rs:113-115
    with pytest.raises(oracle_mod.OracleError):
        oracle_mod.O1(oracle_mod.params_from_config(make_config(n=5000, grid=20)))
    with pytest.raises(oracle_mod.OracleError):
        oracle_mod.O1(oracle_mod.params_from_config(make_config(n=10, grid=50, starting=(0, 0, 0, 11))))
