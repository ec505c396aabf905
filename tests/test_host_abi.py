"""CPU tests of the engine library: it loads, exports every declared symbol, its structs
match the Python layouts, and its host-side code (config parser, geography, disease rates,
world build) agrees with the reference's known answers and bit for bit with the oracle."""
import ctypes as C
import json
import os
import re
import subprocess

import numpy as np
import pytest

from helpers import COVID_FAST, SMALL_POX, diff_records, golden, make_config

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions(header="epi_engine.h"):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(epi_[a-z_]+)\s*\(", text)))


@pytest.mark.parametrize("header,exports", [("epi_engine.h", "EXPORTS"), ("epi_surrogate.h", "MLP_EXPORTS")])
def test_library_exports_every_declared_symbol(engine_built, header, exports):
    from epirust_gb300 import _lib

    L = C.CDLL(engine_built)
    declared = _declared_functions(header)
    assert len(declared) >= 10
    missing = [f for f in declared if not hasattr(L, f)]
    assert not missing, f"missing exports: {missing}"
    assert sorted(getattr(_lib, exports)) == declared
    nm = subprocess.run(["nm", "-D", "--defined-only", engine_built], capture_output=True, text=True).stdout
    for f in declared:
        assert re.search(rf"\bT {f}$", nm, flags=re.M), f


def test_struct_layouts_match(engine_built):
    from epirust_gb300 import _lib

    L = _lib.lib()
    assert L.epi_abi_struct_size(b"epi_params") == C.sizeof(_lib.EpiParams)
    assert L.epi_abi_struct_size(b"epi_agent_record") == _lib.AGENT_DTYPE.itemsize == 56
    assert L.epi_abi_struct_size(b"epi_counts") == C.sizeof(_lib.EpiCounts) == 28
    assert L.epi_abi_struct_size(b"epi_geography") == C.sizeof(_lib.EpiGeography)
    assert L.epi_abi_struct_size(b"epi_mlp_config") == C.sizeof(_lib.MlpConfig) == 48
    assert L.epi_abi_struct_size(b"nope") == 0
    assert (_lib.MlpConfig.members.offset, _lib.MlpConfig.seed.offset) == (36, 40)


def test_mlp_config_rejected_before_any_device_call(engine_built):
    """Invalid network shapes (and more than 64 members) fail with EPI_ERR_CONFIG on the host."""
    from epirust_gb300 import _lib

    L = _lib.lib()
    good = dict(in_dim=8, hidden=512, hidden_layers=3, out_dim=600, batch=256, lr=1e-3, beta1=0.9, beta2=0.999,
                eps=1e-8, members=5, seed=1)
    for bad in (dict(members=65), dict(hidden=100), dict(batch=200), dict(in_dim=65), dict(hidden_layers=0),
                dict(lr=0.0)):
        cfg = _lib.MlpConfig(**{**good, **bad})
        h = C.c_void_p()
        assert L.epi_mlp_create(C.byref(cfg), C.byref(h)) == 1, bad  # EPI_ERR_CONFIG
        assert not h.value


def test_config_parse_matches_reference_fixture(engine_built):
    # common/src/config/mod.rs:164-189
    from epirust_gb300 import Config

    p = Config(json.dumps(golden("auto_pop_config.json"))).params
    assert (p.number_of_agents, p.public_transport_percentage, p.working_percentage) == (10000, 0.2, 0.7)
    assert (p.regular_transmission_start_day, p.high_transmission_start_day, p.last_day) == (5, 20, 40)
    assert (p.asymptomatic_last_day, p.mild_infected_last_day) == (9, 12)
    assert (p.regular_transmission_rate, p.high_transmission_rate, p.death_rate) == (0.025, 0.25, 0.035)
    assert (p.percentage_asymptomatic_population, p.percentage_severe_infected_population) == (0.3, 0.3)
    assert (p.exposed_duration, p.pre_symptomatic_duration) == (48, 48)
    assert (p.grid_size, p.hospital_beds_percentage, p.hours) == (250, 0.003, 10000)
    assert (p.n_vaccinations, p.vaccination_at_hour[0], p.vaccination_percent[0]) == (1, 5000, 0.2)
    assert (p.infected_mild_asymptomatic, p.infected_mild_symptomatic, p.infected_severe, p.exposed) == (2, 3, 4, 5)
    assert not p.has_lockdown and not p.has_build_new_hospital


def test_config_parse_equals_oracle_parse(engine_built, oracle_mod):
    from epirust_gb300 import Config

    for cfg in (golden("small_pox_10k_250.json"), golden("small_pox_1m_2500.json"), golden("auto_pop_config.json")):
        a = Config(json.dumps(cfg)).params
        b = oracle_mod.params_from_config(cfg)
        assert bytes(a) == bytes(b)


def test_disease_overrides_are_accepted_and_unused(engine_built):
    """Config::disease_overrides (common/src/config/mod.rs:49) is parsed by the reference but
    read nowhere in the engine: a config carrying one gives the same parameters."""
    import ctypes as C

    from epirust_gb300 import Config

    cfg = make_config()
    with_override = dict(cfg)
    with_override["disease_overrides"] = [{"population_param": "age", "values": ["60-64", "65-69"],
                                           "disease": dict(cfg["disease"], death_rate=0.3)}]
    a, b = Config(json.dumps(cfg)).params, Config(json.dumps(with_override)).params
    assert C.string_at(C.addressof(a), C.sizeof(a)) == C.string_at(C.addressof(b), C.sizeof(b))


def test_config_defaults_and_errors(engine_built):
    from epirust_gb300 import Config, EpiError

    cfg = make_config()
    del cfg["starting_infections"]
    assert Config(json.dumps(cfg)).params.exposed == 1  # StartingInfections::default
    bad = make_config()
    bad["population"] = {"Csv": {"file": "/nonexistent/x.csv", "cols": []}}
    with pytest.raises(EpiError, match="population file"):
        Config(json.dumps(bad))
    bad = make_config()
    del bad["disease"]
    with pytest.raises(EpiError, match="disease"):
        Config(json.dumps(bad))
    bad = make_config()
    bad["disease"]["death_rate"] = 1.5
    with pytest.raises(EpiError, match="percentages"):
        Config(json.dumps(bad))
    with pytest.raises(EpiError):
        Config("{not json")
    with pytest.raises(EpiError, match="integer"):
        Config(json.dumps(make_config(hours=10)).replace('"hours": 10', '"hours": 10.5'))


def test_geography_known_answers(engine_built):
    from epirust_gb300 import _lib
    from epirust_gb300.engine import define_geography

    L = _lib.lib()
    g = define_geography(10)  # engine/src/geography/mod.rs:76-90
    assert (g.housing.tuple(), g.transport.tuple(), g.work.tuple(), g.hospital.tuple()) == \
        ((0, 0, 3, 10), (4, 0, 5, 10), (6, 0, 7, 10), (8, 0, 8, 10))
    g = define_geography(100)  # grid.rs:377-385
    assert L.epi_geography_increase_hospital_size(C.byref(g), 120) == 0
    assert g.hospital.tuple() == (80, 0, 120, 120)
    g = define_geography(100)  # grid.rs:405-421
    L.epi_resize_hospital(C.byref(g), 1000, 0.02, 0.01)
    assert g.hospital.tuple() == (80, 0, 89, 3)
    g = define_geography(100)
    L.epi_resize_hospital(C.byref(g), 50000, 0.02, 0.01)
    assert g.hospital.tuple() == (80, 0, 89, 100)


@pytest.mark.parametrize("G", [10, 46, 50, 99, 100, 250, 333, 790, 1768, 2500, 8924])
def test_geography_equals_oracle(engine_built, oracle_mod, G):
    from epirust_gb300.engine import define_geography

    a = define_geography(G)
    b = oracle_mod.define_geography(G)
    assert bytes(a) == bytes(b)


def test_disease_rates_known_answers(engine_built, oracle_mod):
    # common/src/disease/mod.rs:145-163
    from epirust_gb300 import Config, _lib

    L = _lib.lib()
    p = Config(json.dumps(make_config(disease=SMALL_POX))).params
    assert L.epi_disease_transmission_rate(C.byref(p), 12) == 0.05
    assert L.epi_disease_transmission_rate(C.byref(p), 22) == 0.5
    assert not L.epi_disease_is_to_be_hospitalized(C.byref(p), 12)
    assert L.epi_disease_is_to_be_hospitalized(C.byref(p), 22)
    for disease in (SMALL_POX, COVID_FAST):
        p = Config(json.dumps(make_config(disease=disease))).params
        q = oracle_mod.params_from_config(make_config(disease=disease))
        for d in list(range(0, 45)) + [0xFFFFFFFE, 0xFFFFFFFF]:
            assert L.epi_disease_transmission_rate(C.byref(p), d) == oracle_mod.transmission_rate(q, d)
            assert bool(L.epi_disease_is_to_be_hospitalized(C.byref(p), d)) == oracle_mod.is_to_be_hospitalized(q, d)


WORLDS = [
    make_config(n=20, grid=50, starting=(2, 3, 4, 5)),
    make_config(n=1000, grid=80, seed=3),
    make_config(n=5000, grid=120, seed=11, pt=0.9, working=0.95, starting=(3, 3, 3, 10),
                interventions=[{"Lockdown": {"at_number_of_infections": 5, "essential_workers_population": 0.3}}]),
    golden("small_pox_10k_250.json"),
    make_config(n=24000, grid=250, seed=2**40 + 17, starting=(0, 0, 0, 37)),
]


@pytest.mark.parametrize("k", range(len(WORLDS)))
def test_world_build_equals_oracle(engine_built, oracle_mod, k):
    """The product's host world build reproduces the oracle's world bit for bit."""
    from epirust_gb300 import Config
    from epirust_gb300.engine import world_build

    cfg = WORLDS[k]
    p = Config(json.dumps(cfg)).params
    recs, geo = world_build(p)
    sim = oracle_mod.O1(oracle_mod.params_from_config(cfg))
    ref = sim.export()
    assert recs.dtype.itemsize == ref.dtype.itemsize
    assert (recs.view(np.uint8) == ref.view(np.uint8)).all(), diff_records(recs, ref)
    assert bytes(geo) == bytes(sim.geography())


def test_world_build_full_size_properties(engine_built):
    """The 1M-agent / 2500-grid world: capacity, occupancy and the population mix."""
    from epirust_gb300 import Config
    from epirust_gb300.engine import world_build

    cfg = golden("small_pox_1m_2500.json")
    recs, geo = world_build(Config(json.dumps(cfg)).params)
    n = len(recs)
    assert n == 1_000_000
    cells = recs["x"].astype(np.int64) * 4096 + recs["y"]
    assert len(np.unique(cells)) == n  # one agent per cell
    assert geo.hospital.tuple() == (2000, 0, 2249, 20)  # beds = ceil(N*0.003 + N*0.002) = 5000 -> 5000/249
    assert (recs["state"] == 1).sum() == 50
    working = recs["work_status"] != 3
    assert abs(working.mean() - 0.7) < 0.005
    staff = recs["work_status"] == 2
    assert abs(staff.sum() / working.sum() - 0.002) < 0.0005
    ess = recs["work_status"] == 1
    assert abs(ess.sum() / (working.sum() - staff.sum()) - 0.1) < 0.005
    pt = (recs["flags"] & 16) != 0
    assert not pt[~working].any() and abs(pt[working].mean() - 0.2) < 0.005
    assert set(np.unique(recs["immunity"])) == {-2, -1, 0, 1, 2}


def test_world_build_errors(engine_built):
    from epirust_gb300 import Config, EpiError
    from epirust_gb300.engine import world_build

    with pytest.raises(EpiError, match="capacity"):
        world_build(Config(json.dumps(make_config(n=5000, grid=50))).params)
    with pytest.raises(EpiError, match="infect"):
        world_build(Config(json.dumps(make_config(n=10, grid=50, starting=(0, 0, 0, 11)))).params)
    with pytest.raises(EpiError, match="offices"):
        world_build(Config(json.dumps(make_config(n=10, grid=30))).params)
