"""epi_tick_hour_noalloc: one hour on caller-owned device arrays, with no device allocation.

Callers whose device memory comes from their own fixed pool or arena, or that must stay out
of the driver's allocator on their hot path, cannot let the library call cudaMalloc.  These
tests pack a mid-epidemic world into device arrays they own (allocated here by torch), run
it hour after hour through the no-allocation entry point of the C ABI -- a whole day and
across the day boundary, so every hour class runs (the hospital scan of hour 0, the sleep
hours, the travel, work, noon, home and walking hours, the deaths and recoveries of hour
23), once with the original hospital and once after BuildNewHospital grew it -- and check
the counts and every agent word after every hour against the engine's regular entry point
(epi_engine_simulate) on the same world.  Integer state: the results must be identical.

The file is named to be collected last, so that a run stopping at the first failure has
already run every other test.
"""
import ctypes as C
import json

import numpy as np
import pytest

from helpers import COVID_FAST, make_config

pytestmark = pytest.mark.gpu

EPI_ERR_CAPACITY = 2
EPI_ERR_ARG = 6


def _rate_class(p, day):
    if p.regular_transmission_start_day < day <= p.high_transmission_start_day:
        return 1
    if p.high_transmission_start_day < day <= p.last_day:
        return 2
    return 0


def _area_codes(recs, geo, grown):
    """current_area rectangle -> area code of the packed state word."""
    a = np.stack([recs["area_x0"], recs["area_y0"], recs["area_x1"], recs["area_y1"]], axis=1)
    home = np.stack([recs["home_x"], recs["home_y"], recs["home_x"] + 1, recs["home_y"] + 1], axis=1)
    office = np.stack([recs["work_x"], recs["work_y"], recs["work_x"] + 9, recs["work_y"] + 9], axis=1)
    code = np.full(len(recs), -1, dtype=np.int64)
    for c, rect in ((5, grown), (4, geo.hospital.tuple()), (3, geo.housing.tuple()), (2, geo.transport.tuple())):
        code[(a == np.array(rect)).all(axis=1)] = c
    code[((a == office).all(axis=1)) & (recs["work_status"] != 3)] = 1
    code[(a == home).all(axis=1)] = 0
    assert (code >= 0).all()
    return code


def _pack(recs, p, geo, grown):
    G = p.grid_size
    x, y = recs["x"].astype(np.uint32), recs["y"].astype(np.uint32)
    pos = x | (y << 16)
    code = _area_codes(recs, geo, grown).astype(np.uint32)
    day = recs["infection_day"].astype(np.uint32)
    st0 = (recs["state"].astype(np.uint32) | (recs["flags"].astype(np.uint32) << 3) | (code << 8)
           | (recs["work_status"].astype(np.uint32) << 11) | ((recs["immunity"].astype(np.int32) + 2).astype(np.uint32) << 13)
           | (day << 16))
    state = np.stack([st0, recs["at_hour"].astype(np.uint32)], axis=1).reshape(-1)
    home = recs["home_x"].astype(np.uint32) | (recs["home_y"].astype(np.uint32) << 16)
    work = recs["work_x"].astype(np.uint32) | (recs["work_y"].astype(np.uint32) << 16)
    wsa = recs["work_start_at"].astype(np.uint32)
    plane = np.zeros((G + 3) * (G + 3) + 16, dtype=np.uint8)
    infected = (recs["state"] >= 2) & (recs["state"] <= 5)
    cls = np.ones(len(recs), dtype=np.uint8)
    for i in np.nonzero(infected & ((recs["flags"] & 1) == 0))[0]:
        d = (int(recs["infection_day"][i]) + int(recs["immunity"][i])) & 0xFFFFFFFF
        cls[i] = 1 + _rate_class(p, d)
    plane[(recs["y"].astype(np.int64) + 1) * (G + 3) + recs["x"] + 1] = cls
    return pos, state, home, work, wsa, plane


def _unpack(pos, state, wsa, like, geo, grown):
    """Packed words back to the record fields the engine's snapshot reports."""
    out = like.copy()
    st0, at = state.reshape(-1, 2)[:, 0], state.reshape(-1, 2)[:, 1]
    out["x"], out["y"] = pos & 0x7FFF, (pos >> 16) & 0x7FFF
    s = st0 & 7
    out["state"] = s
    out["flags"] = (st0 >> 3) & 31
    out["work_status"] = (st0 >> 11) & 3
    out["immunity"] = ((st0 >> 13) & 7).astype(np.int32) - 2
    infected = (s >= 2) & (s <= 5)
    out["infection_day"] = np.where(infected, st0 >> 16, 0)
    out["at_hour"] = np.where((s == 1) | (s == 2), at, 0)
    out["work_start_at"] = np.where(out["work_status"] == 2, wsa, 0)
    code = (st0 >> 8) & 7
    rects = {2: geo.transport.tuple(), 3: geo.housing.tuple(), 4: geo.hospital.tuple(), 5: grown}
    for field, k in (("area_x0", 0), ("area_y0", 1), ("area_x1", 2), ("area_y1", 3)):
        v = np.zeros(len(out), dtype=np.int64)
        hx, hy = out["home_x"].astype(np.int64), out["home_y"].astype(np.int64)
        wx, wy = out["work_x"].astype(np.int64), out["work_y"].astype(np.int64)
        v = np.where(code == 0, (hx, hy, hx + 1, hy + 1)[k], v)
        v = np.where(code == 1, (wx, wy, wx + 9, wy + 9)[k], v)
        for c, r in rects.items():
            v = np.where(code == c, r[k], v)
        out[field] = v
    return out


def _noalloc_against_engine(cfg, warm_hours, hours, grow_hospital):
    """Run `hours` through epi_tick_hour_noalloc and through epi_engine_simulate from the same
    world (the regular engine after `warm_hours`); compare counts and agents every hour."""
    import torch

    from epirust_gb300 import Config, Epidemiology, lib
    from epirust_gb300._lib import EpiGeography

    config = Config(json.dumps(cfg))
    p = config.params
    L = lib()
    geo = EpiGeography()
    assert L.epi_define_geography(p.grid_size, C.byref(geo)) == 0
    assert L.epi_resize_hospital(C.byref(geo), p.number_of_agents, 0.002, p.hospital_beds_percentage) == 0
    grown = (geo.hospital.x0, geo.hospital.y0, p.grid_size, p.grid_size)

    base = Epidemiology(config)
    base.simulate_hours(1, warm_hours)
    world = base.snapshot()
    base.close()

    ref = Epidemiology(config, records=world)
    if grow_hospital:
        ref.increase_hospital_size()
        assert ref.geography().hospital.x1 == p.grid_size

    dev = torch.device("cuda")
    # u32 words travel as int32 tensors (same bits)
    arrays = [torch.from_numpy(a.copy().view(np.int32) if a.dtype == np.uint32 else a.copy()).to(dev)
              for a in _pack(world, p, geo, grown)]
    pos, state, home, work, wsa, plane = arrays
    counts = torch.zeros(8, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    seen_states = set()
    for h in hours:
        want = ref.simulate(h)
        rc = L.epi_tick_hour_noalloc(C.byref(p), h, 1 if grow_hospital else 0, pos.data_ptr(), state.data_ptr(),
                                     home.data_ptr(), work.data_ptr(), wsa.data_ptr(), plane.data_ptr(),
                                     counts.data_ptr(), stream)
        assert rc == 0, L.epi_engine_last_error(None)
        got = counts.cpu().numpy().astype(np.int64)[:6]
        assert list(got) == [want.susceptible, want.exposed, want.infected, want.hospitalized, want.recovered,
                             want.deceased], h
        ref_agents = ref.snapshot()
        out = _unpack(pos.cpu().numpy().view(np.uint32), state.cpu().numpy().view(np.uint32),
                      wsa.cpu().numpy().view(np.uint32), world, geo, grown)
        for name in ref_agents.dtype.names:
            assert (out[name] == ref_agents[name]).all(), (h, name)
        seen_states.update(int(v) for v in np.unique(ref_agents["state"]))
        # the plane the caller owns reflects the new positions: one occupied byte per agent
        assert int((plane.cpu().numpy() != 0).sum()) == len(world), h
    ref.close()
    return ref_agents, seen_states


# hour of day 6 of day 7 through hour of day 1 of day 8: every hour class, in order, while
# agents are exposed, severe, hospitalised, recovering and dying
DAY_HOURS = tuple(range(24 * 7 + 6, 24 * 8 + 2))


def test_noalloc_hours_match_engine(gpu):
    """A whole day and the next day boundary, original hospital."""
    cfg = make_config(n=4000, grid=120, seed=21, disease=COVID_FAST, starting=(5, 5, 5, 30),
                      interventions=[{"Lockdown": {"at_number_of_infections": 10 ** 6,
                                                   "essential_workers_population": 0.2}}])
    agents, states = _noalloc_against_engine(cfg, DAY_HOURS[0] - 1, DAY_HOURS, grow_hospital=False)
    assert {1, 5, 6, 7}.issubset(states)         # exposed, severe, recovered and dead agents took part
    assert (agents["flags"] & 1).any()            # and someone is in hospital


def test_noalloc_hours_match_engine_grown_hospital(gpu):
    """The same day on a world whose hospital BuildNewHospital has grown (staff and patients
    compare their area with the grown rectangle)."""
    cfg = make_config(n=4000, grid=120, seed=22, disease=COVID_FAST, starting=(5, 5, 10, 30), beds=0.001)
    agents, states = _noalloc_against_engine(cfg, DAY_HOURS[0] - 1, DAY_HOURS, grow_hospital=True)
    assert (agents["flags"] & 1).any()


def test_noalloc_rejects_worlds_beyond_its_scratch(gpu):
    import torch

    from epirust_gb300 import Config, lib

    p = Config(json.dumps(make_config(n=1_000_000, grid=3500))).params
    t = torch.zeros(16, dtype=torch.int64, device="cuda")
    ptr = t.data_ptr()
    rc = lib().epi_tick_hour_noalloc(C.byref(p), 7, 0, ptr, ptr, ptr, ptr, ptr, ptr, ptr, None)
    assert rc == EPI_ERR_CAPACITY
    assert b"fixed maximum" in lib().epi_engine_last_error(None)
    # a plane that is not 4-byte aligned is refused before any device work
    small = Config(json.dumps(make_config(n=500, grid=60))).params
    rc = lib().epi_tick_hour_noalloc(C.byref(small), 7, 0, ptr, ptr, ptr, ptr, ptr, ptr + 1, ptr, None)
    assert rc == EPI_ERR_ARG
    assert b"4-byte aligned" in lib().epi_engine_last_error(None)
    # so are per-agent arrays and counts that are not 4-byte aligned
    for k in (0, 2, 3, 4, 6):
        args = [ptr] * 7
        args[k] = ptr + 2
        rc = lib().epi_tick_hour_noalloc(C.byref(small), 7, 0, *args, None)
        assert rc == EPI_ERR_ARG, k
        assert b"4-byte aligned" in lib().epi_engine_last_error(None)
