"""Citizen-state stream: the per-hour (letter, cell) of every agent, encoded on the device
and decoded by epirust_gb300.state_stream, equals the CPU oracle O1's agents hour by hour;
the reference's message form (CitizenStatesAtHr, engine/src/models/events/citizen_state.rs:27-70)
is written from it with the same content."""
import json
import struct

import numpy as np
import pytest

from helpers import COVID_FAST, make_config


def _letters(records):
    s = records["state"].astype(np.int64)
    # S=0 E=1 I_pre..I_severe=2..5 R=6 D=7 -> s e i r d
    return np.select([s == 0, s == 1, s == 6, s == 7], [0, 1, 3, 4], default=2).astype(np.uint8)


def test_reader_decodes_steps_jumps_and_letters(tmp_path):
    from epirust_gb300.state_stream import LETTERS, read_state_stream

    p = tmp_path / "s.bin"
    with open(p, "wb") as f:
        f.write(struct.pack("<4I", 0x53435045, 1, 3, 50))
        f.write(struct.pack("<6H", 10, 10, 20, 20, 30, 30))
        f.write(bytes([0, 1, 2]))
        # hour 5: agent 0 steps to (-1, -1) = code 1, agent 1 stays, agent 2 jumps to (7, 8); letters e, i, r
        f.write(struct.pack("<3I", 5, 3, 1))
        f.write(bytes([1 | (1 << 4), 0 | (2 << 4), 15 | (3 << 4)]))
        f.write(struct.pack("<2I", 2, 7 | (8 << 16)))
        # hour 6: agent 1 steps to (+1, +1) = code 8
        f.write(struct.pack("<3I", 6, 3, 0))
        f.write(bytes([0 | (1 << 4), 8 | (2 << 4), 0 | (3 << 4)]))
    out = list(read_state_stream(str(p)))
    assert [h for h, *_ in out] == [0, 5, 6]
    _, x, y, l = out[1]
    assert list(x) == [9, 20, 7] and list(y) == [9, 20, 8] and "".join(LETTERS[v] for v in l) == "eir"
    _, x, y, l = out[2]
    assert list(x) == [9, 21, 7] and list(y) == [9, 21, 8]


def test_citizen_states_records_have_the_reference_shape(tmp_path):
    """write_citizen_states_json: one {"hr", "citizen_states": [{"citizen_id", "state",
    "location": {"x", "y"}}]} object per recorded hour, as serde_json writes CitizenStatesAtHr."""
    import uuid

    from epirust_gb300.state_stream import write_citizen_states_json

    p = tmp_path / "s.bin"
    with open(p, "wb") as f:
        f.write(struct.pack("<4I", 0x53435045, 1, 2, 50))
        f.write(struct.pack("<4H", 10, 10, 20, 20))
        f.write(bytes([0, 1]))
        f.write(struct.pack("<3I", 5, 2, 0))
        f.write(bytes([1 | (2 << 4), 0 | (4 << 4)]))
    out = tmp_path / "states.jsonl"
    assert write_citizen_states_json(str(p), str(out)) == 1
    rec = json.loads(out.read_text().splitlines()[0])
    assert list(rec) == ["hr", "citizen_states"] and rec["hr"] == 5
    a, b = rec["citizen_states"]
    assert list(a) == ["citizen_id", "state", "location"]
    assert (a["state"], a["location"]) == ("i", {"x": 9, "y": 9})
    assert (b["state"], b["location"]) == ("d", {"x": 20, "y": 20})
    assert uuid.UUID(a["citizen_id"]).version == 4 and a["citizen_id"] != b["citizen_id"]


@pytest.mark.gpu
def test_stream_equals_oracle_every_hour(gpu, oracle_mod, tmp_path):
    from epirust_gb300 import Config, Epidemiology
    from epirust_gb300.state_stream import LETTERS, read_state_stream, write_citizen_states_json

    cfg = make_config(n=4000, grid=120, hours=80, seed=51, disease=COVID_FAST, starting=(3, 3, 3, 30))
    eng = Epidemiology(Config(json.dumps(cfg)))
    path = tmp_path / "hourly.bin"
    eng.open_state_stream(str(path))
    for hour in range(1, 60):
        eng.simulate_hours(hour, 1)
    eng.close_state_stream()
    eng.close()
    sim = oracle_mod.O1(oracle_mod.params_from_config(cfg))
    want = [sim.export()]
    for hour in range(1, 60):
        sim.simulate(hour)
        want.append(sim.export())
    decoded = list(read_state_stream(str(path)))
    assert [h for h, *_ in decoded] == list(range(60))
    for (hour, x, y, letters), ref in zip(decoded, want):
        assert (x == ref["x"]).all() and (y == ref["y"]).all(), hour
        assert (letters == _letters(ref)).all(), hour

    # the reference's message form carries the same content, hour by hour
    jpath = tmp_path / "states.jsonl"
    assert write_citizen_states_json(str(path), str(jpath)) == 59
    with open(jpath) as f:
        for line, ref in zip(f, want[1:]):
            rec = json.loads(line)
            cs = rec["citizen_states"]
            assert len(cs) == len(ref)
            assert [c["location"]["x"] for c in cs] == [int(v) for v in ref["x"]]
            assert [c["location"]["y"] for c in cs] == [int(v) for v in ref["y"]]
            assert "".join(c["state"] for c in cs) == "".join(LETTERS[v] for v in _letters(ref))

    # the same hours in one call (graphs, 24-hour chunks) give the same stream
    eng = Epidemiology(Config(json.dumps(cfg)))
    path2 = tmp_path / "segment.bin"
    eng.open_state_stream(str(path2))
    eng.simulate_hours(1, 59)
    eng.close_state_stream()
    eng.close()
    assert path2.read_bytes() == path.read_bytes()


@pytest.mark.gpu
def test_stream_through_the_run_loop(gpu, oracle_mod, tmp_path):
    from epirust_gb300 import Config, Epidemiology
    from epirust_gb300.state_stream import read_state_stream

    cfg = make_config(n=3000, grid=110, hours=24 * 6, seed=52, disease=COVID_FAST, starting=(0, 0, 5, 20),
                      interventions=[{"Lockdown": {"at_number_of_infections": 20, "essential_workers_population": 0.1}}])
    eng = Epidemiology(Config(json.dumps(cfg)))
    path = tmp_path / "run.bin"
    eng.open_state_stream(str(path))
    rows = eng.run()
    eng.close_state_stream()
    final = eng.snapshot()
    eng.close()
    decoded = list(read_state_stream(str(path)))
    assert [h for h, *_ in decoded][1:] == [int(r) for r in rows["hour"]]
    hour, x, y, letters = decoded[-1]
    assert (x == final["x"]).all() and (y == final["y"]).all() and (letters == _letters(final)).all()
    # and the run it recorded is the oracle's run (rows and final agents)
    sim = oracle_mod.O1(oracle_mod.params_from_config(cfg))
    want = sim.run(1, cfg["hours"], interventions=True, stop=True)
    assert len(want) == len(rows) and all((want[k] == rows[k]).all() for k in rows.dtype.names)
    ref = sim.export()
    assert (x == ref["x"]).all() and (y == ref["y"]).all() and (letters == _letters(ref)).all()
    # per-hour counts agree with the letters (hospitalised agents are infected: letter i)
    for (h, _, _, l), r in zip(decoded[1:], rows):
        assert (l == 0).sum() == r["susceptible"] and (l == 1).sum() == r["exposed"]
        assert (l == 2).sum() == r["infected"] + r["hospitalized"]
        assert (l == 3).sum() == r["recovered"] and (l == 4).sum() == r["deceased"]
