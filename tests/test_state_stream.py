"""Citizen-state stream: the per-hour (letter, cell) of every agent, encoded on the device
and decoded by epirust_gb300.state_stream, equals the engine's own snapshots hour by hour."""
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


@pytest.mark.gpu
def test_stream_equals_hourly_snapshots(gpu, tmp_path):
    from epirust_gb300 import Config, Epidemiology
    from epirust_gb300.state_stream import read_state_stream

    cfg = make_config(n=4000, grid=120, hours=80, seed=51, disease=COVID_FAST, starting=(3, 3, 3, 30))
    eng = Epidemiology(Config(json.dumps(cfg)))
    path = tmp_path / "hourly.bin"
    eng.open_state_stream(str(path))
    snaps = [eng.snapshot().copy()]
    for hour in range(1, 60):
        eng.simulate_hours(hour, 1)
        snaps.append(eng.snapshot().copy())
    eng.close_state_stream()
    eng.close()
    decoded = list(read_state_stream(str(path)))
    assert [h for h, *_ in decoded] == list(range(60))
    for (hour, x, y, letters), snap in zip(decoded, snaps):
        assert (x == snap["x"]).all() and (y == snap["y"]).all(), hour
        assert (letters == _letters(snap)).all(), hour

    # the same hours in one call (graphs, 24-hour chunks) give the same stream
    eng = Epidemiology(Config(json.dumps(cfg)))
    path2 = tmp_path / "segment.bin"
    eng.open_state_stream(str(path2))
    eng.simulate_hours(1, 59)
    eng.close_state_stream()
    eng.close()
    assert path2.read_bytes() == path.read_bytes()


@pytest.mark.gpu
def test_stream_through_the_run_loop(gpu, tmp_path):
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
    # per-hour counts agree with the letters (hospitalised agents are infected: letter i)
    for (h, _, _, l), r in zip(decoded[1:], rows):
        assert (l == 0).sum() == r["susceptible"] and (l == 1).sum() == r["exposed"]
        assert (l == 2).sum() == r["infected"] + r["hospitalized"]
        assert (l == 3).sum() == r["recovered"] and (l == 4).sum() == r["deceased"]
