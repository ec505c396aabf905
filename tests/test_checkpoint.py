"""Checkpoint and resume: a run paused at any hour and continued -- on the same handle, after a
device-side restore, or from a checkpoint file in a new engine -- gives the uninterrupted
run's rows and final world bit for bit; damaged files are refused before any device work."""
import ctypes as C
import json
import struct

import numpy as np
import pytest

from helpers import COVID_FAST, make_config

EPI_ERR_IO = 7


def _fnv1a64(b: bytes) -> int:
    x = 0xCBF29CE484222325
    for c in b:
        x = ((x ^ c) * 0x100000001B3) & 0xFFFFFFFFFFFFFFFF
    return x


def _create(path):
    from epirust_gb300 import _lib

    L = _lib.lib()
    h = C.c_void_p()
    rc = L.epi_engine_create_from_checkpoint(str(path).encode(), C.byref(h))
    return rc, L.epi_engine_last_error(None).decode()


@pytest.mark.parametrize("content,message", [
    (None, "cannot read"),
    (b"\x00" * 200, "checksum"),
    (b"EPCK" + b"\x01" * 100, "checksum"),
])
def test_damaged_checkpoints_are_refused(engine_built, tmp_path, content, message):
    path = tmp_path / "ck.bin"
    if content is not None:
        path.write_bytes(content)
    rc, msg = _create(path)
    assert rc == EPI_ERR_IO and message in msg, msg


def test_checkpoint_of_another_kind_is_refused(engine_built, tmp_path):
    body = struct.pack("<15I", 0x12345678, 1, *([0] * 13)) + b"\x00" * 64
    path = tmp_path / "ck.bin"
    path.write_bytes(body + struct.pack("<Q", _fnv1a64(body)))
    rc, msg = _create(path)
    assert rc == EPI_ERR_IO and "not a checkpoint" in msg, msg
    body = struct.pack("<15I", 0x4B435045, 99, *([0] * 13)) + b"\x00" * 64
    path.write_bytes(body + struct.pack("<Q", _fnv1a64(body)))
    rc, msg = _create(path)
    assert rc == EPI_ERR_IO and "version" in msg, msg


CASE = make_config(n=5000, grid=120, hours=24 * 30, seed=61, disease=COVID_FAST, starting=(0, 0, 5, 30),
                   interventions=[{"Lockdown": {"at_number_of_infections": 25, "essential_workers_population": 0.1}},
                                  {"Vaccinate": {"at_hour": 200, "percent": 0.3}},
                                  {"BuildNewHospital": {"spread_rate_threshold": 8}}])


def _engine():
    from epirust_gb300 import Config, Epidemiology

    return Epidemiology(Config(json.dumps(CASE)))


def _same(a, b):
    return a.shape == b.shape and all((a[k] == b[k]).all() for k in a.dtype.names)


@pytest.mark.gpu
def test_paused_runs_resume_exactly(gpu, tmp_path):
    from epirust_gb300 import Epidemiology

    ref = _engine()
    want = ref.run()
    want_world = ref.snapshot().copy()
    reports = ref.geography().hospital.tuple()
    ref.close()
    assert len(want) > 300

    # same handle: several pauses, at day boundaries and mid-day
    eng = _engine()
    rows, nxt = eng.run_until(50)
    assert len(rows) == 50 and nxt == 51
    rows, nxt = eng.run_until(173)
    assert len(rows) == 173 and nxt == 174
    assert _same(rows, want[:173])
    got = eng.run()
    assert _same(got, want)
    assert (eng.snapshot().view(np.uint8) == want_world.view(np.uint8)).all()
    eng.close()

    # checkpoint file after the lockdown and before the vaccination; a new engine resumes
    eng = _engine()
    rows, nxt = eng.run_until(150)
    path = tmp_path / "run.ck"
    eng.save_checkpoint(str(path))
    eng.close()
    back = Epidemiology.from_checkpoint(str(path))
    assert back.params.hours == CASE["hours"]
    got = back.run()
    assert _same(got, want)
    assert (back.snapshot().view(np.uint8) == want_world.view(np.uint8)).all()
    assert back.geography().hospital.tuple() == reports
    back.check_invariants()
    back.close()


@pytest.mark.gpu
def test_save_restore_keeps_the_run_position(gpu):
    eng = _engine()
    eng.run_until(100)
    eng.save_state()
    first = eng.run()
    eng.restore_state()
    again = eng.run()
    assert _same(first, again)
    # a finished run starts over at hour 1 on the world as it now is
    rows, nxt = eng.run_until(10)
    assert len(rows) == 10 and nxt == 11
    eng.close()


@pytest.mark.gpu
def test_pauses_at_event_hours(gpu):
    """Pauses at the first hour, at day boundaries, around the vaccination hour and at the
    last hour all resume to the uninterrupted run."""
    ref = _engine()
    want = ref.run()
    ref.close()
    eng = _engine()
    for pause in (1, 24, 199, 200, 201, 479, len(want) - 1):
        eng.save_state()
        rows, nxt = eng.run_until(pause)
        assert _same(rows, want[:pause]) and nxt == pause + 1, pause
        got = eng.run()
        assert _same(got, want), pause
        eng.restore_state()
    rows, nxt = eng.run_until(10**6)
    assert _same(rows, want) and nxt == 0
    eng.close()
