"""Host side of the engine in the shape of the reference's single-engine API.

    Config.read(path)                 common/src/config/mod.rs:119-123
    Epidemiology(config, seed)        engine/src/epidemiology_simulation.rs:75-135
      .run()                          run_single_engine, epidemiology_simulation.rs:211-274
      .simulate(hour) -> Counts       CitizenLocationMap::simulate, allocation_map.rs:67-129
      .process_interventions(counts)  allocation_map.rs:306-337
      .write_outputs(dir)             CsvListener / InterventionReporter

Every call goes through the C ABI of include/epi_engine.h into the CUDA engine.
"""
from __future__ import annotations

import ctypes as C
import os
import json
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import AGENT_DTYPE, COUNTS_DTYPE, EpiCounts, EpiGeography, EpiParams, check, lib


@dataclass(frozen=True)
class Counts:
    """One CSV row (engine/src/models/events/counts.rs:25-34)."""
    hour: int
    susceptible: int
    exposed: int
    infected: int
    hospitalized: int
    recovered: int
    deceased: int

    @staticmethod
    def from_c(c: EpiCounts) -> "Counts":
        return Counts(c.hour, c.susceptible, c.exposed, c.infected, c.hospitalized, c.recovered, c.deceased)

    def to_c(self) -> EpiCounts:
        return EpiCounts(self.hour, self.susceptible, self.exposed, self.infected, self.hospitalized,
                         self.recovered, self.deceased)

    def total(self) -> int:
        return (self.susceptible + self.exposed + self.infected + self.hospitalized + self.recovered
                + self.deceased)


class Config:
    """The engine's JSON config, parsed by the library (same schema as the reference)."""

    def __init__(self, text: str):
        self.text = text
        self.params = EpiParams()
        err = C.create_string_buffer(512)
        rc = lib().epi_params_from_json(text.encode(), C.byref(self.params), err, len(err))
        if rc != _lib.EPI_OK:
            raise _lib.EpiError(rc, err.value.decode())

    @staticmethod
    def read(path: str) -> "Config":
        with open(path) as f:
            return Config(f.read())

    @staticmethod
    def from_dict(d: dict) -> "Config":
        return Config(json.dumps(d))

    @property
    def hours(self) -> int:
        return self.params.hours

    @property
    def number_of_agents(self) -> int:
        return self.params.number_of_agents


def define_geography(grid_size: int) -> EpiGeography:
    g = EpiGeography()
    check(lib().epi_define_geography(grid_size, C.byref(g)))
    return g


def interventions_replay(params: EpiParams, rows: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """process_interventions' triggers on the host over hourly counts rows (COUNTS_DTYPE, in
    the order the run loop offers them): per row the EPI_IV_* bits that fire, and whether the
    run loop's device guard would mark that row."""
    rows = np.ascontiguousarray(rows, dtype=COUNTS_DTYPE)
    applied = np.zeros(len(rows), dtype=np.uint32)
    guard = np.zeros(len(rows), dtype=np.uint8)
    check(lib().epi_interventions_replay(C.byref(params), rows.ctypes.data, len(rows), applied.ctypes.data,
                                         guard.ctypes.data))
    return applied, guard


def write_outputs_for_rows(directory: str, engine_id: str, params: EpiParams, rows: np.ndarray) -> None:
    """The reference listeners' CSV and interventions JSON for hourly counts rows, without a
    device (the interventions are replayed over the rows)."""
    rows = np.ascontiguousarray(rows, dtype=COUNTS_DTYPE)
    check(lib().epi_outputs_write(os.fsencode(directory), engine_id.encode(), C.byref(params), rows.ctypes.data,
                                  len(rows)))


def read_population_csv(path: str) -> np.ndarray:
    """Population::Csv rows as flags (bit 0 working, bit 1 public transport)."""
    n = C.c_uint32(0)
    check(lib().epi_population_read_csv(os.fsencode(path), None, 0, C.byref(n)))
    flags = np.zeros(n.value, dtype=np.uint8)
    check(lib().epi_population_read_csv(os.fsencode(path), flags.ctypes.data, n.value, C.byref(n)))
    return flags


def world_build(params: EpiParams) -> tuple[np.ndarray, EpiGeography]:
    """Host world build (population, start points, hospital) as agent records."""
    n = params.number_of_agents
    recs = np.zeros(n, dtype=AGENT_DTYPE)
    g = EpiGeography()
    if params.population_source == 1:
        flags = read_population_csv(params.population_file.decode())
        check(lib().epi_world_build_population(C.byref(params), flags.ctypes.data, len(flags), recs.ctypes.data,
                                               C.byref(g)))
    else:
        check(lib().epi_world_build(C.byref(params), recs.ctypes.data, n, C.byref(g)))
    return recs, g


CHECKPOINT_HEADER_WORDS = 15  # u32 words before the parameters (epi_engine_checkpoint_write)


def checkpoint_params(path: str) -> EpiParams:
    """The parameters stored in a checkpoint file (they follow its 15-word header)."""
    with open(path, "rb") as f:
        head = f.read(4 * CHECKPOINT_HEADER_WORDS + C.sizeof(EpiParams))
    words = np.frombuffer(head[: 4 * CHECKPOINT_HEADER_WORDS], dtype="<u4")
    if len(head) < 4 * CHECKPOINT_HEADER_WORDS + C.sizeof(EpiParams) or words[0] != 0x4B435045 \
            or words[2] != C.sizeof(EpiParams):
        raise ValueError(f"{path}: not a checkpoint of this build")
    return EpiParams.from_buffer_copy(head[4 * CHECKPOINT_HEADER_WORDS:])


class Epidemiology:
    """One single-region engine on the GPU."""

    def __init__(self, config: "Config | EpiParams", seed: int | None = None, records: np.ndarray | None = None):
        self.config = config if isinstance(config, Config) else None
        self.params = EpiParams.from_buffer_copy(config.params if isinstance(config, Config) else config)
        if seed is not None:
            self.params.seed = seed
        h = C.c_void_p()
        if records is None and self.params.population_source == 1:  # Population::Csv
            flags = read_population_csv(self.params.population_file.decode())
            self.params.number_of_agents = len(flags)
            rc = lib().epi_engine_create_population(C.byref(self.params), flags.ctypes.data, len(flags), C.byref(h))
        elif records is None:
            rc = lib().epi_engine_create(C.byref(self.params), C.byref(h))
        else:
            records = np.ascontiguousarray(records, dtype=AGENT_DTYPE)
            self.params.number_of_agents = len(records)
            rc = lib().epi_engine_create_from_records(C.byref(self.params), records.ctypes.data, len(records),
                                                      C.byref(h))
        check(rc, None)
        self._h = h
        self.rows: list[Counts] = []

    # -- lifetime
    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().epi_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    # -- the tick
    def simulate(self, hour: int) -> Counts:
        c = EpiCounts()
        check(lib().epi_engine_simulate(self._h, hour, C.byref(c)), self._h)
        return Counts.from_c(c)

    def simulate_hours(self, first_hour: int, n: int) -> np.ndarray:
        out = np.zeros(n, dtype=COUNTS_DTYPE)
        check(lib().epi_engine_simulate_hours(self._h, first_hour, n, out.ctypes.data), self._h)
        return out

    def process_interventions(self, counts: Counts) -> int:
        applied = C.c_uint32(0)
        c = counts.to_c()
        check(lib().epi_engine_process_interventions(self._h, C.byref(c), C.byref(applied)), self._h)
        return applied.value

    def lock_city(self) -> None:
        check(lib().epi_engine_lock_city(self._h), self._h)

    def unlock_city(self) -> None:
        check(lib().epi_engine_unlock_city(self._h), self._h)

    def vaccinate(self, hour: int, percent: float) -> None:
        check(lib().epi_engine_vaccinate(self._h, hour, percent), self._h)

    def increase_hospital_size(self) -> None:
        check(lib().epi_engine_increase_hospital_size(self._h), self._h)

    # -- the run loop
    def run(self) -> np.ndarray:
        """run_single_engine: hours 1..hours-1 with interventions and the stop rule (a run
        paused by run_until continues where it stopped; the rows start at hour 1)."""
        cap = max(self.params.hours, 1)
        rows = np.zeros(cap, dtype=COUNTS_DTYPE)
        n = C.c_uint32(0)
        check(lib().epi_engine_run(self._h, rows.ctypes.data, cap, C.byref(n)), self._h)
        return rows[: n.value]

    def run_until(self, last_hour: int) -> tuple[np.ndarray, int]:
        """The run loop paused after last_hour: (rows so far, the hour it continues from, 0 when
        the run has ended)."""
        cap = max(self.params.hours, 1)
        rows = np.zeros(cap, dtype=COUNTS_DTYPE)
        n, nxt = C.c_uint32(0), C.c_uint32(0)
        check(lib().epi_engine_run_until(self._h, last_hour, rows.ctypes.data, cap, C.byref(n), C.byref(nxt)), self._h)
        return rows[: n.value], nxt.value

    def save_checkpoint(self, path: str) -> None:
        """Write the world, its intervention state and a paused run's position to a file."""
        check(lib().epi_engine_checkpoint_write(self._h, str(path).encode()), self._h)

    @classmethod
    def from_checkpoint(cls, path: str) -> "Epidemiology":
        """An engine resumed from save_checkpoint's file (run() continues a paused run)."""
        h = C.c_void_p()
        check(lib().epi_engine_create_from_checkpoint(str(path).encode(), C.byref(h)), None)
        self = cls.__new__(cls)
        self._h = h
        self.config = None
        self.rows = []
        self.params = checkpoint_params(str(path))
        return self

    def write_outputs(self, output_dir: str, engine_id: str = "0") -> None:
        check(lib().epi_engine_write_outputs(self._h, output_dir.encode(), engine_id.encode()), self._h)

    # -- inspection
    def population(self) -> int:
        n = C.c_uint32(0)
        check(lib().epi_engine_population(self._h, C.byref(n)), self._h)
        return n.value

    def snapshot(self) -> np.ndarray:
        n = self.population()
        out = np.zeros(n, dtype=AGENT_DTYPE)
        check(lib().epi_engine_snapshot(self._h, out.ctypes.data, n), self._h)
        return out

    def geography(self) -> EpiGeography:
        g = EpiGeography()
        check(lib().epi_engine_geography(self._h, C.byref(g)), self._h)
        return g

    def check_invariants(self) -> None:
        check(lib().epi_engine_check(self._h), self._h)

    def set_stream(self, stream_ptr: int | None) -> None:
        check(lib().epi_engine_set_stream(self._h, C.c_void_p(stream_ptr or 0)), self._h)

    def set_profiling(self, on: bool) -> None:
        check(lib().epi_engine_set_profiling(self._h, 1 if on else 0), self._h)

    def kernel_stats(self) -> dict:
        L = lib()
        k = L.epi_engine_kernel_kinds()
        launches = (C.c_uint32 * k)()
        ms = (C.c_double * k)()
        check(L.epi_engine_kernel_stats(self._h, launches, ms, k), self._h)
        return {L.epi_engine_kernel_name(i).decode(): (launches[i], ms[i]) for i in range(k)}

    def save_state(self) -> None:
        check(lib().epi_engine_save_state(self._h), self._h)

    def restore_state(self) -> None:
        check(lib().epi_engine_restore_state(self._h), self._h)

    def kernels_launched(self) -> int:
        v = C.c_uint64(0)
        check(lib().epi_engine_kernels_launched(self._h, C.byref(v)), self._h)
        return v.value

    def open_state_stream(self, path: str) -> None:
        """Record every later hour's citizen states (letter and cell of every agent) to path;
        epirust_gb300.state_stream.read_state_stream decodes it."""
        check(lib().epi_engine_state_stream_open(self._h, os.fsencode(path)), self._h)

    def close_state_stream(self) -> None:
        check(lib().epi_engine_state_stream_close(self._h), self._h)

    def autotune(self, hours: int = 24) -> dict:
        """Pick the fastest launch shape over hours 1..hours (state restored afterwards)."""
        s = _lib.LaunchShape()
        check(lib().epi_engine_autotune(self._h, hours, C.byref(s)), self._h)
        return {"decide_blocks": s.decide_blocks, "commit_slots": s.commit_slots, "hour_us": s.hour_us}

    def set_launch_shape(self, decide_blocks: int, commit_slots: int) -> None:
        s = _lib.LaunchShape(decide_blocks, commit_slots, 0.0)
        check(lib().epi_engine_set_launch_shape(self._h, C.byref(s)), self._h)

    def launch_shape(self) -> dict:
        s = _lib.LaunchShape()
        check(lib().epi_engine_launch_shape(self._h, C.byref(s)), self._h)
        return {"decide_blocks": s.decide_blocks, "commit_slots": s.commit_slots}

    def hour_bytes(self, hour: int) -> float:
        b = C.c_double(0.0)
        check(lib().epi_engine_hour_bytes(self._h, hour, C.byref(b)), self._h)
        return b.value


class Ensemble:
    """Many independent worlds on one device, advanced together (epi_ensemble_*)."""

    def __init__(self, params: list):
        L = lib()
        self.params = (EpiParams * len(params))(*[EpiParams.from_buffer_copy(p) for p in params])
        h = C.c_void_p()
        rc = L.epi_ensemble_create(self.params, len(params), C.byref(h))
        if rc != _lib.EPI_OK:
            raise _lib.EpiError(rc, L.epi_ensemble_last_error(None).decode())
        self._h = h
        self.replicates = len(params)

    def _check(self, rc):
        if rc != _lib.EPI_OK:
            raise _lib.EpiError(rc, lib().epi_ensemble_last_error(self._h).decode())

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().epi_ensemble_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self) -> list:
        """Per replicate: the structured counts rows of run_single_engine."""
        cap = max(p.hours for p in self.params)
        rows = np.zeros((self.replicates, max(cap, 1)), dtype=COUNTS_DTYPE)
        n = np.zeros(self.replicates, dtype=np.uint32)
        self._check(lib().epi_ensemble_run(self._h, rows.ctypes.data, rows.shape[1], n.ctypes.data))
        return [rows[r, : n[r]] for r in range(self.replicates)]

    def snapshot(self, r: int) -> np.ndarray:
        out = np.zeros(self.params[r].number_of_agents, dtype=AGENT_DTYPE)
        self._check(lib().epi_ensemble_snapshot(self._h, r, out.ctypes.data, len(out)))
        return out

    def check_invariants(self) -> None:
        self._check(lib().epi_ensemble_check(self._h))

    def save_state(self) -> None:
        self._check(lib().epi_ensemble_save_state(self._h))

    def restore_state(self) -> None:
        self._check(lib().epi_ensemble_restore_state(self._h))

    def set_stream(self, stream_ptr: int | None) -> None:
        self._check(lib().epi_ensemble_set_stream(self._h, C.c_void_p(stream_ptr or 0)))

    def set_profiling(self, on: bool) -> None:
        self._check(lib().epi_ensemble_set_profiling(self._h, 1 if on else 0))

    def kernel_stats(self) -> dict:
        L = lib()
        k = L.epi_engine_kernel_kinds()
        launches = (C.c_uint32 * k)()
        ms = (C.c_double * k)()
        self._check(L.epi_ensemble_kernel_stats(self._h, launches, ms, k))
        return {L.epi_engine_kernel_name(i).decode(): (launches[i], ms[i]) for i in range(k)}

    def kernels_launched(self) -> int:
        v = C.c_uint64(0)
        self._check(lib().epi_ensemble_kernels_launched(self._h, C.byref(v)))
        return v.value

    def autotune(self, hours: int = 24) -> dict:
        """Pick the fastest launch shape for all replicates over hours 1..hours."""
        s = _lib.LaunchShape()
        self._check(lib().epi_ensemble_autotune(self._h, hours, C.byref(s)))
        return {"decide_blocks": s.decide_blocks, "commit_slots": s.commit_slots, "hour_us": s.hour_us}

    def hour_bytes(self, hour: int) -> float:
        b = C.c_double(0.0)
        self._check(lib().epi_ensemble_hour_bytes(self._h, hour, C.byref(b)))
        return b.value
