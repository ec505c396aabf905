"""TEST INFRASTRUCTURE ONLY: ctypes access to the CPU oracles (oracle/o1.c, oracle/o2.c).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference legs import
this module, and only as the checker or the timed CPU baseline.  It parses the engine's
JSON config itself (Python json, following common/src/config/*.rs) so that the oracle does
not depend on the product's C++ parser.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libepi_oracle.so")
MAX_VACC = 32


def build() -> str:
    r = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB_PATH


class Params(C.Structure):
    """epi_params of include/epi_engine.h."""
    _fields_ = [
        ("number_of_agents", C.c_uint32), ("public_transport_percentage", C.c_double),
        ("working_percentage", C.c_double), ("grid_size", C.c_uint32), ("hospital_beds_percentage", C.c_double),
        ("hours", C.c_uint32), ("regular_transmission_start_day", C.c_uint32),
        ("high_transmission_start_day", C.c_uint32), ("last_day", C.c_uint32),
        ("asymptomatic_last_day", C.c_uint32), ("mild_infected_last_day", C.c_uint32),
        ("regular_transmission_rate", C.c_double), ("high_transmission_rate", C.c_double),
        ("death_rate", C.c_double), ("percentage_asymptomatic_population", C.c_double),
        ("percentage_severe_infected_population", C.c_double), ("exposed_duration", C.c_uint32),
        ("pre_symptomatic_duration", C.c_uint32), ("infected_mild_asymptomatic", C.c_uint32),
        ("infected_mild_symptomatic", C.c_uint32), ("infected_severe", C.c_uint32), ("exposed", C.c_uint32),
        ("has_lockdown", C.c_int32), ("lockdown_at_number_of_infections", C.c_uint32),
        ("essential_workers_population", C.c_double), ("has_build_new_hospital", C.c_int32),
        ("spread_rate_threshold", C.c_uint32), ("n_vaccinations", C.c_int32),
        ("vaccination_at_hour", C.c_uint32 * MAX_VACC), ("vaccination_percent", C.c_double * MAX_VACC),
        ("hospital_occupancy_trigger", C.c_double), ("seed", C.c_uint64),
        ("population_source", C.c_uint32), ("population_file", C.c_char * 256),
    ]


class Area(C.Structure):
    _fields_ = [("x0", C.c_int32), ("y0", C.c_int32), ("x1", C.c_int32), ("y1", C.c_int32)]

    def tuple(self):
        return (self.x0, self.y0, self.x1, self.y1)


class Geography(C.Structure):
    _fields_ = [("grid_size", C.c_uint32), ("housing", Area), ("transport", Area), ("work", Area),
                ("hospital", Area), ("houses_x", C.c_uint32), ("houses_y", C.c_uint32),
                ("offices_x", C.c_uint32), ("offices_y", C.c_uint32)]


AGENT_DTYPE = np.dtype([
    ("x", "<i4"), ("y", "<i4"), ("state", "u1"), ("flags", "u1"), ("work_status", "u1"), ("immunity", "i1"),
    ("at_hour", "<u4"), ("infection_day", "<u4"), ("work_start_at", "<u4"),
    ("home_x", "<i4"), ("home_y", "<i4"), ("work_x", "<i4"), ("work_y", "<i4"),
    ("area_x0", "<i4"), ("area_y0", "<i4"), ("area_x1", "<i4"), ("area_y1", "<i4"),
], align=True)


def params_from_config(cfg: dict | str, seed: int = 0) -> Params:
    """Config JSON -> Params (common/src/config/mod.rs:44-58 and its submodules)."""
    if isinstance(cfg, str):
        cfg = json.loads(cfg)
    p = Params()
    auto = cfg["population"]["Auto"]
    p.number_of_agents = int(auto["number_of_agents"])
    p.public_transport_percentage = float(auto["public_transport_percentage"])
    p.working_percentage = float(auto["working_percentage"])
    d = cfg["disease"]
    for k in ("regular_transmission_start_day", "high_transmission_start_day", "last_day", "asymptomatic_last_day",
              "mild_infected_last_day", "exposed_duration", "pre_symptomatic_duration"):
        setattr(p, k, int(d[k]))
    for k in ("regular_transmission_rate", "high_transmission_rate", "death_rate",
              "percentage_asymptomatic_population", "percentage_severe_infected_population"):
        setattr(p, k, float(d[k]))
    g = cfg["geography_parameters"]
    p.grid_size = int(g["grid_size"])
    p.hospital_beds_percentage = float(g["hospital_beds_percentage"])
    p.hours = int(cfg["hours"])
    nv = 0
    for iv in cfg["interventions"]:
        (kind, body), = iv.items()
        if kind == "Vaccinate":
            p.vaccination_at_hour[nv] = int(body["at_hour"])
            p.vaccination_percent[nv] = float(body["percent"])
            nv += 1
        elif kind == "Lockdown" and not p.has_lockdown:
            p.has_lockdown = 1
            p.lockdown_at_number_of_infections = int(body["at_number_of_infections"])
            p.essential_workers_population = float(body["essential_workers_population"])
        elif kind == "BuildNewHospital" and not p.has_build_new_hospital:
            p.has_build_new_hospital = 1
            p.spread_rate_threshold = int(body["spread_rate_threshold"])
    p.n_vaccinations = nv
    si = cfg.get("starting_infections")
    if si is None:
        p.exposed = 1
    else:
        p.infected_mild_asymptomatic = int(si["infected_mild_asymptomatic"])
        p.infected_mild_symptomatic = int(si["infected_mild_symptomatic"])
        p.infected_severe = int(si["infected_severe"])
        p.exposed = int(si["exposed"])
    p.hospital_occupancy_trigger = float(cfg.get("hospital_occupancy_trigger", 0.0))
    p.seed = int(cfg.get("seed", seed)) if seed == 0 else seed
    return p


_lib = None


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        build()
    L = C.CDLL(LIB_PATH)
    P, V = C.POINTER, C.c_void_p
    L.o1_create.restype = V
    L.o1_create.argtypes = [P(Params), P(C.c_int)]
    L.o1_create_from_records.restype = V
    L.o1_create_from_records.argtypes = [P(Params), V, C.c_uint32, P(C.c_int)]
    L.o1_free.argtypes = [V]
    L.o1_simulate.argtypes = [V, C.c_uint32, P(C.c_uint32)]
    L.o1_process_interventions.restype = C.c_uint32
    L.o1_process_interventions.argtypes = [V, C.c_uint32, P(C.c_uint32)]
    L.o1_run.argtypes = [V, C.c_uint32, C.c_uint32, V, P(C.c_uint32), C.c_int, C.c_int]
    L.o1_export.argtypes = [V, V]
    L.o1_geography.argtypes = [V, P(Geography)]
    L.o1_population.restype = C.c_uint32
    L.o1_population.argtypes = [V]
    L.o1_lock_city.argtypes = [V]
    L.o1_unlock_city.argtypes = [V]
    L.o1_vaccinate.argtypes = [V, C.c_uint32, C.c_double]
    L.o1_increase_hospital_size.argtypes = [V]
    L.o1_n_reports.restype = C.c_uint32
    L.o1_n_reports.argtypes = [V]
    L.o1_report.argtypes = [V, C.c_uint32, P(C.c_uint32), C.c_char_p, C.c_char_p]
    L.o1_transmission_rate.restype = C.c_double
    L.o1_transmission_rate.argtypes = [P(Params), C.c_uint32]
    L.o1_is_to_be_hospitalized.argtypes = [P(Params), C.c_uint32]
    L.o1_define_geography.argtypes = [C.c_uint32, P(Geography)]
    L.o1_resize_hospital.argtypes = [P(Geography), C.c_int32, C.c_double, C.c_double]
    L.o1_geography_increase_hospital_size.argtypes = [P(Geography), C.c_uint32]
    L.o1_philox.argtypes = [P(C.c_uint32), P(C.c_uint32), P(C.c_uint32)]
    L.o1_philox2x32.argtypes = [P(C.c_uint32), C.c_uint32, P(C.c_uint32)]
    L.o1_area_neighbors.argtypes = [C.c_int32] * 6 + [P(C.c_int32), P(C.c_uint32)]
    L.o1_area_cells.restype = C.c_uint32
    L.o1_area_cells.argtypes = [C.c_int32] * 4 + [P(C.c_int32), C.c_uint32]
    L.o1_area_factory.restype = C.c_uint32
    L.o1_area_factory.argtypes = [C.c_int32] * 4 + [C.c_uint32, P(C.c_int32), C.c_uint32]
    L.o2_create_from_records.restype = V
    L.o2_create_from_records.argtypes = [P(Params), V, C.c_uint32, C.c_int, P(C.c_int)]
    L.o2_free.argtypes = [V]
    L.o2_simulate.argtypes = [V, C.c_uint32, P(C.c_uint32)]
    L.o2_run.argtypes = [V, C.c_uint32, C.c_uint32, V, P(C.c_uint32), C.c_int, C.c_int]
    L.o2_export.argtypes = [V, V]
    L.o2_process_interventions.restype = C.c_uint32
    L.o2_process_interventions.argtypes = [V, C.c_uint32, P(C.c_uint32)]
    _lib = L
    return L


class OracleError(RuntimeError):
    pass


ROW_DTYPE = np.dtype([(k, "<u4") for k in
                      ("hour", "susceptible", "exposed", "infected", "hospitalized", "recovered", "deceased")])


class O1:
    """The bit-exact scalar oracle (lowest index wins, Philox draw slots)."""

    def __init__(self, params: Params, records: np.ndarray | None = None):
        self.params = params
        st = C.c_int(0)
        if records is None:
            self._h = lib().o1_create(C.byref(params), C.byref(st))
        else:
            records = np.ascontiguousarray(records, dtype=AGENT_DTYPE)
            self._h = lib().o1_create_from_records(C.byref(params), records.ctypes.data, len(records), C.byref(st))
        if st.value != 0:
            lib().o1_free(self._h)
            self._h = None
            raise OracleError(f"oracle create failed with status {st.value}")

    def __del__(self):
        if getattr(self, "_h", None):
            lib().o1_free(self._h)
            self._h = None

    @property
    def n(self) -> int:
        return lib().o1_population(self._h)

    def simulate(self, hour: int) -> np.ndarray:
        c = (C.c_uint32 * 6)()
        rc = lib().o1_simulate(self._h, hour, c)
        if rc:
            raise OracleError(f"o1_simulate status {rc}")
        return np.array(list(c), dtype=np.uint32)

    def process_interventions(self, hour: int, counts) -> int:
        c = (C.c_uint32 * 6)(*[int(v) for v in counts])
        return lib().o1_process_interventions(self._h, hour, c)

    def run(self, first_hour: int, last_hour_excl: int, interventions: bool = True, stop: bool = True) -> np.ndarray:
        n = max(last_hour_excl - first_hour, 0)
        rows = np.zeros(max(n, 1), dtype=ROW_DTYPE)
        k = C.c_uint32(0)
        rc = lib().o1_run(self._h, first_hour, last_hour_excl, rows.ctypes.data, C.byref(k), int(interventions),
                          int(stop))
        if rc:
            raise OracleError(f"o1_run status {rc}")
        return rows[: k.value]

    def export(self) -> np.ndarray:
        out = np.zeros(self.n, dtype=AGENT_DTYPE)
        lib().o1_export(self._h, out.ctypes.data)
        return out

    def geography(self) -> Geography:
        g = Geography()
        lib().o1_geography(self._h, C.byref(g))
        return g

    def lock_city(self):
        lib().o1_lock_city(self._h)

    def unlock_city(self):
        lib().o1_unlock_city(self._h)

    def vaccinate(self, hour: int, percent: float):
        lib().o1_vaccinate(self._h, hour, percent)

    def increase_hospital_size(self):
        lib().o1_increase_hospital_size(self._h)

    def reports(self) -> list[tuple[int, str, str]]:
        out = []
        for k in range(lib().o1_n_reports(self._h)):
            h = C.c_uint32(0)
            name = C.create_string_buffer(64)
            data = C.create_string_buffer(64)
            lib().o1_report(self._h, k, C.byref(h), name, data)
            out.append((h.value, name.value.decode(), data.value.decode()))
        return out


class O2:
    """Reference-semantics port: hash map, threaded map phase, serial resolve in hash order."""

    def __init__(self, params: Params, records: np.ndarray, threads: int = 1):
        records = np.ascontiguousarray(records, dtype=AGENT_DTYPE)
        st = C.c_int(0)
        self._h = lib().o2_create_from_records(C.byref(params), records.ctypes.data, len(records), threads,
                                               C.byref(st))
        self.n = len(records)
        if st.value != 0:
            lib().o2_free(self._h)
            self._h = None
            raise OracleError(f"o2 create failed with status {st.value}")

    def __del__(self):
        if getattr(self, "_h", None):
            lib().o2_free(self._h)
            self._h = None

    def simulate(self, hour: int) -> np.ndarray:
        c = (C.c_uint32 * 6)()
        rc = lib().o2_simulate(self._h, hour, c)
        if rc:
            raise OracleError(f"o2_simulate status {rc}")
        return np.array(list(c), dtype=np.uint32)

    def run(self, first_hour: int, last_hour_excl: int, interventions: bool = True, stop: bool = True,
            keep_rows: bool = True) -> np.ndarray:
        n = max(last_hour_excl - first_hour, 0)
        rows = np.zeros(max(n, 1), dtype=ROW_DTYPE) if keep_rows else None
        k = C.c_uint32(0)
        rc = lib().o2_run(self._h, first_hour, last_hour_excl, rows.ctypes.data if keep_rows else None,
                          C.byref(k), int(interventions), int(stop))
        if rc:
            raise OracleError(f"o2_run status {rc}")
        return rows[: k.value] if keep_rows else np.zeros(k.value, dtype=ROW_DTYPE)

    def export(self) -> np.ndarray:
        out = np.zeros(self.n, dtype=AGENT_DTYPE)
        lib().o2_export(self._h, out.ctypes.data)
        return out


def philox(ctr, key) -> list[int]:
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().o1_philox(c, k, o)
    return list(o)


def philox2x32(ctr, key: int) -> list[int]:
    c = (C.c_uint32 * 2)(*ctr)
    o = (C.c_uint32 * 2)()
    lib().o1_philox2x32(c, key, o)
    return list(o)


def define_geography(G: int) -> Geography:
    g = Geography()
    lib().o1_define_geography(G, C.byref(g))
    return g


def resize_hospital(g: Geography, n: int, staff: float, beds: float) -> Geography:
    lib().o1_resize_hospital(C.byref(g), n, staff, beds)
    return g


def increase_hospital_size(g: Geography, grid_size: int) -> Geography:
    lib().o1_geography_increase_hospital_size(C.byref(g), grid_size)
    return g


def transmission_rate(p: Params, day: int) -> float:
    return lib().o1_transmission_rate(C.byref(p), day)


def is_to_be_hospitalized(p: Params, day: int) -> bool:
    return bool(lib().o1_is_to_be_hospitalized(C.byref(p), day))


def area_neighbors(area, point) -> list[tuple[int, int]]:
    out = (C.c_int32 * 16)()
    n = C.c_uint32(0)
    lib().o1_area_neighbors(*area, *point, out, C.byref(n))
    return [(out[2 * i], out[2 * i + 1]) for i in range(n.value)]


def area_cells(area) -> list[tuple[int, int]]:
    cap = 4096
    out = (C.c_int32 * (2 * cap))()
    n = lib().o1_area_cells(*area, out, cap)
    return [(out[2 * i], out[2 * i + 1]) for i in range(min(n, cap))]


def area_factory(start, end, size: int) -> list[tuple[int, int, int, int]]:
    cap = 4096
    out = (C.c_int32 * (4 * cap))()
    n = lib().o1_area_factory(*start, *end, size, out, cap)
    return [tuple(out[4 * i: 4 * i + 4]) for i in range(min(n, cap))]
