"""ctypes binding of include/epi_engine.h.

The library is built in-tree (epirust_gb300/build.py) and loaded from
epirust_gb300/_build/libepirust_gb300.so.  There is no fallback: if the library is missing
or fails to load, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libepirust_gb300.so")

EPI_OK = 0
ERRORS = {1: "EPI_ERR_CONFIG", 2: "EPI_ERR_CAPACITY", 3: "EPI_ERR_CUDA", 4: "EPI_ERR_TIMEOUT",
          5: "EPI_ERR_INVARIANT", 6: "EPI_ERR_ARG", 7: "EPI_ERR_IO"}
MAX_VACCINATIONS = 32

S, E, I_PRE, I_ASYM, I_MILD, I_SEVERE, R, D = range(8)
WS_NORMAL, WS_ESSENTIAL, WS_HOSPITAL_STAFF, WS_NA = range(4)
F_HOSPITALIZED, F_ISOLATED, F_VACCINATED, F_WORK_QUARANTINED, F_PUBLIC_TRANSPORT = 1, 2, 4, 8, 16
IV_VACCINATION, IV_LOCKDOWN, IV_LOCKDOWN_REVOKED, IV_BUILD_NEW_HOSPITAL = 1, 2, 4, 8


class EpiParams(C.Structure):
    _fields_ = [
        ("number_of_agents", C.c_uint32),
        ("public_transport_percentage", C.c_double),
        ("working_percentage", C.c_double),
        ("grid_size", C.c_uint32),
        ("hospital_beds_percentage", C.c_double),
        ("hours", C.c_uint32),
        ("regular_transmission_start_day", C.c_uint32),
        ("high_transmission_start_day", C.c_uint32),
        ("last_day", C.c_uint32),
        ("asymptomatic_last_day", C.c_uint32),
        ("mild_infected_last_day", C.c_uint32),
        ("regular_transmission_rate", C.c_double),
        ("high_transmission_rate", C.c_double),
        ("death_rate", C.c_double),
        ("percentage_asymptomatic_population", C.c_double),
        ("percentage_severe_infected_population", C.c_double),
        ("exposed_duration", C.c_uint32),
        ("pre_symptomatic_duration", C.c_uint32),
        ("infected_mild_asymptomatic", C.c_uint32),
        ("infected_mild_symptomatic", C.c_uint32),
        ("infected_severe", C.c_uint32),
        ("exposed", C.c_uint32),
        ("has_lockdown", C.c_int32),
        ("lockdown_at_number_of_infections", C.c_uint32),
        ("essential_workers_population", C.c_double),
        ("has_build_new_hospital", C.c_int32),
        ("spread_rate_threshold", C.c_uint32),
        ("n_vaccinations", C.c_int32),
        ("vaccination_at_hour", C.c_uint32 * MAX_VACCINATIONS),
        ("vaccination_percent", C.c_double * MAX_VACCINATIONS),
        ("hospital_occupancy_trigger", C.c_double),
        ("seed", C.c_uint64),
        ("population_source", C.c_uint32),
        ("population_file", C.c_char * 256),
    ]


class EpiCounts(C.Structure):
    _fields_ = [(k, C.c_uint32) for k in
                ("hour", "susceptible", "exposed", "infected", "hospitalized", "recovered", "deceased")]


class EpiArea(C.Structure):
    _fields_ = [("x0", C.c_int32), ("y0", C.c_int32), ("x1", C.c_int32), ("y1", C.c_int32)]

    def tuple(self):
        return (self.x0, self.y0, self.x1, self.y1)


class EpiGeography(C.Structure):
    _fields_ = [("grid_size", C.c_uint32), ("housing", EpiArea), ("transport", EpiArea), ("work", EpiArea),
                ("hospital", EpiArea), ("houses_x", C.c_uint32), ("houses_y", C.c_uint32),
                ("offices_x", C.c_uint32), ("offices_y", C.c_uint32)]


# numpy view of epi_agent_record (56 bytes, C layout)
AGENT_DTYPE = np.dtype([
    ("x", "<i4"), ("y", "<i4"), ("state", "u1"), ("flags", "u1"), ("work_status", "u1"), ("immunity", "i1"),
    ("at_hour", "<u4"), ("infection_day", "<u4"), ("work_start_at", "<u4"),
    ("home_x", "<i4"), ("home_y", "<i4"), ("work_x", "<i4"), ("work_y", "<i4"),
    ("area_x0", "<i4"), ("area_y0", "<i4"), ("area_x1", "<i4"), ("area_y1", "<i4"),
], align=True)
COUNTS_DTYPE = np.dtype([(k, "<u4") for k in
                         ("hour", "susceptible", "exposed", "infected", "hospitalized", "recovered", "deceased")])

# Every symbol include/epi_engine.h declares.
EXPORTS = [
    "epi_params_from_json", "epi_define_geography", "epi_resize_hospital", "epi_geography_increase_hospital_size", "epi_disease_transmission_rate",
    "epi_disease_is_to_be_hospitalized", "epi_interventions_replay", "epi_outputs_write", "epi_world_build", "epi_engine_create", "epi_engine_create_json",
    "epi_engine_create_from_records", "epi_engine_destroy", "epi_engine_last_error", "epi_engine_set_stream",
    "epi_engine_simulate", "epi_engine_simulate_hours", "epi_engine_process_interventions", "epi_engine_lock_city",
    "epi_engine_unlock_city", "epi_engine_vaccinate", "epi_engine_increase_hospital_size", "epi_engine_run",
    "epi_engine_write_outputs", "epi_engine_population", "epi_engine_snapshot", "epi_engine_geography",
    "epi_engine_check", "epi_engine_set_profiling", "epi_engine_kernel_stats", "epi_engine_kernel_name",
    "epi_engine_kernel_kinds", "epi_abi_struct_size", "epi_engine_hour_bytes", "epi_engine_save_state",
    "epi_engine_restore_state", "epi_engine_kernels_launched", "epi_tick_hour_noalloc",
    "epi_ensemble_create", "epi_ensemble_destroy", "epi_ensemble_last_error", "epi_ensemble_set_stream",
    "epi_ensemble_replicates", "epi_ensemble_run", "epi_ensemble_snapshot", "epi_ensemble_check",
    "epi_ensemble_save_state", "epi_ensemble_restore_state", "epi_ensemble_set_profiling", "epi_ensemble_kernel_stats",
    "epi_ensemble_kernels_launched", "epi_ensemble_hour_bytes", "epi_engine_autotune", "epi_engine_set_launch_shape",
    "epi_engine_launch_shape", "epi_ensemble_autotune", "epi_engine_state_stream_open", "epi_engine_state_stream_close",
    "epi_population_read_csv", "epi_world_build_population", "epi_engine_create_population",
    "epi_engine_run_until", "epi_engine_checkpoint_write", "epi_engine_create_from_checkpoint",
]


class LaunchShape(C.Structure):
    _fields_ = [("decide_blocks", C.c_uint32), ("commit_slots", C.c_uint32), ("hour_us", C.c_double)]

# include/epi_surrogate.h
MLP_EXPORTS = [
    "epi_mlp_create", "epi_mlp_destroy", "epi_mlp_last_error", "epi_mlp_set_stream", "epi_mlp_param_count",
    "epi_mlp_get_params", "epi_mlp_set_params", "epi_mlp_set_dataset", "epi_mlp_train", "epi_mlp_gradients",
    "epi_mlp_predict", "epi_mlp_score", "epi_mlp_kernels_launched", "epi_mlp_members",
]


class MlpConfig(C.Structure):
    _fields_ = [
        ("in_dim", C.c_uint32), ("hidden", C.c_uint32), ("hidden_layers", C.c_uint32), ("out_dim", C.c_uint32),
        ("batch", C.c_uint32), ("lr", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float), ("eps", C.c_float),
        ("members", C.c_uint32), ("seed", C.c_uint64),
    ]

_lib = None


class EpiError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def _sig(lib, name, res, args):
    f = getattr(lib, name)
    f.restype = res
    f.argtypes = args


def lib():
    """Load the engine library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"engine library not built: {LIB_PATH} (run epirust_gb300.build.build())")
    L = C.CDLL(LIB_PATH)
    P, V = C.POINTER, C.c_void_p
    _sig(L, "epi_params_from_json", C.c_int, [C.c_char_p, P(EpiParams), C.c_char_p, C.c_size_t])
    _sig(L, "epi_define_geography", C.c_int, [C.c_uint32, P(EpiGeography)])
    _sig(L, "epi_resize_hospital", C.c_int, [P(EpiGeography), C.c_int32, C.c_double, C.c_double])
    _sig(L, "epi_geography_increase_hospital_size", C.c_int, [P(EpiGeography), C.c_uint32])
    _sig(L, "epi_disease_transmission_rate", C.c_double, [P(EpiParams), C.c_uint32])
    _sig(L, "epi_disease_is_to_be_hospitalized", C.c_int, [P(EpiParams), C.c_uint32])
    _sig(L, "epi_interventions_replay", C.c_int, [P(EpiParams), V, C.c_uint32, V, V])
    _sig(L, "epi_outputs_write", C.c_int, [C.c_char_p, C.c_char_p, P(EpiParams), V, C.c_uint32])
    _sig(L, "epi_world_build", C.c_int, [P(EpiParams), V, C.c_size_t, P(EpiGeography)])
    _sig(L, "epi_engine_create", C.c_int, [P(EpiParams), P(V)])
    _sig(L, "epi_engine_create_json", C.c_int, [C.c_char_p, C.c_uint64, P(V)])
    _sig(L, "epi_engine_create_from_records", C.c_int, [P(EpiParams), V, C.c_size_t, P(V)])
    _sig(L, "epi_engine_destroy", None, [V])
    _sig(L, "epi_engine_last_error", C.c_char_p, [V])
    _sig(L, "epi_engine_set_stream", C.c_int, [V, V])
    _sig(L, "epi_engine_simulate", C.c_int, [V, C.c_uint32, P(EpiCounts)])
    _sig(L, "epi_engine_simulate_hours", C.c_int, [V, C.c_uint32, C.c_uint32, V])
    _sig(L, "epi_engine_process_interventions", C.c_int, [V, P(EpiCounts), P(C.c_uint32)])
    _sig(L, "epi_engine_lock_city", C.c_int, [V])
    _sig(L, "epi_engine_unlock_city", C.c_int, [V])
    _sig(L, "epi_engine_vaccinate", C.c_int, [V, C.c_uint32, C.c_double])
    _sig(L, "epi_engine_increase_hospital_size", C.c_int, [V])
    _sig(L, "epi_engine_run", C.c_int, [V, V, C.c_uint32, P(C.c_uint32)])
    _sig(L, "epi_engine_run_until", C.c_int, [V, C.c_uint32, V, C.c_uint32, P(C.c_uint32), P(C.c_uint32)])
    _sig(L, "epi_engine_checkpoint_write", C.c_int, [V, C.c_char_p])
    _sig(L, "epi_engine_create_from_checkpoint", C.c_int, [C.c_char_p, P(V)])
    _sig(L, "epi_engine_write_outputs", C.c_int, [V, C.c_char_p, C.c_char_p])
    _sig(L, "epi_engine_population", C.c_int, [V, P(C.c_uint32)])
    _sig(L, "epi_engine_snapshot", C.c_int, [V, V, C.c_size_t])
    _sig(L, "epi_engine_geography", C.c_int, [V, P(EpiGeography)])
    _sig(L, "epi_engine_check", C.c_int, [V])
    _sig(L, "epi_engine_set_profiling", C.c_int, [V, C.c_int])
    _sig(L, "epi_engine_kernel_stats", C.c_int, [V, P(C.c_uint32), P(C.c_double), C.c_int])
    _sig(L, "epi_engine_kernel_name", C.c_char_p, [C.c_int])
    _sig(L, "epi_engine_kernel_kinds", C.c_int, [])
    _sig(L, "epi_abi_struct_size", C.c_size_t, [C.c_char_p])
    _sig(L, "epi_engine_hour_bytes", C.c_int, [V, C.c_uint32, P(C.c_double)])
    _sig(L, "epi_engine_save_state", C.c_int, [V])
    _sig(L, "epi_engine_restore_state", C.c_int, [V])
    _sig(L, "epi_engine_kernels_launched", C.c_int, [V, P(C.c_uint64)])
    _sig(L, "epi_ensemble_create", C.c_int, [V, C.c_uint32, P(V)])
    _sig(L, "epi_ensemble_destroy", None, [V])
    _sig(L, "epi_ensemble_last_error", C.c_char_p, [V])
    _sig(L, "epi_ensemble_set_stream", C.c_int, [V, V])
    _sig(L, "epi_ensemble_replicates", C.c_int, [V, P(C.c_uint32)])
    _sig(L, "epi_ensemble_run", C.c_int, [V, V, C.c_uint32, V])
    _sig(L, "epi_ensemble_snapshot", C.c_int, [V, C.c_uint32, V, C.c_size_t])
    _sig(L, "epi_ensemble_check", C.c_int, [V])
    _sig(L, "epi_ensemble_save_state", C.c_int, [V])
    _sig(L, "epi_ensemble_restore_state", C.c_int, [V])
    _sig(L, "epi_ensemble_set_profiling", C.c_int, [V, C.c_int])
    _sig(L, "epi_ensemble_kernel_stats", C.c_int, [V, P(C.c_uint32), P(C.c_double), C.c_int])
    _sig(L, "epi_ensemble_kernels_launched", C.c_int, [V, P(C.c_uint64)])
    _sig(L, "epi_ensemble_hour_bytes", C.c_int, [V, C.c_uint32, P(C.c_double)])
    _sig(L, "epi_tick_hour_noalloc", C.c_int, [P(EpiParams), C.c_uint32, C.c_uint32, V, V, V, V, V, V, V, V])
    _sig(L, "epi_engine_autotune", C.c_int, [V, C.c_uint32, P(LaunchShape)])
    _sig(L, "epi_engine_set_launch_shape", C.c_int, [V, P(LaunchShape)])
    _sig(L, "epi_engine_launch_shape", C.c_int, [V, P(LaunchShape)])
    _sig(L, "epi_ensemble_autotune", C.c_int, [V, C.c_uint32, P(LaunchShape)])
    _sig(L, "epi_engine_state_stream_open", C.c_int, [V, C.c_char_p])
    _sig(L, "epi_engine_state_stream_close", C.c_int, [V])
    _sig(L, "epi_population_read_csv", C.c_int, [C.c_char_p, V, C.c_uint32, P(C.c_uint32)])
    _sig(L, "epi_world_build_population", C.c_int, [P(EpiParams), V, C.c_uint32, V, P(EpiGeography)])
    _sig(L, "epi_engine_create_population", C.c_int, [P(EpiParams), V, C.c_uint32, P(V)])
    F = P(C.c_float)
    _sig(L, "epi_mlp_create", C.c_int, [P(MlpConfig), P(V)])
    _sig(L, "epi_mlp_destroy", C.c_int, [V])
    _sig(L, "epi_mlp_last_error", C.c_char_p, [V])
    _sig(L, "epi_mlp_set_stream", C.c_int, [V, V])
    _sig(L, "epi_mlp_param_count", C.c_int, [V, P(C.c_uint64)])
    _sig(L, "epi_mlp_get_params", C.c_int, [V, F])
    _sig(L, "epi_mlp_set_params", C.c_int, [V, F])
    _sig(L, "epi_mlp_set_dataset", C.c_int, [V, F, F, C.c_uint32])
    _sig(L, "epi_mlp_train", C.c_int, [V, C.c_uint32, C.c_uint64, F])
    _sig(L, "epi_mlp_gradients", C.c_int, [V, F, F, C.c_uint32, F, F])
    _sig(L, "epi_mlp_predict", C.c_int, [V, F, C.c_uint32, F])
    _sig(L, "epi_mlp_score", C.c_int, [V, F, C.c_uint32, F, F])
    _sig(L, "epi_mlp_kernels_launched", C.c_int, [V, P(C.c_uint64)])
    _sig(L, "epi_mlp_members", C.c_int, [V, P(C.c_uint32)])
    _lib = L
    return L


def check(rc: int, handle=None) -> None:
    if rc != EPI_OK:
        msg = lib().epi_engine_last_error(handle)
        raise EpiError(rc, msg.decode() if msg else "")
