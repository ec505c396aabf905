"""GB300-native engine tick for EpiRust-style agent-based epidemic simulations.

The hourly tick (movement with deterministic cell claims, Moore-neighbour infection, the
disease state machine, interventions and the counts reduction) runs as hand-written sm_103a
CUDA kernels behind the C ABI of include/epi_engine.h; this package is the Python host of
that ABI.
"""
from ._lib import AGENT_DTYPE, COUNTS_DTYPE, EpiError, EpiParams, lib  # noqa: F401
from .engine import Config, Counts, Ensemble, Epidemiology, define_geography, world_build  # noqa: F401
