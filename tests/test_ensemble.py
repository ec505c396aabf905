"""The batched ensemble: R worlds of uneven size in one launch per hour.

Each replicate must evolve exactly as a lone engine created from the same parameters
(hourly counts, and the final agents when neither run stopped early), and the lone engine is
itself pinned to the oracle by test_gpu_parity.py.
"""
import json

import numpy as np
import pytest

from helpers import COVID_FAST, make_config

pytestmark = pytest.mark.gpu


def _mixed_configs():
    return [
        make_config(n=3000, grid=120, hours=24 * 12, seed=1, disease=COVID_FAST, starting=(5, 5, 5, 20)),
        make_config(n=700, grid=60, hours=24 * 20, seed=2, starting=(0, 0, 0, 3)),
        make_config(n=5000, grid=130, hours=24 * 15, seed=3, disease=COVID_FAST, starting=(0, 0, 10, 30),
                    interventions=[{"Lockdown": {"at_number_of_infections": 20, "essential_workers_population": 0.1}},
                                   {"Vaccinate": {"at_hour": 100, "percent": 0.3}}]),
        make_config(n=257, grid=50, hours=24 * 9 + 5, seed=4, disease=COVID_FAST, starting=(2, 2, 2, 2)),
        make_config(n=4096, grid=110, hours=24 * 14, seed=5, disease=COVID_FAST, starting=(0, 0, 30, 30), occupancy=0.5,
                    interventions=[{"BuildNewHospital": {"spread_rate_threshold": 5}}]),
        make_config(n=1200, grid=80, hours=24 * 30, seed=6, starting=(0, 0, 0, 1)),
    ]


def test_ensemble_replicates_equal_single_engines(gpu):
    from epirust_gb300 import Config, Ensemble, Epidemiology

    cfgs = _mixed_configs()
    params = [Config(json.dumps(c)).params for c in cfgs]
    ens = Ensemble(params)
    rows = ens.run()
    ens.check_invariants()
    for r, cfg in enumerate(cfgs):
        eng = Epidemiology(Config(json.dumps(cfg)))
        want = eng.run()
        got = rows[r]
        assert len(got) == len(want), (r, len(got), len(want))
        assert (got == want).all(), r
        a, b = ens.snapshot(r), eng.snapshot()  # also after an early stop
        assert (a.view(np.uint8) == b.view(np.uint8)).all(), r
        eng.close()


def test_ensemble_rerun_from_saved_state_repeats(gpu):
    from epirust_gb300 import Config, Ensemble

    params = [Config(json.dumps(c)).params for c in _mixed_configs()[:4]]
    ens = Ensemble(params)
    ens.save_state()
    first = ens.run()
    ens.restore_state()
    second = ens.run()
    for a, b in zip(first, second):
        assert (a == b).all()


def test_replicate_generator_shapes_small(gpu):
    """The 256-replicate generator (log-uniform populations, sqrt grids) at 16 small replicates."""
    from epirust_gb300 import Ensemble, Epidemiology
    from epirust_gb300.workloads import ensemble_params

    params = ensemble_params(replicates=16, hours=24 * 10, n_min=2e3, n_max=2e4)
    ens = Ensemble(params)
    rows = ens.run()
    ens.check_invariants()
    for r in (0, 7, 15):
        eng = Epidemiology(params[r])
        assert (rows[r] == eng.run()).all(), r
        eng.close()
    for p, rr in zip(params, rows):
        tot = rr["susceptible"].astype(np.int64) + rr["exposed"] + rr["infected"] + rr["hospitalized"] + \
            rr["recovered"] + rr["deceased"]
        assert (tot == p.number_of_agents).all()
