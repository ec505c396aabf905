"""Launch shapes and the autotuner: the tick's results never depend on the k_decide grid or
the agents per k_commit thread (1..8), and autotuning leaves the world where it found it."""
import json

import numpy as np
import pytest

from helpers import COVID_FAST, make_config, rows_to_array

pytestmark = pytest.mark.gpu


def _engine(cfg):
    from epirust_gb300 import Config, Epidemiology

    return Epidemiology(Config(json.dumps(cfg)))


def _rows(r):
    return np.stack([r[k] for k in r.dtype.names], axis=1).astype(np.int64)


def test_every_launch_shape_gives_the_same_hours(gpu, oracle_mod):
    cfg = make_config(n=6000, grid=130, hours=24 * 6, seed=31, disease=COVID_FAST, starting=(2, 2, 2, 30))
    sim = oracle_mod.O1(oracle_mod.params_from_config(cfg))
    want = rows_to_array(sim.run(1, 130, interventions=False, stop=False))
    n_chunks = (6000 + 255) // 256
    for blocks, slots in [(None, None), (n_chunks, 1), (1, 2), (7, 4), (3, 5), (n_chunks, 8), (2, 3)]:
        eng = _engine(cfg)
        if blocks:
            eng.set_launch_shape(blocks, slots)
            assert eng.launch_shape() == {"decide_blocks": blocks, "commit_slots": slots}
        got = _rows(eng.simulate_hours(1, 129))
        assert (got == want).all(), (blocks, slots)
        a, b = eng.snapshot(), sim.export()
        assert (a.view(np.uint8) == b.view(np.uint8)).all(), (blocks, slots)
        eng.close()


def test_bad_launch_shapes_are_refused(gpu):
    from epirust_gb300 import EpiError

    eng = _engine(make_config(n=3000, grid=120, seed=1))
    for blocks, slots in [(0, 4), (10**6, 4), (4, 0), (4, 9)]:
        with pytest.raises(EpiError, match="ARG"):
            eng.set_launch_shape(blocks, slots)
    eng.close()


def test_autotune_keeps_the_world_and_the_run(gpu, oracle_mod):
    cfg = make_config(n=5000, grid=120, hours=24 * 20, seed=32, disease=COVID_FAST, starting=(0, 0, 5, 20),
                      interventions=[{"Lockdown": {"at_number_of_infections": 30, "essential_workers_population": 0.1}}])
    eng = _engine(cfg)
    before = eng.snapshot().copy()
    launched = eng.kernels_launched()
    shape = eng.autotune(24)
    assert 1 <= shape["commit_slots"] <= 8 and shape["decide_blocks"] >= 1 and shape["hour_us"] > 0
    assert eng.launch_shape() == {"decide_blocks": shape["decide_blocks"], "commit_slots": shape["commit_slots"]}
    assert (eng.snapshot().view(np.uint8) == before.view(np.uint8)).all()
    assert eng.kernels_launched() == launched
    got = _rows(eng.run())
    want = rows_to_array(oracle_mod.O1(oracle_mod.params_from_config(cfg)).run(1, cfg["hours"], True, True))
    assert got.shape == want.shape and (got == want).all()
    eng.close()


def test_ensemble_autotune_keeps_replicates_equal_to_single_engines(gpu):
    from epirust_gb300 import Config, Ensemble

    cfgs = [make_config(n=n, grid=g, hours=24 * 8, seed=40 + i, disease=COVID_FAST, starting=(1, 1, 1, 10))
            for i, (n, g) in enumerate([(2000, 100), (700, 60), (4100, 120)])]
    ens = Ensemble([Config(json.dumps(c)).params for c in cfgs])
    shape = ens.autotune(12)
    assert 1 <= shape["commit_slots"] <= 8
    rows = ens.run()
    for c, r in zip(cfgs, rows):
        eng = _engine(c)
        assert (_rows(r) == _rows(eng.run())).all()
        eng.close()
    ens.close()
