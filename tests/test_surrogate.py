"""The learned surrogate: the CPU oracle pinned by finite differences, the sweep helpers on
the host, and (on the GPU) the tcgen05 network against the oracle -- forward, gradients,
Adam -- plus what the trained network gains over the method without it."""
import math

import numpy as np
import pytest

from oracle import mlp as omlp


def _rand_layers(shapes, rng, scale=1.0):
    return [(rng.uniform(-scale, scale, (n, k)) / math.sqrt(k), rng.uniform(-scale, scale, n) / math.sqrt(k))
            for n, k in shapes]


# ---------------------------------------------------------------- CPU: the oracle itself
def test_bf16_rounding_known_values():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -2.5, 3.0e-39, 65504.0], dtype=np.float32)
    got = omlp.bf16(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: even mantissa wins (1.0); 1 + 3*2^-8 rounds up
    want = [1.0, 1.0, 1.0 + 2 ** -6, 1.0, -2.5, float(np.float32(3.0e-39)), 65536.0]
    assert got[0] == want[0] and got[1] == want[1] and got[3] == want[3] and got[4] == want[4]
    assert got[2] == 1.0 + 2 * 2 ** -7
    assert got[6] == want[6]
    assert abs(got[5] - want[5]) <= 2 ** -133


def test_oracle_gradients_match_central_differences():
    rng = np.random.default_rng(5)
    shapes = omlp.layer_shapes(3, 6, 2, 5)
    layers = _rand_layers(shapes, rng, 2.0)
    x, t = rng.normal(size=(7, 3)), rng.normal(size=(7, 5))
    _, grads = omlp.loss_and_gradients(layers, x, t, emulate=False)
    picks = [(l, kind, idx) for l, (n, k) in enumerate(shapes)
             for kind, idx in (("w", (n - 1, k - 1)), ("w", (0, 0)), ("b", (n // 2,)))]
    num = omlp.numeric_gradients(layers, x, t, picks)
    ana = np.array([grads[l][0][idx] if kind == "w" else grads[l][1][idx] for l, kind, idx in picks])
    assert np.allclose(ana, num, rtol=1e-6, atol=1e-9), np.c_[ana, num]


def test_oracle_emulated_rounding_is_close_to_exact():
    rng = np.random.default_rng(6)
    layers = _rand_layers(omlp.layer_shapes(8, 64, 2, 20), rng)
    x, t = rng.random((32, 8)), rng.random((32, 20))
    le, ge = omlp.loss_and_gradients(layers, x, t, emulate=True)
    lx, gx = omlp.loss_and_gradients(layers, x, t, emulate=False)
    assert abs(le - lx) / lx < 0.02
    for (a, _), (b, _) in zip(ge, gx):
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < 0.05


def test_adam_oracle_first_step_is_signed_lr():
    g = np.array([3.0, -0.5, 1e-3])
    p, m, v = omlp.adam_step(np.zeros(3), g, np.zeros(3), np.zeros(3), 1, 1e-3, 0.9, 0.999, 1e-8)
    assert np.allclose(p, -1e-3 * np.sign(g), rtol=1e-4)


# ---------------------------------------------------------------- CPU: sweep helpers
def test_latin_hypercube_one_point_per_stratum():
    from epirust_gb300.surrogate import latin_hypercube

    u = latin_hypercube(64, 8, seed=3)
    assert u.shape == (64, 8) and (u >= 0).all() and (u < 1).all()
    for j in range(8):
        assert sorted(np.floor(u[:, j] * 64).astype(int)) == list(range(64))


def test_config_for_maps_every_parameter(engine_built):
    from epirust_gb300.surrogate import PARAMS, config_for, denormalise
    from epirust_gb300.workloads import params_of

    u = np.linspace(0.1, 0.9, len(PARAMS))
    d = denormalise(u)[0]
    p = params_of(config_for(d, 2000, 120, 24 * 10 + 1, seed=4))
    assert p.regular_transmission_rate == pytest.approx(d["regular_transmission_rate"])
    assert p.high_transmission_rate == pytest.approx(d["high_transmission_rate"])
    assert p.death_rate == pytest.approx(d["death_rate"])
    assert p.has_lockdown == 1 and p.lockdown_at_number_of_infections == d["lockdown_at_number_of_infections"]
    assert p.essential_workers_population == pytest.approx(d["essential_workers_population"])
    assert p.n_vaccinations == 1 and p.vaccination_at_hour[0] == d["vaccination_hour"]
    assert p.vaccination_percent[0] == pytest.approx(d["vaccination_percent"])
    assert p.exposed == d["initial_infected"]
    assert all(isinstance(d[q.name], int) for q in PARAMS if q.integer)


def test_curves_from_rows_samples_days_and_keeps_last_counts():
    from epirust_gb300 import COUNTS_DTYPE
    from epirust_gb300.surrogate import curves_from_rows

    rows = np.zeros(30, dtype=COUNTS_DTYPE)
    rows["hour"] = np.arange(1, 31)
    rows["infected"] = np.arange(1, 31)
    rows["susceptible"] = 100 - np.arange(1, 31)
    c = curves_from_rows(rows, 100, 3)  # day 1 at hour 24; days 2, 3 after the run stopped
    assert c.shape == (6, 3)
    assert c[2, 0] == 24 / 100 and c[2, 1] == 30 / 100 and c[2, 2] == 30 / 100
    assert c[0, 0] == 76 / 100


# ---------------------------------------------------------------- GPU: network vs oracle
C4 = dict(in_dim=8, out_dim=600, hidden=512, hidden_layers=3, batch=256)


def _net(gpu, **kw):
    from epirust_gb300.surrogate import Surrogate

    cfg = dict(C4)
    cfg.update(kw)
    return Surrogate(**cfg)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 128, 300])
def test_forward_matches_oracle(gpu, n):
    """predict() (tcgen05 products, padded rows) equals the BF16-emulating oracle.
    Tolerance: relative Frobenius error 2e-3 (FP32 vs float64 accumulation and the odd BF16
    rounding of an activation that lands on the other side of a tie)."""
    rng = np.random.default_rng(n)
    net = _net(gpu, seed=1)
    layers = _rand_layers(omlp.layer_shapes(8, 512, 3, 600), rng)
    net.set_params(omlp.flatten(layers))
    x = rng.random((n, 8))
    got = net.predict(x).astype(np.float64)
    want, _ = omlp.forward(omlp.unflatten(net.get_params(), net.shapes), x, emulate=True)
    err = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert err < 2e-3, err
    s = net.score(x, want[0])
    assert np.allclose(s, ((got - want[0]) ** 2).sum(axis=1), rtol=1e-3, atol=1e-6)
    assert net.kernels_launched() > 0
    net.close()


@pytest.mark.gpu
def test_smaller_calls_after_larger_ones(gpu):
    """A handle's prediction buffers keep the rows of its largest call so far.  Predictions of a
    later, smaller call equal, member for member and bit for bit, those of a fresh handle and
    the same rows of the larger call (every member's rows start at the same place in every
    buffer, whatever the call's size); so do scores, up to the order in which the output tiles'
    partial sums are added (relative 1e-5)."""
    rng = np.random.default_rng(5)
    x = rng.random((1000, 8))
    target = rng.random(600)
    a, b = _net(gpu, seed=2, members=3), _net(gpu, seed=2, members=3)
    big = a.predict_members(x)
    big_score = a.score_members(x, target)
    for n in (100, 300, 129):
        small = a.predict_members(x[:n])
        assert np.array_equal(small, big[:, :n]), n
        assert np.allclose(a.score_members(x[:n], target), big_score[:, :n], rtol=1e-5, atol=0), n
    assert np.array_equal(b.predict_members(x[:300]), big[:, :300])
    assert np.allclose(b.score_members(x[:129], target), big_score[:, :129], rtol=1e-5, atol=0)
    a.close()
    b.close()


@pytest.mark.gpu
def test_gradients_match_oracle(gpu):
    """Loss and every layer's weight and bias gradients of one 256-sample minibatch.
    Tolerance: loss 1e-3 relative; gradients 2e-2 relative Frobenius per tensor (BF16 dZ
    rounding amplifies the accumulation-order differences)."""
    rng = np.random.default_rng(2)
    net = _net(gpu, seed=2)
    layers = _rand_layers(omlp.layer_shapes(8, 512, 3, 600), rng)
    net.set_params(omlp.flatten(layers))
    layers = omlp.unflatten(net.get_params(), net.shapes)
    x, t = rng.random((256, 8)), rng.random((256, 600)) * 0.5
    loss, g = net.gradients(x, t)
    want_loss, want = omlp.loss_and_gradients(layers, x, t, emulate=True)
    assert loss == pytest.approx(want_loss, rel=1e-3)
    got = omlp.unflatten(g, net.shapes)
    for l, ((gw, gb), (ww, wb)) in enumerate(zip(got, want)):
        assert np.linalg.norm(gw - ww) / np.linalg.norm(ww) < 2e-2, l
        assert np.linalg.norm(gb - wb) / np.linalg.norm(wb) < 2e-2, l
    net.close()


@pytest.mark.gpu
def test_adam_step_matches_oracle(gpu):
    """One training step on a one-minibatch set == oracle Adam on the GPU's own gradients."""
    rng = np.random.default_rng(3)
    net = _net(gpu, seed=3)
    p0 = net.get_params().astype(np.float64)
    x, t = rng.random((256, 8)), rng.random((256, 600)) * 0.5
    _, g = net.gradients(x, t)
    net.set_dataset(x, t)
    losses = net.train(1, seed=0)
    p1 = net.get_params().astype(np.float64)
    want, _, _ = omlp.adam_step(p0, g.astype(np.float64), 0.0, 0.0, 1, 1e-3, 0.9, 0.999, 1e-8)
    # the update is lr * g / (|g| + eps): compare it where |g| is well above eps
    sel = np.abs(g) > 1e-6
    assert np.allclose(p1[sel], want[sel], rtol=0, atol=2e-6)
    assert losses[0] > 0
    net.close()


@pytest.mark.gpu
def test_training_fits_a_smooth_map(gpu):
    rng = np.random.default_rng(4)
    x = rng.random((2048, 8))
    basis = np.linspace(0, 1, 600)
    y = 0.5 + 0.25 * np.sin(np.outer(x[:, 0] * 3 + x[:, 1], basis * 6) + x[:, 2:3] * 2) * x[:, 3:4]
    net = _net(gpu, seed=4)
    net.set_dataset(x, y)
    losses = net.train(400, seed=1)
    assert np.isfinite(losses).all()
    assert losses[-20:].mean() < 0.05 * losses[:5].mean(), (losses[:5], losses[-5:])
    pred = net.predict(x[:256])
    assert np.mean((pred - y[:256]) ** 2) == pytest.approx(losses[-20:].mean(), rel=1.0)
    net.close()


@pytest.mark.gpu
def test_surrogate_gain_over_method_without_it(gpu):
    """Train on GPU-ABM ensembles (small worlds, 20 days), then (1) held-out curves: the
    network's error is well under the error of predicting the training mean; (2) a sweep
    for a hidden target: with the same ABM budget, surrogate-screened candidates land closer
    to the target than unscreened ones."""
    from epirust_gb300.surrogate import (Surrogate, config_for, denormalise, latin_hypercube, screen,
                                         simulate_curves, uniform_candidates, unit_distance)

    days, agents, grid = 20, 3000, 137
    hours = 24 * days + 1
    u = latin_hypercube(768, 8, seed=7)
    cfgs = [config_for(d, agents, grid, hours, seed=1000 + i) for i, d in enumerate(denormalise(u))]
    y = simulate_curves(cfgs, days)
    xtr, ytr, xte, yte = u[:640], y[:640], u[640:], y[640:]
    net = Surrogate(in_dim=8, out_dim=6 * days, hidden=256, hidden_layers=2, batch=128, seed=10, members=3)
    net.set_dataset(xtr, ytr)
    net.train(1500, seed=0)
    pred = net.predict(xte)
    mse_net = np.mean((pred - yte) ** 2)
    mse_mean = np.mean((ytr.mean(axis=0) - yte) ** 2)
    assert mse_net < 0.5 * mse_mean, (mse_net, mse_mean)

    hidden = np.array([[0.7, 0.6, 0.3, 0.8, 0.4, 0.9, 0.2, 0.7]])
    target = simulate_curves([config_for(denormalise(hidden)[0], agents, grid, hours, seed=99)], days)[0]
    cand = uniform_candidates(4096, 8, seed=8)
    best, _, _ = screen(net, cand, target, keep=16, days=days)
    budget = [config_for(d, agents, grid, hours, seed=2000 + i) for i, d in enumerate(denormalise(cand[best]))]
    rand = cand[np.random.default_rng(9).choice(len(cand), 16, replace=False)]
    budget += [config_for(d, agents, grid, hours, seed=3000 + i) for i, d in enumerate(denormalise(rand))]
    abm = simulate_curves(budget, days)
    err = ((abm - target) ** 2).mean(axis=1)
    assert err[:16].min() <= err[16:].min()
    assert np.median(err[:16]) < np.median(err[16:])

    # the ABM fallback: candidates outside the kept set that some member would keep and whose
    # members' peaks disagree by more than 5 % are handed to the ABM, most promising first
    from epirust_gb300.surrogate import member_peak_spread, screen_with_fallback

    sc = screen_with_fallback(net, cand, target, keep=16, days=days, peak_tolerance=0.05, max_fallback=64)
    assert np.array_equal(sc["kept"], best)
    fb = sc["fallback"]
    assert len(fb) > 0 and not set(fb.tolist()) & set(best.tolist())
    assert len(fb) == min(64, sc["fallback_eligible"]) and sc["fallback_eligible"] <= sc["uncertain"]
    members = net.score_members(cand, target)
    cut = members.mean(axis=0)[best].max()
    assert (members[:, fb].min(axis=0) <= cut).all()
    assert (member_peak_spread(net, cand[fb], days) > 0.05).all()
    net.close()


@pytest.mark.gpu
def test_members_equal_lone_networks(gpu):
    """Member m of a 3-member handle (one launch per kernel for all members) equals a
    one-member network created with seed + m and trained with shuffle seed + m: parameters
    and predictions bit for bit (products, bias reductions and Adam are deterministic);
    scores and losses within float-atomic summation order."""
    rng = np.random.default_rng(5)
    shape = dict(out_dim=120, hidden=256, hidden_layers=2, batch=128)
    x, y = rng.random((640, 8)), rng.random((640, 120)) * 0.5
    xp = rng.random((300, 8))
    ens = _net(gpu, seed=20, members=3, **shape)
    ens.set_dataset(x, y)
    le = ens.train(40, seed=7)
    pe, ye, se = ens.get_params(), ens.predict_members(xp), ens.score_members(xp, y[0])
    assert le.shape == (3, 40) and pe.shape == (3, ens.n_params) and ye.shape == (3, 300, 120)
    assert np.allclose(ens.predict(xp), ye.mean(axis=0), rtol=1e-6, atol=1e-7)
    g_loss, g = ens.gradients(x[:128], y[:128])
    for m in range(3):
        one = _net(gpu, seed=20 + m, **shape)
        one.set_dataset(x, y)
        lo = one.train(40, seed=7 + m)
        assert np.array_equal(one.get_params(), pe[m]), m
        assert np.array_equal(one.predict(xp), ye[m]), m
        assert np.allclose(one.score(xp, y[0]), se[m], rtol=1e-5, atol=1e-7), m
        assert np.allclose(lo, le[m], rtol=1e-4), m
        l1, g1 = one.gradients(x[:128], y[:128])
        assert np.array_equal(g1, g[m]) and l1 == pytest.approx(float(g_loss[m]), rel=1e-5), m
        one.close()
    # set_params on the stack == per-member set_params
    ens.set_params(pe[::-1].copy())
    assert np.array_equal(ens.get_params(), pe[::-1])
    ens.close()


@pytest.mark.gpu
def test_transfer_tune_fits_larger_worlds(gpu):
    """transfer_tune: a copy of the ensemble (weights and output scaling bit for bit before any
    step) fine-tuned on ABM runs of a ten times larger world predicts held-out curves of that
    world better than the network trained on the small worlds alone."""
    from epirust_gb300.surrogate import (Surrogate, compartment_scaling, config_for, denormalise, latin_hypercube,
                                         simulate_curves, uniform_candidates)
    from epirust_gb300.sweep import grid_for, transfer_tune

    days, small, big = 20, 2000, 20000
    hours = 24 * days + 1
    u = latin_hypercube(640, 8, seed=11)
    y = simulate_curves([config_for(d, small, grid_for(small), hours, seed=5000 + i, per_agents=small)
                         for i, d in enumerate(denormalise(u))], days)
    net = Surrogate(in_dim=8, out_dim=6 * days, hidden=256, hidden_layers=2, batch=128, seed=3, members=2)
    net.set_output_scaling(*compartment_scaling(y, days))
    net.set_dataset(u, y)
    net.train(1000, seed=1)

    ue = uniform_candidates(64, 8, seed=21)
    copy, info0 = transfer_tune(net, agents=big, points=4, steps=0, days=days, seed=13, per_agents=small)
    assert np.array_equal(copy.predict_members(ue), net.predict_members(ue))
    assert np.array_equal(copy.get_params(), net.get_params())
    copy.close()

    tuned, info = transfer_tune(net, agents=big, points=256, steps=400, lr=2e-4, days=days, seed=13,
                                per_agents=small, abm_batch=256)
    assert info["points"] == 256 and info["agents"] == big and info["grid"] == grid_for(big) and info["abm_s"] > 0
    yb = simulate_curves([config_for(d, big, grid_for(big), hours, seed=9000 + i, per_agents=small)
                          for i, d in enumerate(denormalise(ue))], days)
    mse_tuned = np.mean((tuned.predict(ue) - yb) ** 2)
    mse_small = np.mean((net.predict(ue) - yb) ** 2)
    assert mse_tuned < mse_small, (mse_tuned, mse_small)
    tuned.close()
    net.close()
