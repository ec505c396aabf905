"""Surrogate training on GPU-ABM ensembles and the surrogate-screened parameter sweep.

train_on_abm():  Latin-hypercube parameter points -> batched GPU-ABM runs -> daily S/E/I/H/R/D
                 curves (normalised) -> an ensemble of MLPs (one handle, every kernel launch
                 covering all members) trained with Adam on the tensor cores; held-out error
                 against the ABM and against the training-mean curve.
transfer_tune(): the trained ensemble fine-tuned on a few hundred ABM runs of the sweep's
                 (larger) world size.
screened_sweep(): a target curve from hidden parameters (ABM at full size), candidates scored
                 by the fine-tuned surrogate ensemble, the best re-run by the batched ABM with several
                 replicates each together with the candidates the ABM takes over where the
                 members disagree (the fallback), and an ABM-only sweep measured on the same
                 budget of unscreened candidates.

Times are wall-clock around calls that return after the device has finished (the ABM
through epi_ensemble_run, the network through epi_mlp_*).
"""
from __future__ import annotations

import math
import time

import numpy as np

from .surrogate import (PARAMS, Surrogate, screen_with_fallback, compartment_scaling, config_for, denormalise, latin_hypercube,
                        peak_height, relative_peak_error, simulate_curves, uniform_candidates, unit_distance)


def _flops(in_dim: int, hidden: int, layers: int, out_dim: int) -> float:
    """Multiply-adds x 2 of one forward pass (unpadded shapes)."""
    dims = [in_dim] + [hidden] * layers + [out_dim]
    return 2.0 * sum(dims[i] * dims[i + 1] for i in range(len(dims) - 1))


def grid_for(agents: int, density: float = 0.16) -> int:
    return int(math.ceil(math.sqrt(agents / density)))


def train_on_abm(runs: int = 4096, held_out: int = 512, agents: int = 100_000, days: int = 100,
                 members: int = 5, steps: int = 3000, seed: int = 4, hidden: int = 512, hidden_layers: int = 3,
                 batch: int = 256, abm_batch: int = 512, per_agents: int = 100_000, curves: np.ndarray | None = None,
                 noise_runs: int = 128, mean_points: int = 128, mean_replicates: int = 8, grid: int | None = 790):
    """curves: ABM curves of this design computed before (skips the ABM stage).  noise_runs
    held-out points are simulated again with other seeds to measure the ABM's own peak-height
    spread, the floor of any surrogate's error against single runs.  mean_points held-out
    points are run mean_replicates more times and the network's peak height is judged against
    the mean of those runs (the ABM ensemble mean, which is what a sweep compares).  grid: the
    training worlds' grid side (790 for the 100,000-agent runs of the training workload; None
    for ceil(sqrt(agents / 0.16)))."""
    grid = grid_for(agents) if grid is None else grid
    hours = 24 * days + 1
    u = latin_hypercube(runs, len(PARAMS), seed)
    cfgs = [config_for(d, agents, grid, hours, seed=seed * 1_000_003 + i, per_agents=per_agents)
            for i, d in enumerate(denormalise(u))]
    t0 = time.perf_counter()
    y = simulate_curves(cfgs, days, batch=abm_batch) if curves is None else np.asarray(curves, dtype=np.float32)
    t_abm = time.perf_counter() - t0
    n_tr = runs - held_out
    xtr, ytr, xte, yte = u[:n_tr], y[:n_tr], u[n_tr:], y[n_tr:]
    mean, scale = compartment_scaling(ytr, days)
    t0 = time.perf_counter()
    net = Surrogate(in_dim=len(PARAMS), out_dim=6 * days, hidden=hidden, hidden_layers=hidden_layers, batch=batch,
                    seed=seed * 101, members=members)
    net.set_output_scaling(mean, scale)
    net.set_dataset(xtr, ytr)
    losses = np.atleast_2d(net.train(steps, seed=seed * 7))
    t_train = time.perf_counter() - t0
    mean_pred = net.predict(xte)
    mse_net = float(np.mean((mean_pred - yte) ** 2))
    mse_mean = float(np.mean((ytr.mean(axis=0) - yte) ** 2))
    pe = relative_peak_error(mean_pred, yte, days)
    # the ABM's own spread: held-out points run again with other seeds, peak against peak
    n_rep = min(noise_runs, held_out)
    t0 = time.perf_counter()
    rep_cfgs = [config_for(d, agents, grid, hours, seed=seed * 1_000_003 + 500_000 + i, per_agents=per_agents)
                for i, d in enumerate(denormalise(xte[:n_rep]))]
    pe_rep = relative_peak_error(simulate_curves(rep_cfgs, days, batch=abm_batch), yte[:n_rep], days) if n_rep else None
    t_rep = time.perf_counter() - t0
    # the network against the ABM ensemble mean of held-out points (fresh seeds)
    n_mean = min(mean_points, held_out)
    ens_info = None
    if n_mean and mean_replicates:
        t0 = time.perf_counter()
        mean_cfgs = [config_for(d, agents, grid, hours, seed=seed * 1_000_003 + 700_000 + 97 * i + r, per_agents=per_agents)
                     for i, d in enumerate(denormalise(xte[:n_mean])) for r in range(mean_replicates)]
        runs_m = simulate_curves(mean_cfgs, days, batch=abm_batch).reshape(n_mean, mean_replicates, -1)
        ens_mean = runs_m.mean(axis=1)
        pe_mean = relative_peak_error(mean_pred[:n_mean], ens_mean, days)
        # a single ABM run against the same mean (leave-one-out), for scale
        loo = np.stack([(ens_mean * mean_replicates - runs_m[:, r]) / (mean_replicates - 1) for r in range(mean_replicates)],
                       axis=1) if mean_replicates > 1 else None
        pe_single = (np.concatenate([relative_peak_error(runs_m[:, r], loo[:, r], days) for r in range(mean_replicates)])
                     if loo is not None else None)
        ens_info = {
            "points": n_mean, "replicates": mean_replicates, "s": time.perf_counter() - t0,
            "median": float(np.median(pe_mean)), "p90": float(np.quantile(pe_mean, 0.9)),
            "within_5pct": float(np.mean(pe_mean <= 0.05)),
            "single_run_vs_mean_of_others_median": float(np.median(pe_single)) if pe_single is not None else None,
            "note": "network peak height against the mean of mean_replicates fresh ABM runs per held-out point"}
    samples = members * steps * batch
    flop = 3.0 * _flops(len(PARAMS), hidden, hidden_layers, 6 * days) * samples  # forward + backward ~ 3x forward
    info = {
        "runs": runs, "held_out": held_out, "agents": agents, "grid": grid, "days": days,
        "abm_s": t_abm, "abm_agent_hours_per_s": runs * agents * (hours - 1) / t_abm,
        "members": members, "steps": steps, "batch": batch, "train_s": t_train,
        "train_samples_per_s": samples / t_train, "train_tflops": flop / t_train / 1e12,
        "final_loss": [float(l[-20:].mean()) for l in losses],
        "held_out_mse": mse_net, "mean_curve_mse": mse_mean, "gain_vs_mean_curve": mse_mean / max(mse_net, 1e-30),
        "held_out_peak_rel_err_median": float(np.median(pe)), "held_out_peak_rel_err_p90": float(np.quantile(pe, 0.9)),
        "held_out_peak_within_5pct": float(np.mean(pe <= 0.05)),
    }
    if pe_rep is not None:
        info["abm_replicate_peak_rel_err"] = {
            "runs": n_rep, "median": float(np.median(pe_rep)), "p90": float(np.quantile(pe_rep, 0.9)),
            "within_5pct": float(np.mean(pe_rep <= 0.05)), "s": t_rep,
            "note": "the same held-out parameters run again with other seeds: the ABM's own peak-height spread"}
    if ens_info is not None:
        info["held_out_peak_rel_err_vs_abm_mean"] = ens_info
    info["curves"] = y
    return net, info


def transfer_tune(net, agents: int = 1_000_000, points: int = 512, steps: int = 600, lr: float = 2e-4,
                  days: int = 100, seed: int = 31, per_agents: int = 100_000, abm_batch: int = 64):
    """A copy of the surrogate ensemble `net`, trained on smaller worlds, fine-tuned to
    `agents`-agent worlds: `points` Latin-hypercube parameter points run once each by the
    batched ABM at that size, then `steps` Adam steps at learning rate `lr` from net's weights
    (same output scaling, fresh moments).  Per-capita curves of a ten times larger world on a
    grid of the same density are close to, but not the same as, those of the training worlds:
    against 8-replicate ABM means at 1M agents the 100k-agent network's peak height was off by
    4.2 % (median, uniformly drawn points) and 6.0 % (the candidates a sweep keeps), and by
    3.2 % and 3.7 % after 512 runs and 600 steps.  Returns (tuned, info)."""
    grid = grid_for(agents)
    hours = 24 * days + 1
    u = latin_hypercube(points, len(PARAMS), seed)
    t0 = time.perf_counter()
    cfgs = [config_for(d, agents, grid, hours, seed=seed * 1_000_003 + i, per_agents=per_agents)
            for i, d in enumerate(denormalise(u))]
    y = simulate_curves(cfgs, days, batch=abm_batch)
    t_abm = time.perf_counter() - t0
    t0 = time.perf_counter()
    c = net.cfg
    tuned = Surrogate(in_dim=c.in_dim, out_dim=c.out_dim, hidden=c.hidden, hidden_layers=c.hidden_layers, batch=c.batch,
                      lr=lr, seed=seed, members=net.members)
    tuned.set_params(net.get_params())
    tuned.set_output_scaling(net.y_mean, net.y_scale)
    tuned.set_dataset(u, y)
    tuned.train(steps, seed=seed * 7)
    t_train = time.perf_counter() - t0
    return tuned, {"agents": agents, "grid": grid, "points": points, "steps": steps, "lr": lr,
                   "abm_s": t_abm, "train_s": t_train}


def screened_sweep(net, candidates: int = 65_536, keep: int = 256, replicates: int = 8, agents: int = 1_000_000,
                   days: int = 100, seed: int = 99, peak_tolerance: float = 0.05, abm_batch: int = 64,
                   per_agents: int = 100_000, max_fallback: int | None = None, transfer_points: int = 512,
                   transfer_steps: int = 600, transfer_lr: float = 2e-4):
    """The surrogate-screened sweep and an ABM-only sweep of the same budget.

    A target curve comes from the ABM at `agents` agents with hidden parameters (seed).  The
    surrogate ensemble (trained on smaller worlds) is first fine-tuned to `agents`-agent worlds
    on transfer_points ABM runs (transfer_tune; 0 skips it).  It scores every candidate; the
    best `keep` are re-run by the batched ABM with `replicates` replicates each, and so are the
    fallback candidates of screen_with_fallback (outside the kept set, members disagreeing on
    their rank and on their peak by more than peak_tolerance).  The sweep's answer is the
    re-run candidate whose replicate-mean curve is closest to the target.  The screened
    sweep's time counts the fine-tuning runs.  The ABM-only sweep spends the same number of ABM
    runs (re-runs and fine-tuning runs) on unscreened candidates (uniformly drawn): it is
    measured on that sample, and its time for all `candidates` is extrapolated from the
    measured rate."""
    grid = grid_for(agents)
    hours = 24 * days + 1
    rng = np.random.default_rng(seed)
    hidden = rng.random((1, len(PARAMS)))
    t0 = time.perf_counter()
    target = simulate_curves([config_for(denormalise(hidden)[0], agents, grid, hours, seed=seed, per_agents=per_agents)],
                             days)[0]
    t_target = time.perf_counter() - t0
    cand = uniform_candidates(candidates, len(PARAMS), seed + 1)

    # the surrogate fine-tuned to the sweep's world size
    t0 = time.perf_counter()
    tuned, tinfo = (transfer_tune(net, agents, transfer_points, transfer_steps, transfer_lr, days, seed + 3, per_agents,
                                  abm_batch) if transfer_points else (net, None))
    t_transfer = time.perf_counter() - t0

    # surrogate screen (and the candidates handed to the ABM because the members disagree)
    t0 = time.perf_counter()
    sc = screen_with_fallback(tuned, cand, target, keep, days, peak_tolerance, max_fallback)
    t_screen = time.perf_counter() - t0
    rerun = np.concatenate([sc["kept"], sc["fallback"]])
    n_kept = len(sc["kept"])
    sur_mean = tuned.predict(cand[rerun])
    sur_mean_untuned = net.predict(cand[rerun]) if tuned is not net else sur_mean
    # the ABM-only sweep's sample: the same budget of runs (re-runs and fine-tuning runs) on
    # unscreened candidates, whose replicate means also judge the network away from the target
    budget = len(rerun)
    budget_r = budget + (-(-transfer_points // replicates) if tuned is not net else 0)
    rand_idx = np.random.default_rng(seed + 2).choice(candidates, budget_r, replace=False)
    sur_rand = tuned.predict(cand[rand_idx])
    sur_rand_untuned = net.predict(cand[rand_idx]) if tuned is not net else sur_rand
    if tuned is not net:
        tuned.close()

    def abm(points: np.ndarray, base_seed: int) -> np.ndarray:
        cfgs = [config_for(d, agents, grid, hours, seed=base_seed + 97 * i + r, per_agents=per_agents)
                for i, d in enumerate(denormalise(points)) for r in range(replicates)]
        return simulate_curves(cfgs, days, batch=abm_batch).reshape(len(points), replicates, -1)

    t0 = time.perf_counter()
    runs_s = abm(cand[rerun], 10_000)
    t_abm_screened = time.perf_counter() - t0
    mean_s = runs_s.mean(axis=1)
    err_s = ((mean_s - target) ** 2).mean(axis=1)
    pick = int(np.argmin(err_s))

    # the ABM-only sweep, measured on its sample
    t0 = time.perf_counter()
    runs_r = abm(cand[rand_idx], 20_000)
    t_abm_random = time.perf_counter() - t0
    mean_r = runs_r.mean(axis=1)
    err_r = ((mean_r - target) ** 2).mean(axis=1)
    pick_r = int(np.argmin(err_r))

    # the stated criterion: surrogate peak height against the ABM replicate mean, at sweep scale,
    # over the re-run candidates (chosen for predicted curves near the target) and over the
    # unscreened sample (uniform over the parameter ranges)
    peak_err = relative_peak_error(sur_mean, mean_s, days)
    peak_err_untuned = relative_peak_error(sur_mean_untuned, mean_s, days)
    peak_err_u = relative_peak_error(sur_rand, mean_r, days)
    peak_err_u_untuned = relative_peak_error(sur_rand_untuned, mean_r, days)
    abm_only_s = candidates * replicates * t_abm_random / (budget_r * replicates)
    screened_s = t_transfer + t_screen + t_abm_screened
    top = np.argsort(err_s)[:8]
    top_r = np.argsort(err_r)[:8]

    def per_param(u: np.ndarray) -> dict:
        """|recovered - hidden| per parameter, in units of its range."""
        return {p.name: round(float(abs(u[k] - hidden[0, k])), 4) for k, p in enumerate(PARAMS)}

    def fit_weighted(points: np.ndarray, errs: np.ndarray) -> np.ndarray:
        """Mean of the best eight candidates weighted by 1 / curve error."""
        w = 1.0 / np.maximum(errs, 1e-30)
        return (points * w[:, None]).sum(axis=0) / w.sum()

    est_s = fit_weighted(cand[rerun][top], err_s[top])
    est_r = fit_weighted(cand[rand_idx][top_r], err_r[top_r])
    return {
        "candidates": candidates, "keep": n_kept, "replicates": replicates, "agents": agents, "grid": grid,
        "days": days, "target_peak": float(peak_height(target[None], days)[0]),
        "kept_abm_peak_median": float(np.median(peak_height(mean_s[:n_kept], days))), "target_abm_s": t_target, "screen_s": t_screen, "abm_screened_s": t_abm_screened,
        "abm_random_s": t_abm_random, "abm_run_s": t_abm_screened / (budget * replicates),
        "abm_agent_hours_per_s": budget * replicates * agents * (hours - 1) / t_abm_screened,
        "kept_members_disagree": int(sc["kept_flagged"].sum()),
        "fallback_uncertain_rank": sc["uncertain"], "fallback_eligible": sc["fallback_eligible"],
        "fallback_rerun_by_abm": int(len(sc["fallback"])),
        "pick_from_fallback": bool(pick >= n_kept),
        "fallback_best_curve_mse": float(err_s[n_kept:].min()) if budget > n_kept else None,
        "surrogate_peak_rel_err_median": float(np.median(peak_err[:n_kept])),
        "surrogate_peak_within_5pct": float(np.mean(peak_err[:n_kept] <= 0.05)),
        "surrogate_peak_rel_err_median_fallback": float(np.median(peak_err[n_kept:])) if budget > n_kept else None,
        "surrogate_peak_rel_err_median_untuned": float(np.median(peak_err_untuned[:n_kept])),
        "surrogate_peak_rel_err_uniform": {
            "points": int(budget_r), "median": float(np.median(peak_err_u)), "p90": float(np.quantile(peak_err_u, 0.9)),
            "within_5pct": float(np.mean(peak_err_u <= 0.05)), "median_untuned": float(np.median(peak_err_u_untuned)),
            "note": "network peak height against the replicate means of the ABM-only sample's uniformly drawn "
                    "candidates at sweep scale"},
        "transfer": dict(tinfo, s=t_transfer) if tinfo else None,
        "screened_best_param_err": float(unit_distance(cand[rerun][pick], hidden)[0]),
        "screened_top8_param_err_mean": float(unit_distance(cand[rerun][top], hidden).mean()),
        "screened_best_curve_mse": float(err_s[pick]),
        "screened_best_peak_rel_err_vs_target": float(relative_peak_error(mean_s[pick:pick + 1], target[None], days)[0]),
        "screened_best_param_abs_err": per_param(cand[rerun][pick]),
        "screened_top8_weighted_param_err": float(unit_distance(est_s, hidden)[0]),
        "screened_top8_weighted_param_abs_err": per_param(est_s),
        "abm_only_best_param_err": float(unit_distance(cand[rand_idx][pick_r], hidden)[0]),
        "abm_only_top8_weighted_param_err": float(unit_distance(est_r, hidden)[0]),
        "abm_only_top8_param_err_mean": float(unit_distance(cand[rand_idx][top_r], hidden).mean()),
        "abm_only_best_curve_mse": float(err_r[pick_r]),
        "abm_only_best_peak_rel_err_vs_target": float(relative_peak_error(mean_r[pick_r:pick_r + 1], target[None],
                                                                           days)[0]),
        # candidates whose ABM replicate-mean peak lies within 5 % of the target's, by stage
        "screened_within_5pct_of_target_peak": int((relative_peak_error(mean_s, target[None], days) <= 0.05).sum()),
        "abm_only_within_5pct_of_target_peak": int((relative_peak_error(mean_r, target[None], days) <= 0.05).sum()),
        "abm_only_sample_runs": budget_r * replicates,
        "abm_only_sweep_s_measured_sample": t_abm_random,
        "abm_only_sweep_s_extrapolated": abm_only_s, "screened_sweep_s": screened_s,
        "sweep_speedup": abm_only_s / screened_s,
    }
