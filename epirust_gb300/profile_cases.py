"""Small, fixed workloads for profilers (ncu) and quick timing: each runs one hot path of the
package and exits.

    python -m epirust_gb300.profile_cases tick --agents 1000000 --grid 2500 --hours 48
        the 1M-agent / 2,500-grid small-pox world (tests/golden/small_pox_1m_2500.json) resized, hours 1..hours-1
        through simulate_hours (one CUDA graph per call); --events adds CUDA events per kernel,
        --shape 608,2 sets the launch shape (k_decide grid, agents per k_commit thread)
    python -m epirust_gb300.profile_cases run [--shape 608,2]
        the 1M-agent / 2,500-grid run loop once (bench.py's step: 4,799 hours with the interventions)
    python -m epirust_gb300.profile_cases ensemble --replicates 256 --hours 49
        the 256-replicate ensemble (30.6M agents) through the run loop, hours
        1..hours-1
    python -m epirust_gb300.profile_cases mlp-train --steps 30 [--members M]
        the surrogate network 8 -> 512 x 3 -> 600 (M members in one handle), batch 256, on a
        seeded synthetic set of 4,096 samples: `steps` Adam steps (one graph replay each)
    python -m epirust_gb300.profile_cases mlp-screen --candidates 65536 [--members M]
        the network (M members) scoring `candidates` parameter vectors against a curve
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
WORLD_1M = os.path.join(os.path.dirname(HERE), "tests", "golden", "small_pox_1m_2500.json")


def tick(args) -> dict:
    from .engine import Config, Epidemiology

    with open(WORLD_1M) as f:
        cfg = json.load(f)
    cfg["population"]["Auto"]["number_of_agents"] = args.agents
    cfg["geography_parameters"]["grid_size"] = args.grid
    eng = Epidemiology(Config(json.dumps(cfg)))
    if args.shape:  # "blocks,slots": the k_decide grid and agents per k_commit thread
        eng.set_launch_shape(*(int(v) for v in args.shape.split(",")))
    eng.set_profiling(args.events)
    t0 = time.perf_counter()
    eng.simulate_hours(1, args.hours - 1)
    dt = time.perf_counter() - t0
    out = {"hours": args.hours - 1, "s": dt, "agent_hours_per_s": args.agents * (args.hours - 1) / dt}
    if args.events:
        out["kernels"] = {k: v for k, v in eng.kernel_stats().items() if v[0]}
    eng.close()
    return out


def run(args) -> dict:
    """The 1M-agent run loop (2,500 grid, 4,800 h, lockdown, vaccination and the
    hospital build): the workload of bench.py's step, once, at the launch shape given."""
    from .engine import Config, Epidemiology

    with open(WORLD_1M) as f:
        cfg = json.load(f)
    eng = Epidemiology(Config(json.dumps(cfg)))
    if args.shape:
        eng.set_launch_shape(*(int(v) for v in args.shape.split(",")))
    t0 = time.perf_counter()
    rows = eng.run()
    dt = time.perf_counter() - t0
    n = cfg["population"]["Auto"]["number_of_agents"]
    eng.close()
    return {"hours": len(rows), "s": dt, "agent_hours_per_s": n * len(rows) / dt}


def ensemble(args) -> dict:
    """The 256-replicate ensemble (10k-500k agents each) through the run loop for
    hours 1..hours-1."""
    from .engine import Ensemble
    from .workloads import ensemble_params

    params = ensemble_params(replicates=args.replicates)
    for p in params:
        p.hours = args.hours
    ens = Ensemble(params)
    t0 = time.perf_counter()
    rows = ens.run()
    dt = time.perf_counter() - t0
    ah = sum(float(p.number_of_agents) * len(r) for p, r in zip(params, rows))
    ens.close()
    return {"replicates": len(params), "hours": args.hours - 1, "s": dt, "agent_hours_per_s": ah / dt}


def _net(members: int = 1):
    from .surrogate import Surrogate

    return Surrogate(in_dim=8, out_dim=600, hidden=512, hidden_layers=3, batch=256, seed=1, members=members)


def mlp_train(args) -> dict:
    rng = np.random.default_rng(0)
    x = rng.random((4096, 8))
    y = np.sin(x @ rng.normal(size=(8, 600))) * 0.5
    net = _net(args.members)
    net.set_dataset(x, y)
    t0 = time.perf_counter()
    losses = np.atleast_2d(net.train(args.steps, seed=0))
    dt = time.perf_counter() - t0
    net.close()
    return {"steps": args.steps, "members": args.members, "s": dt, "ms_per_step": 1000 * dt / max(args.steps, 1),
            "first_loss": float(losses[:, 0].mean()), "last_loss": float(losses[:, -1].mean())}


def mlp_screen(args) -> dict:
    rng = np.random.default_rng(1)
    net = _net(args.members)
    cand = rng.random((args.candidates, 8))
    target = rng.random(600)
    net.score(cand[:1024], target)  # warm-up (buffers, tensor maps)
    t0 = time.perf_counter()
    s = net.score(cand, target)
    dt = time.perf_counter() - t0
    net.close()
    return {"candidates": args.candidates, "s": dt, "best": float(s.min())}


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    sub = ap.add_subparsers(dest="case", required=True)
    t = sub.add_parser("tick")
    t.add_argument("--agents", type=int, default=1_000_000)
    t.add_argument("--grid", type=int, default=2500)
    t.add_argument("--hours", type=int, default=48)
    t.add_argument("--events", action="store_true")
    t.add_argument("--shape", default="", help="launch shape 'blocks,slots' (k_decide grid, agents per k_commit thread)")
    r = sub.add_parser("run")
    r.add_argument("--shape", default="608,2", help="launch shape 'blocks,slots' (k_decide grid, agents per k_commit thread)")
    e = sub.add_parser("ensemble")
    e.add_argument("--replicates", type=int, default=256)
    e.add_argument("--hours", type=int, default=49)
    m = sub.add_parser("mlp-train")
    m.add_argument("--steps", type=int, default=30)
    m.add_argument("--members", type=int, default=1)
    s = sub.add_parser("mlp-screen")
    s.add_argument("--candidates", type=int, default=65536)
    s.add_argument("--members", type=int, default=1)
    args = ap.parse_args()
    fn = {"tick": tick, "run": run, "ensemble": ensemble, "mlp-train": mlp_train, "mlp-screen": mlp_screen}[args.case]
    print(json.dumps(fn(args)))


if __name__ == "__main__":
    main()
