"""Benchmark of the single-engine hourly tick (agent-hours/s).

Workload: the 1,000,000-agent / 2,500-grid run of 4,800 hours (small pox; 50 exposed;
Lockdown at 1,000 infections with 10% essential workers; vaccination of 20% of the
susceptible at hour 2,400; hospital build at 70% occupancy) -- tests/golden/small_pox_1m_2500.json.

One step = one full run of that workload (epi_engine_run: all hours, interventions and the
stop rule), restarted from the same initial world (a device-side restore) each step.
  value  agent-hours/s with the world resident in HBM, CUDA events on the engine's stream
  e2e    the same through the C ABI from host buffers: create from host records (upload),
         run, hourly counts back to the host, destroy -- every step
The L2 (129 MB) is flushed between steps by writing a 512 MiB buffer; within a step the
1M-agent working set (~60 MB) is L2-resident by design.

--impl reference times the CPU port of the reference's own tick data flow (hash map,
threaded map phase, serial resolve; oracle/o2.c) on all host cores, over consecutive 24-hour
windows of the same run from a world built by the oracle (the engine library is not loaded
in that process); both arms print the same `config` object.  Under torchrun the
engine runs as independent replicas (one per GPU, different seeds): the tick has no
exchange step to shard.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

DEFAULT_CONFIG = os.path.join(ROOT, "tests", "golden", "small_pox_1m_2500.json")
METRIC = "agent-hours/s"
# Algorithmic bytes of one k_decide launch per agent: pos 4 + st 8 + home 4 + work 4 read,
# st 8 + tgt 4 written; plus one read of the (G+1)^2 byte occupancy plane and of the
# (G+1)^2 infectious-neighbour counts.
DECIDE_BYTES_PER_AGENT = 32
DECIDE_PLANES = 2
# Whole-tick algorithmic bytes per agent-hour of the reference-layout accounting (agent record
# read 25 B + written 11 B, claim write and clear, plane write, and the occupancy and
# infectiousness planes amortised over the agents -- 76 B at 1M agents / 2500 grid in a
# movement hour; 16 B at hour of day 0, 3 B in the sleep hours, 12 B at hour 23), the
# per-unit figure of the run roofline below.
def tick_bytes_per_agent_hour(hod: int, agents: int, grid: int) -> float:
    if hod == 0:
        return 16.0
    if 1 <= hod <= 6:
        return 3.0
    if hod == 23:
        return 12.0
    return 36.0 + 8.0 + 1.0 + 5.0 * (grid + 1) ** 2 / agents


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def aggregate_replicas(ms_total: float, agent_hours: float, device: str = "cpu") -> tuple[float, float]:
    """Replicas only: the job's time is the slowest rank's, its work the sum over ranks."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([ms_total, agent_hours], dtype=torch.float64, device=device)
    ms_max = t[0].clone()
    dist.all_reduce(ms_max, op=dist.ReduceOp.MAX)
    dist.all_reduce(t[1:], op=dist.ReduceOp.SUM)
    return float(ms_max), float(t[1])


def replica_seed(seed: int, rank: int) -> int:
    """Every rank simulates an independent world."""
    return seed + 1000 * rank


def _agent_hours(rows, n_agents: int) -> float:
    return float(n_agents) * float(len(rows))


def cpu_baseline(cfg: dict, records, seconds: float = 12.0, max_hours: int = 240) -> dict:
    """O2 (the reference-semantics port) on all host cores over the first hours of the run."""
    import numpy as np  # noqa: F401

    from oracle import oracle

    threads = os.cpu_count() or 1
    params = oracle.params_from_config(cfg)
    sim = oracle.O2(params, records, threads=threads)
    t0 = time.perf_counter()
    hours = 0
    while hours < max_hours and (time.perf_counter() - t0) < seconds:
        sim.run(1 + hours, 2 + hours, interventions=True, stop=False, keep_rows=False)
        hours += 1
    dt = time.perf_counter() - t0
    n = len(records)
    out = {"value": n * hours / dt, "unit": METRIC, "cores": threads, "kind": "port",
           "sample": f"oracle/o2.c (reference data flow: FNV hash map, threaded map phase, serial "
                     f"resolve) on the same {n}-agent world, hours 1..{hours} ({dt:.1f} s)"}
    # the same port with the reference CLI's default thread count (-t 4), and the scalar
    # bit-exact oracle O1 on one thread, each over a short sample of the same hours
    variants = {}
    for name, make in (("o2_threads_4", lambda: oracle.O2(params, records, threads=4)),
                       ("o1_single_thread", lambda: oracle.O1(params, records))):
        sim = make()
        t0 = time.perf_counter()
        h = 0
        while h < max_hours and (time.perf_counter() - t0) < seconds / 4:
            sim.run(1 + h, 2 + h, interventions=True, stop=False)
            h += 1
        variants[name] = {"value": n * h / (time.perf_counter() - t0), "hours": h}
    # the reference's own default world (10,000 agents, 250 grid, small pox, 2,400 h) run in full
    # by the same port on all cores, world from the oracle's build
    with open(os.path.join(ROOT, "tests", "golden", "small_pox_10k_250.json")) as f:
        c1 = json.load(f)
    p1 = oracle.params_from_config(c1)
    recs1 = oracle.O1(p1).export()
    sim = oracle.O2(p1, recs1, threads=threads)
    t0 = time.perf_counter()
    rows = sim.run(1, int(c1["hours"]), interventions=True, stop=True)
    variants["o2_default_world_full_run"] = {"value": len(recs1) * len(rows) / (time.perf_counter() - t0),
                                       "hours": len(rows), "agents": len(recs1), "threads": threads}
    out["variants"] = variants
    return out


def workload_config(cfg: dict, world: int) -> dict:
    """The `config` object of both arms' JSON lines (identical, so the two lines describe
    one workload)."""
    auto = cfg["population"]["Auto"]
    return {
        "workload": "plain single-engine tick: 1M agents, 2500 grid, 4800 h, lockdown + vaccination + hospital "
                    "build (tests/golden/small_pox_1m_2500.json); metric per agent-hour, so the CPU reference arm "
                    "times consecutive windows of the same run and reports agent-hours/s over them",
        "agents": int(auto["number_of_agents"]), "grid": int(cfg["geography_parameters"]["grid_size"]),
        "hours": int(cfg["hours"]), "seed": int(cfg.get("seed", 0)),
        "interventions": "lockdown at >1000 infected (10% essential), vaccinate 20% of susceptible at hour 2400, "
                         "hospital build at 70% occupancy",
        "parallelism": f"replicas{world}",
        "l2": "GPU arm: flushed between steps (512 MiB write); inputs L2-resident within a step",
    }


def run_reference(args, cfg):
    """The reference's tick data flow on the host cores: oracle/o2.c (FNV hash map keyed by
    cell, threaded map phase, serial resolve in hash order, swap) over the same world, built
    by the oracle's own world build (oracle/o1.c) -- nothing of the engine library is loaded.
    One step = the next `ref_hours` hours of one continuing run (interventions on), so the
    warm-up and timed steps together cover hours 1 .. (warmup + steps) * ref_hours."""
    world, rank, _ = _dist()
    if rank != 0:
        return
    from oracle import oracle

    oracle.build()
    params = oracle.params_from_config(cfg)
    t0 = time.perf_counter()
    records = oracle.O1(params).export()
    build_s = time.perf_counter() - t0
    threads = os.cpu_count() or 1
    n = len(records)
    sample_hours = args.ref_hours
    sim = oracle.O2(params, records, threads=threads)
    hour = [1]

    def step():
        first = hour[0]
        t0 = time.perf_counter()
        sim.run(first, first + sample_hours, interventions=True, stop=False, keep_rows=False)
        hour[0] = first + sample_hours
        return time.perf_counter() - t0

    for _ in range(args.warmup):
        step()
    timed_first = hour[0]
    times = [step() for _ in range(args.steps)]
    total = sum(times)
    value = n * sample_hours * args.steps / total
    sample = (f"oracle/o2.c on {threads} threads, {n}-agent world from the oracle's world build ({build_s:.1f} s, "
              f"untimed); timed hours {timed_first}..{hour[0] - 1} of one run, {sample_hours} h per step, after "
              f"{args.warmup} warm-up steps")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": workload_config(cfg, world),
        "hours_per_step": sample_hours,
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_batched(args, stream, flush) -> dict:
    """The batched ensemble: 256 replicates (10k-500k agents, sqrt grids, 2,400 h) in one launch per hour."""
    import torch

    from epirust_gb300 import Ensemble
    from epirust_gb300.workloads import ensemble_params

    params = ensemble_params(replicates=args.replicates)
    agents = sum(p.number_of_agents for p in params)
    t0 = time.perf_counter()
    ens = Ensemble(params)
    build_s = time.perf_counter() - t0
    ens.set_stream(stream.cuda_stream)
    shape = ens.autotune(24)
    ens.save_state()
    for _ in range(1):
        ens.restore_state()
        ens.run()
    steps = max(1, min(args.steps, 3))
    ms_total, agent_hours = 0.0, 0.0
    for k in range(steps):
        with torch.cuda.stream(stream):
            flush.fill_(k & 0xFF)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        ens.restore_state()
        rows = ens.run()
        ev1.record(stream)
        ev1.synchronize()
        ms_total += ev0.elapsed_time(ev1)
        agent_hours += sum(float(p.number_of_agents) * len(r) for p, r in zip(params, rows))
    # roofline of the ensemble's dominant kernel: one more run with event nodes around every kernel
    ens.restore_state()
    ens.set_profiling(True)
    ens.run()
    stats = ens.kernel_stats()
    ens.close()
    batched_value = agent_hours / (ms_total / 1000.0)
    launches_d, ms_d = stats["k_decide"]
    avg_ms = ms_d / max(launches_d, 1)
    cells = sum((p.grid_size + 1) ** 2 for p in params)
    alg = DECIDE_BYTES_PER_AGENT * agents + DECIDE_PLANES * cells
    peak, peak_kind = _peaks()
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "k_decide_ens_traffic.txt")
    if os.path.exists(tpath):
        with open(tpath) as f:
            captured = int(f.readline().rsplit(":", 1)[1])
        traffic = int(captured * agents / 30_602_061)  # captured on this workload; scales with agents
    roofline = {"bound": "hbm", "kernel": "k_decide_ens", "achieved": alg / (avg_ms / 1000.0) / 1e9, "peak": peak,
                "unit": "GB/s", "frac": alg / (avg_ms / 1000.0) / 1e9 / peak, "peak_kind": peak_kind,
                "traffic": traffic, "alg_bytes_per_launch": alg, "avg_launch_ms": avg_ms,
                "kernels": {k: {"launches": v[0], "ms": v[1]} for k, v in stats.items() if v[0]}}

    # the same replicates one at a time through the plain single-engine path (every 4th one,
    # graphs warm: one untimed run per engine first)
    from epirust_gb300 import Epidemiology

    seq_ms, seq_ah = 0.0, 0.0
    sample = params[::4]
    for p in sample:
        eng = Epidemiology(p)
        eng.set_stream(stream.cuda_stream)
        eng.save_state()
        eng.run()
        eng.restore_state()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        r = eng.run()
        ev1.record(stream)
        ev1.synchronize()
        seq_ms += ev0.elapsed_time(ev1)
        seq_ah += float(p.number_of_agents) * len(r)
        eng.close()
    sequential_value = seq_ah / (seq_ms / 1000.0)
    return {"value": batched_value, "unit": METRIC, "replicates": len(params), "agents": agents,
            "sequential_plain_value": sequential_value, "sequential_sample": len(sample),
            "speedup_vs_sequential_plain": batched_value / sequential_value,
            "ms_per_step": ms_total / steps, "steps": steps, "world_build_and_upload_s": build_s,
            "launch_shape": shape, "roofline": roofline,
            "workload": "256 replicates, populations log-uniform in [10k, 500k], grid ceil(sqrt(N/0.16)), regular "
                        "rate U[0.02, 0.10], 0.05% exposed, 2400 h, no interventions, seeds from 11"}


def run_surrogate(args) -> dict:
    """Surrogate training on GPU-ABM ensembles (4,096 Latin-hypercube runs of 100,000 agents,
    100 days, 5 MLP members 8 -> 512 x 3 -> 600 trained with Adam in BF16 on the tensor cores)
    and the screened sweep (the members fine-tuned on `sweep_transfer` runs of 1,000,000
    agents; 65,536 candidates, the best `sweep_keep` and the fallback candidates where the
    members disagree re-run at 1,000,000 agents with 8 replicates each; an ABM-only sweep
    measured on the same budget of unscreened candidates)."""
    from epirust_gb300.sweep import screened_sweep, train_on_abm

    net, train = train_on_abm(runs=args.train_runs, held_out=args.train_runs // 8, steps=args.train_steps)
    train.pop("curves")
    sweep = screened_sweep(net, keep=args.sweep_keep, replicates=args.sweep_replicates,
                           transfer_points=args.sweep_transfer)
    net.close()
    sweep["note"] = ("abm_only_sweep_s_extrapolated = every candidate x replicates through the ABM at the rate "
                     "measured on its sample (abm_only_sample_runs unscreened runs, the screened sweep's budget: "
                     "re-runs and fine-tuning runs); screened_sweep_s counts the fine-tuning runs")
    return {"metric": "surrogate sweep speedup @<=5% peak err", "training": train, "sweep": sweep}


def run_gpu(args, cfg):
    import numpy as np
    import torch

    from epirust_gb300 import AGENT_DTYPE, Config, Epidemiology, build
    from epirust_gb300.engine import world_build

    build.build()
    world, rank, local = _dist()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev_index = torch.cuda.current_device()
    cfg = dict(cfg)
    cfg["seed"] = replica_seed(int(cfg.get("seed", 0)), rank)
    config = Config(json.dumps(cfg))
    n = config.number_of_agents
    G = config.params.grid_size
    cells = (G + 1) ** 2
    records, _ = world_build(config.params)

    stream = torch.cuda.Stream()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")

    eng = Epidemiology(config, records=records)
    eng.set_stream(stream.cuda_stream)
    shape = eng.autotune(72)  # launch shapes of the tick kernels (results do not depend on them)
    eng.save_state()

    def step():
        eng.restore_state()
        return eng.run()

    for _ in range(args.warmup):
        with torch.cuda.stream(stream):
            flush.fill_(1)
        step()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()
        torch.cuda.synchronize()

    # ---- timed region: device-resident world
    sampler = ClockSampler(dev_index)
    sampler.start()
    launches0 = eng.kernels_launched()
    barrier()
    ms_total, agent_hours = 0.0, 0.0
    t_wall = time.perf_counter()
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(k & 0xFF)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        rows = step()
        ev1.record(stream)
        ev1.synchronize()
        ms_total += ev0.elapsed_time(ev1)
        agent_hours += _agent_hours(rows, n)
    barrier()
    wall = time.perf_counter() - t_wall
    clocks = sampler.stop()
    launches = eng.kernels_launched() - launches0
    hours_per_step = len(rows)

    if world > 1:
        ms_total, agent_hours = aggregate_replicas(ms_total, agent_hours, "cuda")
    value = agent_hours / (ms_total / 1000.0)

    # ---- e2e: host records -> create (upload) -> run -> counts on the host -> destroy
    pinned = torch.from_numpy(records.view(np.uint8)).pin_memory()
    host_records = pinned.numpy().view(AGENT_DTYPE)
    e2e_steps = max(1, min(args.steps, 3))
    e2e_ms, e2e_ah = 0.0, 0.0
    for _ in range(e2e_steps):
        with torch.cuda.stream(stream):
            flush.fill_(3)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e = Epidemiology(config, records=host_records)
        e.set_launch_shape(shape["decide_blocks"], shape["commit_slots"])
        r = e.run()
        e.close()
        e2e_ms += 1000.0 * (time.perf_counter() - t0)
        e2e_ah += _agent_hours(r, n)
    e2e_value = e2e_ah / (e2e_ms / 1000.0)

    # ---- roofline of the dominant kernel: one more run of the same workload whose hour graphs
    # carry CUDA event nodes around every kernel (on the engine's stream)
    prof = Epidemiology(config, records=records)
    prof.set_stream(stream.cuda_stream)
    prof.set_launch_shape(shape["decide_blocks"], shape["commit_slots"])
    prof.set_profiling(True)
    prof.run()
    stats = prof.kernel_stats()
    prof.close()
    total_kernel_ms = sum(ms for _, ms in stats.values())
    launches_d, ms_d = stats["k_decide"]
    avg_ms = ms_d / max(launches_d, 1)
    alg_bytes = DECIDE_BYTES_PER_AGENT * n + DECIDE_PLANES * cells
    achieved = alg_bytes / (avg_ms / 1000.0) / 1e9
    peak, peak_kind = _peaks()
    # issue roofline: warp instructions per k_decide launch (committed ncu launch list, scaled
    # by agents) over the launch time, against 4 schedulers x SMs x the maximum SM clock
    issue = None
    ipath = os.path.join(ROOT, "profiles", "k_decide_issue.txt")
    if os.path.exists(ipath):
        with open(ipath) as f:
            inst = int(f.readline().rsplit(":", 1)[1]) * n / 1_000_000
        sms = torch.cuda.get_device_properties(dev_index).multi_processor_count
        mhz = clocks.get("sm_max_mhz") or 2070.0
        peak_issue = 4.0 * sms * mhz * 1e6
        issue = {"achieved": inst / (avg_ms / 1000.0), "peak": peak_issue, "unit": "warp-instructions/s",
                 "frac": inst / (avg_ms / 1000.0) / peak_issue, "inst_per_launch": inst}
    traffic = None  # DRAM bytes of one k_decide launch from the committed ncu capture
    tpath = os.path.join(ROOT, "profiles", "k_decide_traffic.txt")
    if os.path.exists(tpath):
        with open(tpath) as f:
            first = f.readline()
        traffic = int(first.rsplit(":", 1)[1]) * n // 1_000_000  # captured at 1M agents; scales with agents

    # run roofline: every simulated hour's algorithmic bytes over the timed step
    run_bytes = sum(n * tick_bytes_per_agent_hour(h % 24, n, G) for h in range(1, hours_per_step + 1))
    run_achieved = run_bytes / (ms_total / args.steps / 1000.0) / 1e9

    batched = run_batched(args, stream, flush) if not args.no_batched else None

    surrogate = run_surrogate(args) if rank == 0 and not args.no_surrogate else None

    cpu = cpu_baseline(cfg, records, seconds=args.cpu_seconds) if rank == 0 and not args.no_cpu else None

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": workload_config(cfg, world),
            "hours_per_step": hours_per_step, "launch_shape": shape, "wall_s": wall,
            "roofline": {"bound": "hbm", "kernel": "k_decide", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                         "alg_bytes_per_launch": alg_bytes, "avg_launch_ms": avg_ms,
                         "share_of_kernel_time": ms_d / total_kernel_ms if total_kernel_ms else None,
                         "issue": issue,
                         "run": {"achieved": run_achieved, "peak": peak, "unit": "GB/s", "frac": run_achieved / peak,
                                 "bytes_per_step": run_bytes,
                                 "basis": "whole run: per agent-hour 76 B (movement hours at 1M/2500), 16 B (hour 0), "
                                          "3 B (hours 1-6), 12 B (hour 23), reference-layout accounting"},
                         "kernels": {k: {"launches": v[0], "ms": v[1]} for k, v in stats.items() if v[0]}},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": int(host_records.nbytes),
                    "d2h_bytes_per_step": int(hours_per_step * 32), "steps": e2e_steps},
            "gpu_launches": int(launches),
            "clocks": clocks,
            "batched": batched,
            "surrogate": surrogate,
        }
        if batched:
            batched["speedup_vs_plain"] = batched["value"] / value
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default=DEFAULT_CONFIG)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--ref-hours", type=int, default=24)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--replicates", type=int, default=256)
    ap.add_argument("--no-surrogate", action="store_true")
    ap.add_argument("--train-runs", type=int, default=4096)
    ap.add_argument("--train-steps", type=int, default=3000)
    ap.add_argument("--sweep-keep", type=int, default=256)
    ap.add_argument("--sweep-transfer", type=int, default=512,
                    help="1M-agent ABM runs the surrogate is fine-tuned on before the screen (0: none)")
    ap.add_argument("--sweep-replicates", type=int, default=8)
    args = ap.parse_args()
    with open(args.config) as f:
        cfg = json.load(f)
    if args.impl == "reference":
        run_reference(args, cfg)
    else:
        run_gpu(args, cfg)


if __name__ == "__main__":
    main()
