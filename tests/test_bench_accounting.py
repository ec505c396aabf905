"""bench.py's accounting, checked on the CPU: the per-agent-hour bytes of the whole-tick
roofline."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def test_run_roofline_bytes_per_agent_hour():
    """The whole-tick numerator of bench.py's run roofline: 76 B per agent in a movement hour
    of the 1M-agent / 2,500-grid world, 16 B at hour 0, 3 B in hours 1-6, 12 B at hour 23,
    52.8 B per agent-hour over a day."""
    import bench

    per_hour = [bench.tick_bytes_per_agent_hour(h, 1_000_000, 2500) for h in range(24)]
    assert per_hour[0] == 16.0 and per_hour[23] == 12.0 and set(per_hour[1:7]) == {3.0}
    assert abs(per_hour[9] - 76.27) < 0.01
    assert abs(sum(per_hour) / 24 - 52.8) < 0.1


def test_reference_arm_is_the_oracle_port_on_the_same_config():
    """bench.py --impl reference: the CPU port of the reference's tick data flow (O2) on a world
    from the oracle's own build, with the same `config` object as the GPU arm's line, and
    without loading the engine library in its process."""
    import json
    import subprocess

    import bench

    code = (
        "import json, runpy, sys\n"
        "sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0', '--ref-hours', '1']\n"
        "runpy.run_path('bench.py', run_name='__main__')\n"
        "maps = open('/proc/self/maps').read()\n"
        "print(json.dumps({'engine_lib': 'libepirust_gb300' in maps, 'engine_module': 'epirust_gb300' in sys.modules}))\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(ln) for ln in r.stdout.splitlines() if ln.startswith("{")]
    line, probe = lines[0], lines[-1]
    assert probe == {"engine_lib": False, "engine_module": False}
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["unit"] == bench.METRIC
    with open(bench.DEFAULT_CONFIG) as f:
        cfg = json.load(f)
    assert line["config"] == bench.workload_config(cfg, 1)
    assert line["cpu_baseline"]["kind"] == "port" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
