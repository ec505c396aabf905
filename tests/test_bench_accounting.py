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
