"""Host logic of bench.py's CPU legs (no GPU): the oracle-rate probe that sizes the reference
arm's sample times at least one substep, even with a zero time budget."""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import bench  # noqa: E402
from bubbles_gb300 import scenes  # noqa: E402


def test_oracle_rate_probe_times_one_substep():
    sc, pos = scenes.small_pcisph()
    rate, steps, iters, t = bench.cpu_oracle_rate(sc, pos, None, 0.0, 1, max_steps=1)
    assert steps == 1 and iters >= 1 and t > 0 and rate > 0
