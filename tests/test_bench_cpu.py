"""bench.py's host logic without a GPU: the timed schedule of graph chunks and
the reference arm's isolation from the product library."""
from __future__ import annotations

import subprocess
import sys

import pytest

from conftest import REPO


@pytest.mark.parametrize("first,steps,gap", [(0, 10000, 10), (5, 20, 10), (3, 7, 10), (0, 3, 10), (10, 25, 5)])
def test_schedule_covers_the_steps_in_period_aligned_chunks(first, steps, gap):
    sys.path.insert(0, str(REPO))
    import bench

    sched = bench.schedule(first, steps, gap)
    assert sum(sched) == steps and all(n > 0 for n in sched)
    at = first
    for k, n in enumerate(sched):
        # every chunk after the first starts on a period boundary, none crosses one
        assert k == 0 or at % gap == 0
        assert (at % gap) + n <= gap
        at += n


def test_reference_arm_does_not_load_libnwgb():
    """The CPU reference arm derives its configuration in a child process and
    runs the oracle: libnwgb.so is never mapped into the arm's process."""
    code = ("import sys; sys.path.insert(0, %r); import bench; "
            "cfg, pos, vel = bench.workload_config('wca_small_4k', 0, isolated=True); "
            "sys.path.insert(0, %r); import oracle; oracle.lib(); "
            "maps = open('/proc/self/maps').read(); "
            "print(cfg.n_beads, 'libnwgb.so' in maps, 'libnworacle.so' in maps)") % (str(REPO), str(REPO / "oracle"))
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, check=True).stdout.split()
    assert out == ["4000", "False", "True"]
