"""The multi-rank path of bench.py on CPU ranks (gloo, world size 2): every
rank runs its own replica, the job's throughput is the units of all ranks over
the slowest rank's time, only rank 0 prints, and the reference arm runs on
rank 0 alone.  No GPU: the collectives are the gloo ones."""
from __future__ import annotations

import io
import os
import sys
from contextlib import redirect_stdout
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(REPO))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    r, w, local = bench.env_rank()
    # rank k processed 1000 * (k + 1) units in 10 * (k + 1) ms
    value, ms_max = bench.job_rate(dist, 10.0 * (r + 1), 1000.0 * (r + 1))
    # the reference arm: ranks other than 0 leave at once, printing nothing
    buf = io.StringIO()
    if r != 0:
        with redirect_stdout(buf):
            rc = bench.run_reference(type("A", (), {"workload": "wca_small_4k", "steps": 1})())
    else:
        rc = 0
    dist.barrier()
    dist.destroy_process_group()
    Path(out_dir, f"r{r}.txt").write_text(f"{r} {w} {local} {value} {ms_max} {rc} {len(buf.getvalue())}")


@pytest.mark.timeout(300)
def test_two_cpu_ranks_aggregate_like_the_bench(tmp_path):
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn")
    rows = sorted(Path(tmp_path, f"r{k}.txt").read_text().split() for k in range(2))
    for k, row in enumerate(rows):
        r, w, local, value, ms_max, rc, printed = row
        assert (int(r), int(w), int(local)) == (k, 2, k)
        # (1000 + 2000) units over the slowest rank's 20 ms, on every rank
        assert abs(float(value) - 3000.0 / 0.020) < 1e-6 and float(ms_max) == 20.0
        assert int(rc) == 0 and int(printed) == 0
