"""bench.py's multi-rank reduction on CPU: two gloo ranks, the slowest rank's
time and the sum of all ranks' cell updates (replicas, weak scaling)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    w, r, _ = bench.dist_env()
    dist = bench.dist_init(w, "gloo")
    bench.barrier(dist)
    ms, units = bench.aggregate(dist, local_ms=10.0 + 5.0 * r, local_units=1000.0 * (r + 1))
    out[r] = (ms, units)
    dist.destroy_process_group()


def test_aggregate_two_gloo_ranks():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        for r in range(world):
            assert out[r] == (15.0, 3000.0)   # max over ranks, sum over ranks


def test_traffic_figures_match_their_profiles():
    """Each DRAM-traffic figure bench.py reports comes from the committed ncu
    summary it names, which states the same number."""
    import re
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    for key, (traffic, path) in bench.TRAFFIC.items():
        assert key in bench.KERNELS, key
        with open(os.path.join(root, path)) as f:
            figures = [int(v) for v in re.findall(r"traffic_bytes_per_launch\[[^\]]*\]: (\d+)", f.read())]
        assert traffic in figures, (key, path)
