"""The N > 1 path of bench.py on CPU: two gloo ranks (127.0.0.1), the
rendezvous, barrier and max-over-ranks timing the benchmark uses, and the
reference arm running on rank 0 only (replicas: no data-path collective)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_dir):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
    sys.path.insert(0, ROOT)
    import bench
    r, n, dist = bench.dist_setup()
    assert (r, n) == (rank, world) and dist is not None
    bench.barrier(dist)
    got = bench.max_over_ranks(dist, 10.0 + rank)
    args = type("A", (), {"warmup": 0, "steps": 1, "workload": "C2", "shots": 1, "nt": 10, "cpu_seconds": 0.0})()
    ref = None if rank == 0 else bench.reference_arm(args, rank, world, dist)
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(f"{got} {ref is None}\n")
    dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    port = _free_port()
    mp.spawn(_rank, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    for rank in range(2):
        got, none = (tmp_path / f"rank{rank}.txt").read_text().split()
        assert float(got) == 11.0          # the max over ranks, as the timing uses
        assert none == "True" or rank == 0  # the reference arm runs on rank 0 only
