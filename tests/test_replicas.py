"""The multi-GPU (replica) reduction of bench.py on CPU: two gloo ranks, each with its own
time and counts; every rank gets the slowest time and the summed rays and paths."""
import json
import os
import socket

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out_dir: str):
    import torch.distributed as td
    from mcrt_gb300.replicas import aggregate
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    td.init_process_group("gloo", rank=rank, world_size=world)
    try:
        res = aggregate(100.0 + 50.0 * rank, 1000 * (rank + 1), 10 * (rank + 1), "cpu")
        with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
            json.dump(res, f)
    finally:
        td.destroy_process_group()


def test_replica_reduction_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    mp.spawn(_rank, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    for r in range(2):
        t, rays, paths = json.load(open(tmp_path / f"r{r}.json"))
        assert t == 150.0 and rays == 3000 and paths == 30


def test_replica_reduction_without_process_group():
    from mcrt_gb300.replicas import aggregate
    assert aggregate(12.5, 7, 3, "cpu") == (12.5, 7, 3)
