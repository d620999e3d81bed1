"""The bench's N>1 path on CPU: world_size-2 gloo ranks reduce only the
max elapsed time and the summed work (replicas share no data)."""
import json
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms, units = bench.world_aggregate(10.0 * (rank + 1), 100 * (rank + 1), dist, "cpu")
    with open(f"{out}.{rank}", "w") as f:
        json.dump([ms, units], f)
    dist.barrier()
    dist.destroy_process_group()


def test_world_aggregate_gloo(tmp_path):
    import torch.multiprocessing as mp
    out = str(tmp_path / "agg")
    mp.spawn(_rank, args=(2, _free_port(), out), nprocs=2, join=True)
    for r in range(2):
        with open(f"{out}.{r}") as f:
            ms, units = json.load(f)
        assert ms == 20.0 and units == 300.0


def test_world_aggregate_single_process():
    import bench
    assert bench.world_aggregate(5.0, 7, None, "cpu") == (5.0, 7.0)
