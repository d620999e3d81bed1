"""The engine side of the sharded state on one GPU: an engine shard's
amplitudes seen by torch without a copy (q1g_state_device_amplitudes),
written in place and taken back by the engine (q1g_state_amplitudes_written)
with their norm, and a one-rank ShardedState over NCCL against the oracle.
Exchanges between ranks need two GPUs; their logic is tested on CPU
(test_sharded_multirank.py)."""
import os
import socket

import numpy as np
import pytest

from oracle import oracle as orc
from q1tsim_gb300 import Plan
from q1tsim_gb300 import gates as G

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


@pytest.mark.parametrize("prec,tol", [("c128", 1e-12), ("c64", 2e-6)])
def test_engine_shard_amplitudes_in_place(prec, tol):
    from q1tsim_gb300.sharded import EngineShard
    n = 13
    sh = EngineShard(n, 1, prec)
    a = sh.amplitudes()
    assert a.is_cuda and a.numel() == 1 << n
    rng = np.random.default_rng(4)
    host = (rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)) * 0.01
    a.copy_(torch.from_numpy(host).to(a.dtype))
    sh.amplitudes_written()
    assert abs(sh.column_norms()[0] - np.sum(np.abs(host) ** 2)) <= 1e-6 * np.sum(np.abs(host) ** 2)
    gl = [(G.U3(*rng.uniform(0, 6, 3)).matrix(), [q]) for q in range(n)] + \
         [(G.CX().matrix(), [q, q + 1]) for q in range(0, n - 1, 2)]
    mats = np.concatenate([np.ascontiguousarray(m).ravel() for m, _ in gl]).view(np.float64)
    o = orc.OracleState.from_amplitudes(host, 1)
    for m, b in gl:
        o.apply_gate(m, b)
    # a fused (complex64: tensor-core) plan keeps the written norm
    sh.state.apply_plan(Plan(n, [b for _, b in gl], 5 if prec == "c64" else 3), mats)
    got = sh.state.states()[:, 0]
    assert np.max(np.abs(got - o.states()[:, 0])) <= tol


def _init_one_rank():
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(_free_port())
    dist.init_process_group("nccl", rank=0, world_size=1)
    return dist


def test_sharded_state_one_rank_on_gpu():
    from q1tsim_gb300.sharded import ShardedState
    dist = _init_one_rank()
    try:
        n = 12
        st = ShardedState(n, 2000, "c128")
        rng = np.random.default_rng(6)
        o = orc.OracleState.new(n, 2000)
        for _ in range(30):
            k = int(rng.integers(1, 3))
            bits = [int(b) for b in rng.choice(n, k, replace=False)]
            m = G.U3(*rng.uniform(0, 6, 3)).matrix() if k == 1 else G.CX().matrix()
            st.apply_gate(m, bits)
            o.apply_gate(m, bits)
        assert np.max(np.abs(st.states()[:, 0] - o.states()[:, 0])) <= 1e-12
        u = np.sort(rng.random(2000))
        cbits = list(range(n))
        got, want = np.zeros(2000, dtype=np.uint64), np.zeros(2000, dtype=np.uint64)
        st.peek_all_into(cbits, got, u)
        o.peek_all_into(cbits, want, uniforms=u)
        assert np.array_equal(got, want)
    finally:
        dist.destroy_process_group()
