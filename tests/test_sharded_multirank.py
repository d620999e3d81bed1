"""The sharded state (q1tsim_gb300/sharded.py) on CPU: world_size 2 and 4
gloo ranks, each shard held by the oracle (a complex128 restatement of
VectorState).  Gates on global and local qubits, the global/local exchanges
and the cross-shard sampling give the unsharded oracle's amplitudes
(1e-12) and, for the same uniforms, the same classical words.  The
exchange and sampling logic is the same on GPUs (engine shards, NCCL);
with one GPU per run it is not measured on hardware."""
import json
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


class OracleShard:
    """A rank's shard kept as a CPU tensor and updated by the oracle."""

    def __init__(self, nr_bits, nr_shots, precision):
        self.n = nr_bits
        self.a = torch.zeros(1 << nr_bits, dtype=torch.complex128)
        self.a[0] = 1.0

    def _oracle(self, shots=1):
        from oracle import oracle as orc
        return orc.OracleState.from_amplitudes(self.a.numpy().copy(), shots)

    def apply_gate(self, mat, bits):
        o = self._oracle()
        o.apply_gate(np.asarray(mat), bits)
        self.a.copy_(torch.from_numpy(o.states()[:, 0].copy()))

    def amplitudes(self):
        return self.a

    def amplitudes_written(self):
        pass

    def column_norms(self):
        return np.array([float((self.a.abs() ** 2).sum())])

    def peek_all_into(self, cbits, res, uniforms):
        self._oracle(len(res)).peek_all_into(cbits, res, uniforms=uniforms)


def _circuit(n, seed):
    """Random 1-3 qubit gates, many of them on the global (top) qubits."""
    from q1tsim_gb300 import gates as G
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(40):
        k = int(rng.integers(1, 4))
        bits = [int(b) for b in rng.choice(n, k, replace=False)]
        if k == 1:
            m = G.U3(*rng.uniform(0, 2 * np.pi, 3)).matrix()
        elif k == 2:
            m = np.kron(G.U3(*rng.uniform(0, 6, 3)).matrix(), G.H().matrix()) @ G.CX().matrix()
        else:
            m = G.CCX().matrix() @ np.kron(np.kron(G.RY(rng.uniform(0, 6)).matrix(), G.S().matrix()),
                                           G.U3(*rng.uniform(0, 6, 3)).matrix())
        out.append((m, bits))
    return out


def _rank(rank, world, port, n, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from q1tsim_gb300.sharded import ShardedState
    st = ShardedState(n, 3000, "c128", shard_factory=OracleShard)
    for m, bits in _circuit(n, 5):
        st.apply_gate(m, bits)
    exchanges = st.exchanges
    full = st.states()[:, 0]
    u = np.sort(np.random.default_rng(9).random(3000))
    cbits = [int(c) for c in np.random.default_rng(10).permutation(n)]
    res = np.zeros(len(u), dtype=np.uint64)
    st.peek_all_into(cbits, res, u)
    if rank == 0:
        with open(out, "w") as f:
            json.dump({"re": full.real.tolist(), "im": full.imag.tolist(), "words": res.tolist(),
                       "cbits": cbits, "u": u.tolist(), "exchanges": exchanges}, f)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 4])
def test_sharded_state_matches_oracle(tmp_path, world):
    import torch.multiprocessing as mp
    from oracle import oracle as orc
    n = 8
    out = str(tmp_path / "sharded.json")
    mp.spawn(_rank, args=(world, _free_port(), n, out), nprocs=world, join=True)
    with open(out) as f:
        d = json.load(f)
    o = orc.OracleState.new(n, len(d["u"]))
    for m, bits in _circuit(n, 5):
        o.apply_gate(m, bits)
    want = o.states()[:, 0]
    got = np.array(d["re"]) + 1j * np.array(d["im"])
    assert np.max(np.abs(got - want)) <= 1e-12
    # gates on the global qubits went through half-shard exchanges
    assert d["exchanges"] >= 5
    words = np.zeros(len(d["u"]), dtype=np.uint64)
    o.peek_all_into(d["cbits"], words, uniforms=np.array(d["u"]))
    assert np.array_equal(np.array(d["words"], dtype=np.uint64), words)
