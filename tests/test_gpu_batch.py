"""Batched executor: many circuits in one persistent launch, each giving the
same classical results as running it alone through Circuit.execute with the
same uniform stream (oracle backend: src/circuit.rs:643-762 per circuit)."""
import numpy as np
import pytest

from oracle import oracle as orc
from q1tsim_gb300 import Circuit, Rng, VectorState, workloads
from q1tsim_gb300 import gates as G
from q1tsim_gb300.batch import Batch

pytestmark = pytest.mark.gpu


def run_alone(c, shots, seed, backend="oracle"):
    q = orc.OracleState.new(c.nr_qbits, shots) if backend == "oracle" else VectorState(c.nr_qbits, shots, "c64")
    c.execute_with(shots, Rng(seed), q)
    return c.cstate().copy()


def test_batch_matches_each_circuit_alone():
    circuits = workloads.batch_workload(32, seed=5, qmin=3, qmax=11, dmin=2, dmax=9)
    seeds = [1000 + i for i in range(len(circuits))]
    shots = 300
    b = Batch(4)
    for c, s in zip(circuits, seeds):
        b.add(c, shots, s)
    res = b.run()
    agree, total = 0, 0
    for c, s, r in zip(circuits, seeds, res):
        alone = run_alone(c, shots, s)
        agree += int(np.sum(alone == r))
        total += shots
    # identical except, with vanishing probability, FP32 rounding at a
    # sampling boundary (the batch runs in complex64, the oracle in complex128)
    assert agree / total >= 0.999, agree / total


def test_batch_rerun_is_deterministic_and_graph_replays():
    circuits = workloads.batch_workload(16, seed=9, qmin=8, qmax=14, dmin=5, dmax=12)
    b = Batch(3)
    for i, c in enumerate(circuits):
        b.add(c, 512, 77 + i)
    r1 = b.run()
    r2 = b.run()
    for x, y in zip(r1, r2):
        assert np.array_equal(x, y)
    info = b.info()
    assert info["circuits"] == 16 and info["runs"] == 16 * 512 and info["last_ms"] > 0


def test_batch_equals_single_state_gpu_path():
    """The same circuit through the single-state GPU path (plans, measure,
    conditional, measure_all on a VectorState) and through the batch."""
    c = workloads.mid_measure_circuit(9, 6, 123)
    shots = 20000
    b = Batch(4)
    b.add(c, shots, 3)
    words = b.run()[0]
    alone = run_alone(c, shots, 3, backend="gpu")
    assert np.mean(words == alone) >= 0.999


def test_batch_rejects_unsupported_programs():
    c = Circuit(3, 3)
    c.add_gate(G.CCX(), [0, 1, 2])
    c.measure(0, 0)
    c.measure(1, 1)
    b = Batch(4)
    with pytest.raises(Exception):
        b.add(c, 10, 1)


def test_batch_warp_tiles_match_oracle():
    """States of 10 to 16 qubits take the warp-tile path: blocks on low and
    high positions, one or two columns after the mid-circuit measurement."""
    circuits = workloads.batch_workload(10, seed=21, qmin=10, qmax=16, dmin=4, dmax=12)
    seeds = [500 + i for i in range(len(circuits))]
    shots = 256
    b = Batch(4)
    for c, s in zip(circuits, seeds):
        b.add(c, shots, s)
    res = b.run()
    agree, total = 0, 0
    for c, s, r in zip(circuits, seeds, res):
        alone = run_alone(c, shots, s)
        agree += int(np.sum(alone == r))
        total += shots
    assert agree / total >= 0.999, agree / total
