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
    c = Circuit(3, 6)
    c.add_gate(G.CCX(), [0, 1, 2])
    for k in range(5):     # a fifth measurement would need 32 run columns
        c.measure(k % 3, k)
    b = Batch(4)
    with pytest.raises(Exception):
        b.add(c, 10, 1)
    c = Circuit(3, 3)
    c.h(0)
    c.add_conditional_gate([0, 1], 1, G.X(), [2])     # two control bits
    with pytest.raises(Exception):
        Batch(4).add(c, 10, 1)


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


def _final_sampling_check(c, shots, seed, words, nmeasure):
    """Words of the batch against the oracle for a circuit with mid-circuit
    measurements: the measured bits must agree run by run; each outcome of
    the final measure_all is recomputed from the oracle's columns and the
    circuit's uniform stream, and an outcome that differs must have its
    uniform within complex64 rounding (1e-5) of a boundary of the oracle's
    outcome.  Returns the number of differing words."""
    from q1tsim_gb300 import Circuit as Circ
    n = c.nr_qbits
    pre = Circ(n, c.nr_cbits, precision="c128", fusion_width=0)
    pre.ops = list(c.ops[:-1])        # everything but the final measure_all
    o = orc.OracleState.new(n, shots)
    rng = Rng(seed)
    pre.execute_with(shots, rng, o)
    mid = pre.cstate()
    midmask = np.uint64((1 << nmeasure) - 1)
    assert np.array_equal(words & midmask, mid & midmask)
    cols, counts = o.states(), o.counts
    ctr, r0, ndiff = rng.counter, 0, 0
    for k, m in enumerate(counts):
        if m == 0:
            continue
        e = -np.log1p(-orc.uniforms(seed, np.arange(ctr, ctr + m + 1, dtype=np.uint64)))
        s = np.cumsum(e)
        u = s[:m] / s[m]
        p = np.abs(cols[:, k]) ** 2
        P = np.cumsum(p) / p.sum()
        idx = np.searchsorted(P, u, side="right")
        got = np.zeros(m, dtype=np.int64)
        w = words[r0:r0 + m]
        for q in range(n):
            got |= ((w >> np.uint64(nmeasure + q)) & np.uint64(1)).astype(np.int64) << (n - 1 - q)
        for j in np.nonzero(got != idx)[0]:
            lo = P[idx[j] - 1] if idx[j] > 0 else 0.0
            hi = P[idx[j]]
            assert min(u[j] - lo, hi - u[j]) <= 1e-5, (k, j, u[j], lo, hi)
            ndiff += 1
        ctr += m + 1
        r0 += m
    return ndiff


@pytest.mark.parametrize("nmeasure", [2, 3, 4])
def test_batch_several_measurements_match_oracle(nmeasure):
    """Circuits with 2 to 4 mid-circuit measurements (each splits every run
    column, up to 16 columns) and gates conditioned on the measured bits, in
    one launch: at least 99.9 % of the classical words equal the oracle's
    for the same uniform stream, the mid-circuit bits all do, and every
    differing outcome lies within complex64 rounding of a sampling boundary."""
    rng = np.random.default_rng(40 + nmeasure)
    circuits = [workloads.mid_measure_circuit(int(rng.integers(6, 13)), int(rng.integers(4, 10)),
                                              int(rng.integers(2 ** 62)), nmeasure=nmeasure) for _ in range(12)]
    seeds = [700 + i for i in range(len(circuits))]
    shots = 400
    b = Batch(4)
    for c, s in zip(circuits, seeds):
        b.add(c, shots, s)
    res = b.run()
    agree, total, diffs = 0, 0, 0
    for c, s, r in zip(circuits, seeds, res):
        alone = run_alone(c, shots, s)
        agree += int(np.sum(alone == r))
        total += shots
        diffs += _final_sampling_check(c, shots, s, r, nmeasure)
    assert agree / total >= 0.999, agree / total
    assert diffs == total - agree
