"""Size-independent properties at the benchmark's full sizes (30 and 32
qubits), where the oracle cannot follow: a circuit followed by its inverse
returns to |0...0>; complex128 fused into double-float blocks equals
gate-by-gate complex128; the norm survives a 32-qubit tensor-core plan; shots
of a 30-qubit GHZ state land only on its two outcomes; complex64 fused
against complex128 at 28 qubits meets the 1 - F and outcome-TV targets.
States are compared on the device (q1g_state_compare)."""
import math

import numpy as np
import pytest

from q1tsim_gb300 import Plan, Rng, VectorState, workloads
from q1tsim_gb300 import gates as G

pytestmark = pytest.mark.gpu


def brick(n, depth, seed):
    """(matrix, bits) of the U3/CX brick circuit the bench runs."""
    rng = np.random.default_rng(seed)
    out = []
    for layer in range(depth):
        for q in range(n):
            out.append((G.U3(*rng.uniform(0.0, 2 * math.pi, 3)).matrix(), [q]))
        for q in range(0 if layer % 2 == 0 else 1, n - 1, 2):
            out.append((G.CX().matrix(), [q, q + 1]))
    return out


def flat(gates):
    return np.concatenate([np.ascontiguousarray(m, dtype=np.complex128).ravel() for m, _ in gates]).view(np.float64)


def test_round_trip_30_qubits_tensor_cores():
    """U then U^dagger (gates reversed and conjugate-transposed), complex64
    fused into 5-qubit tensor-core passes: back to |0...0> to 1 - F <= 1e-5."""
    n = 30
    fwd = brick(n, 8, 11)
    gates = fwd + [(m.conj().T, b) for m, b in reversed(fwd)]
    s = VectorState(n, 1, "c64")
    s.apply_plan(Plan(n, [b for _, b in gates], 5), flat(gates))
    zero = VectorState(n, 1, "c64")
    acc = zero.compare(s)
    assert acc["infidelity"] <= 1e-5, acc
    assert abs(acc["norm_b"] - 1.0) <= 1e-6, acc


def test_c128_fused_equals_gate_by_gate_30_qubits():
    """complex128 fused into 3-qubit double-float warp-tile blocks against
    gate-by-gate complex128, at 30 qubits: within the 1e-12 contract."""
    n = 30
    gates = brick(n, 3, 12)
    bits, mats = [b for _, b in gates], flat(gates)
    plain = VectorState(n, 1, "c128")
    plain.apply_plan(Plan(n, bits, 0), mats)
    fused = VectorState(n, 1, "c128")
    fused.apply_plan(Plan(n, bits, 3), mats)
    acc = plain.compare(fused)
    assert acc["max_abs_diff"] <= 1e-12, acc
    assert abs(acc["norm_b"] - 1.0) <= 1e-12, acc


def test_fused_c64_accuracy_against_c128_28_qubits():
    """The bench's brick pattern at 28 qubits, depth 24, complex64 fused into
    5-qubit tensor-core passes against plain complex128 on the GPU: 1 - F
    <= 1e-5 and outcome total variation <= 1e-6 (the accuracy targets of the
    FP32-fused mode)."""
    n = 28
    gates = brick(n, 24, 14)
    bits, mats = [b for _, b in gates], flat(gates)
    plain = VectorState(n, 1, "c128")
    plain.apply_plan(Plan(n, bits, 0), mats)
    fused = VectorState(n, 1, "c64")
    fused.apply_plan(Plan(n, bits, 5), mats)
    acc = plain.compare(fused)
    assert acc["infidelity"] <= 1e-5, acc
    assert acc["tv"] <= 1e-6, acc
    assert abs(acc["norm_b"] - 1.0) <= 1e-6, acc


def test_norm_kept_by_32_qubit_tensor_core_plan():
    """The 32-qubit state (32 GiB) after a fused plan keeps its norm (the
    norm correction after tensor-core plans, applied before the compare,
    restores it to 1e-12)."""
    n = 32
    gates = brick(n, 4, 13)
    s = VectorState(n, 1, "c64")
    s.apply_plan(Plan(n, [b for _, b in gates], 5), flat(gates))
    acc = s.compare(s)
    assert abs(acc["norm_a"] - 1.0) <= 1e-6, acc
    assert acc["infidelity"] <= 1e-12 and acc["max_abs_diff"] == 0.0, acc


def test_ghz_30_qubits_million_shots():
    """H and a CX chain on 30 qubits, then 10^6 Z shots: only 0...0 and
    1...1 occur, each about half the time (5 sigma)."""
    n, shots = 30, 1_000_000
    c = workloads.ghz(n, precision="c64", fusion_width=5, measure=True)
    c.execute(shots, Rng(2024))
    words = c.cstate()
    ones = (1 << n) - 1
    assert np.all((words == 0) | (words == ones))
    k = int(np.sum(words == ones))
    assert abs(k - shots / 2) <= 5 * math.sqrt(shots / 4), k
