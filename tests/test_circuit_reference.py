"""The reference's circuit tests for the vector path (src/circuit.rs), replayed
through this package's Circuit interpreter on the oracle backend (CPU): the
measurement, peek and reset ops, their X/Y-basis forms, conditional gates and
the three histograms, with the reference's binomial acceptance rule where it
tests statistics."""
import numpy as np

from oracle import oracle as orc
from q1tsim_gb300 import Circuit, Rng
from q1tsim_gb300 import gates as G
from refcheck import measurement_ok


def run(c, nr_shots, seed):
    c.execute_with(nr_shots, Rng(seed), orc.OracleState.new(c.nr_qbits, nr_shots))
    return c


def test_execute():
    """src/circuit.rs:1456-1468"""
    c = Circuit(2, 2)
    c.x(0)
    c.x(1)
    c.cx(0, 1)
    c.measure(0, 0)
    c.measure(1, 1)
    run(c, 5, 0)
    assert list(c.cstate()) == [0b01] * 5


def test_measure():
    """src/circuit.rs:1471-1517"""
    n = 1024
    c = Circuit(2, 2)
    c.x(0)
    c.measure(0, 0)
    c.measure(1, 1)
    assert run(c, n, 1).histogram_vec() == [0, n, 0, 0]
    c = Circuit(2, 2)
    c.x(0)
    c.measure_x(0, 0)
    c.measure_x(1, 1)
    assert all(measurement_ok(v, n, 0.25) for v in run(c, n, 2).histogram_vec())
    c = Circuit(2, 2)
    c.x(0)
    c.h(0)
    c.h(1)
    c.measure_x(0, 0)
    c.measure_x(1, 1)
    assert run(c, n, 3).histogram_vec() == [0, n, 0, 0]
    c = Circuit(2, 2)
    c.x(0)
    c.measure_y(0, 0)
    c.measure_y(1, 1)
    assert all(measurement_ok(v, n, 0.25) for v in run(c, n, 4).histogram_vec())


def _three_peeks(h):
    return h[0] + h[2] + h[4] + h[6], h[0] + h[1] + h[4] + h[5], h[0] + h[1] + h[2] + h[3]


def _split(hist, width):
    """Per group of `width` classical bits, the counts of its values."""
    mask = (1 << width) - 1
    out = [[0] * (1 << width) for _ in range(3)]
    for key, count in hist.items():
        for g in range(3):
            out[g][(key >> (width * g)) & mask] += count
    return out


def test_peek():
    """src/circuit.rs:1520-1573"""
    n = 1024
    c = Circuit(1, 3)
    c.h(0)
    c.peek(0, 0)
    c.h(0)
    c.peek(0, 1)
    c.h(0)
    c.peek(0, 2)
    n00, n10, n20 = _three_peeks(run(c, n, 5).histogram_vec())
    assert measurement_ok(n00, n, 0.5) and n10 == n and measurement_ok(n20, n, 0.5)
    c = Circuit(2, 6)
    c.h(0)
    c.h(1)
    c.peek(0, 0)
    c.h(0)
    c.peek(0, 1)
    c.h(0)
    c.peek(0, 2)
    n0, n1, n2 = _split(run(c, n, 6).histogram(), 1)
    assert all(measurement_ok(v, n, 0.5) for v in n0)
    assert n1 == [n, 0]
    assert all(measurement_ok(v, n, 0.5) for v in n2)


def test_peek_basis():
    """src/circuit.rs:1576-1616"""
    n = 1024
    c = Circuit(1, 3)
    c.peek_basis(0, 0, "x")
    c.h(0)
    c.peek_basis(0, 1, "x")
    c.h(0)
    c.peek_basis(0, 2, "x")
    n00, n10, n20 = _three_peeks(run(c, n, 7).histogram_vec())
    assert measurement_ok(n00, n, 0.5) and n10 == n and measurement_ok(n20, n, 0.5)
    c = Circuit(2, 6)
    c.peek_basis(0, 0, "y")
    c.h(0)
    c.peek_basis(0, 1, "y")
    c.sdg(0)
    c.peek_basis(0, 2, "y")
    n00, n10, n20 = _three_peeks(run(c, n, 8).histogram_vec())
    assert measurement_ok(n00, n, 0.5) and measurement_ok(n10, n, 0.5) and n20 == 0


def test_conditional():
    """src/circuit.rs:1619-1651: c_state set before reexecute."""
    c = Circuit(2, 2)
    c.add_conditional_gate([0, 1], 1, G.X(), [1])
    c.measure_all([0, 1])
    run(c, 5, 9)
    assert list(c.cstate()) == [0] * 5
    for control, target, qb, want in [([0, 1], 1, [1], [0b10, 0, 0, 0, 0]),
                                      ([0, 1], 2, [1], [0, 0b10, 0b10, 0, 0]),
                                      ([1], 1, [0], [0, 0b01, 0b01, 0b01, 0])]:
        c = Circuit(2, 2)
        c.q_state = orc.OracleState.new(2, 5)
        c.c_state = np.array([0b01, 0b10, 0b10, 0b11, 0b00], dtype=np.uint64)
        c.add_conditional_gate(control, target, G.X(), qb)
        c.measure_all([0, 1])
        c.reexecute(Rng(10))
        assert list(c.cstate()) == want


def test_measure_all():
    """src/circuit.rs:1654-1685"""
    n = 1024
    c = Circuit(2, 2)
    c.x(0)
    c.measure_all([0, 1])
    assert run(c, n, 11).histogram_vec() == [0, n, 0, 0]
    c = Circuit(2, 2)
    c.x(0)
    c.measure_all([1, 0])
    assert run(c, n, 12).histogram_vec() == [0, 0, n, 0]
    c = Circuit(2, 2)
    c.h(0)
    c.h(1)
    c.measure_all([0, 1])
    assert all(measurement_ok(v, n, 0.25) for v in run(c, n, 13).histogram_vec())


def test_measure_all_basis():
    """src/circuit.rs:1688-1732"""
    n = 1024
    c = Circuit(2, 2)
    c.h(0)
    c.h(1)
    c.measure_all_basis([0, 1], "x")
    assert run(c, n, 14).histogram_vec() == [n, 0, 0, 0]
    c = Circuit(2, 2)
    c.x(0)
    c.h(0)
    c.h(1)
    c.measure_all_basis([0, 1], "x")
    assert run(c, n, 15).histogram_vec() == [0, n, 0, 0]
    c = Circuit(2, 2)
    c.x(0)
    c.h(0)
    c.h(1)
    c.s(0)
    c.s(1)
    c.measure_all_basis([0, 1], "y")
    assert run(c, n, 16).histogram_vec() == [0, n, 0, 0]
    c = Circuit(2, 2)
    c.measure_all_basis([0, 1], "y")
    assert all(measurement_ok(v, n, 0.25) for v in run(c, n, 17).histogram_vec())


def test_peek_all():
    """src/circuit.rs:1735-1791"""
    n = 1024
    c = Circuit(1, 3)
    c.h(0)
    c.peek_all([0])
    c.h(0)
    c.peek_all([1])
    c.h(0)
    c.peek_all([2])
    n00, n10, n20 = _three_peeks(run(c, n, 18).histogram_vec())
    assert measurement_ok(n00, n, 0.5) and n10 == n and measurement_ok(n20, n, 0.5)
    c = Circuit(2, 6)
    c.h(0)
    c.h(1)
    c.peek_all([0, 1])
    c.h(0)
    c.peek_all([2, 3])
    c.h(0)
    c.peek_all([4, 5])
    n0, n1, n2 = _split(run(c, n, 19).histogram(), 2)
    assert all(measurement_ok(v, n, 0.25) for v in n0)
    assert n1[1] == 0 and n1[3] == 0
    assert measurement_ok(n1[0], n, 0.5) and measurement_ok(n1[2], n, 0.5)
    assert all(measurement_ok(v, n, 0.25) for v in n2)


def test_peek_all_basis():
    """src/circuit.rs:1794-1848"""
    n = 1024
    c = Circuit(1, 3)
    c.peek_all_basis([0], "x")
    c.h(0)
    c.peek_all_basis([1], "x")
    c.h(0)
    c.peek_all_basis([2], "x")
    n00, n10, n20 = _three_peeks(run(c, n, 20).histogram_vec())
    assert measurement_ok(n00, n, 0.5) and n10 == n and measurement_ok(n20, n, 0.5)
    c = Circuit(2, 6)
    c.h(0)
    c.h(1)
    c.peek_all_basis([0, 1], "y")
    c.s(1)
    c.peek_all_basis([2, 3], "y")
    c.s(0)
    c.peek_all_basis([4, 5], "y")
    n0, n1, n2 = _split(run(c, n, 21).histogram(), 2)
    assert all(measurement_ok(v, n, 0.25) for v in n0)
    assert n1[2] == 0 and n1[3] == 0
    assert measurement_ok(n1[0], n, 0.5) and measurement_ok(n1[1], n, 0.5)
    assert n2 == [n, 0, 0, 0]


def _two_hadamards(n, seed):
    c = Circuit(2, 2)
    c.add_gate(G.H(), [0])
    c.add_gate(G.H(), [1])
    c.measure(0, 0)
    c.measure(1, 1)
    return run(c, n, seed)


def test_histograms():
    """src/circuit.rs:1851-1921"""
    n = 4096
    h = _two_hadamards(n, 22).histogram()
    assert sorted(h) == [0, 1, 2, 3] and sum(h.values()) == n
    assert all(measurement_ok(v, n, 0.25) for v in h.values())
    hv = _two_hadamards(n, 23).histogram_vec()
    assert sum(hv) == n and all(measurement_ok(v, n, 0.25) for v in hv)
    hs = _two_hadamards(n, 24).histogram_string()
    assert sorted(hs) == ["00", "01", "10", "11"] and sum(hs.values()) == n
    assert all(measurement_ok(v, n, 0.25) for v in hs.values())


def test_reset():
    """src/circuit.rs:1924-1966"""
    n = 1024
    c = Circuit(2, 2)
    c.h(0)
    c.z(0)
    c.reset(0)
    c.measure(0, 0)
    c.measure(1, 1)
    assert run(c, n, 25).histogram_vec() == [n, 0, 0, 0]
    c = Circuit(2, 2)
    c.h(0)
    c.z(0)
    c.x(1)
    c.reset(0)
    c.measure(0, 0)
    c.measure(1, 1)
    assert run(c, n, 26).histogram_vec() == [0, 0, n, 0]
    c = Circuit(2, 2)
    c.h(0)
    c.z(0)
    c.h(1)
    c.reset(0)
    c.measure(0, 0)
    c.measure(1, 1)
    h = run(c, n, 27).histogram_vec()
    assert measurement_ok(h[0], n, 0.5) and h[1] == 0 and measurement_ok(h[2], n, 0.5) and h[3] == 0


def test_reset_all():
    """src/circuit.rs:1969-1985"""
    n = 1024
    c = Circuit(5, 5)
    c.h(0)
    c.z(0)
    c.x(4)
    c.h(3)
    c.reset_all()
    c.measure_all([0, 1, 2, 3, 4])
    h = run(c, n, 28).histogram_vec()
    assert h[0] == n and all(v == 0 for v in h[1:])
