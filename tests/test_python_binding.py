"""The reference's Python binding API (python/q1tsim.py) on the GPU engine:
q1tsim_gb300.q1tsim.  Construction and error behaviour need no GPU; the
execution tests follow the binding's own examples (python/test.py,
python/test_cstate.py) with statistical checks."""
import math

import numpy as np
import pytest

from q1tsim_gb300 import q1tsim
from refcheck import measurement_ok


def test_construction_and_context_manager():
    with q1tsim.Circuit(3, 2) as c:
        assert c.nr_qbits() == 3
        assert c.nr_cbits() == 2
    assert q1tsim.Circuit(1).nr_cbits() == 0


def test_every_shortcut_and_name_builds():
    c = q1tsim.Circuit(3, 3)
    p = q1tsim.RefParam(0.3)
    for call in (lambda: c.ch(0, 1), lambda: c.crx(0.1, 0, 1), lambda: c.cry(p, 1, 2), lambda: c.crz(0.2, 2, 0),
                 lambda: c.cx(0, 1), lambda: c.cy(1, 2), lambda: c.cz(2, 0), lambda: c.h(0), lambda: c.i(1),
                 lambda: c.rx(p, 2), lambda: c.ry(0.4, 0), lambda: c.rz(0.5, 1), lambda: c.s(2), lambda: c.sdg(0),
                 lambda: c.swap(0, 2), lambda: c.t(1), lambda: c.tdg(2), lambda: c.u1(0.6, 0),
                 lambda: c.u2(0.1, 0.2, 1), lambda: c.u3(0.1, 0.2, 0.3, 2), lambda: c.v(0), lambda: c.vdg(1),
                 lambda: c.x(2), lambda: c.y(0), lambda: c.z(1)):
        assert call() is None
    c.add_gate("u3", [0], [0.1, p, 0.3])   # names are case-insensitive, parameters by value or reference
    c.add_conditional_gate([0, 1], 2, "X", [2])
    c.measure(0, 0)
    c.measure_x(1, 1)
    c.measure_y(2, 2)
    c.peek_z(0, 0)
    c.measure_all([0, 1, 2])
    c.peek_all_basis([2, 1, 0], "x")
    c.reset(1)
    c.reset_all()


@pytest.mark.parametrize("name,qbits,params,msg", [
    ("Foo", [0], None, "Unknown gate"),
    ("CCX", [0, 1, 2], None, "Unknown gate"),          # not in the binding's gate table
    ("RX", [0], None, "Invalid number of arguments"),
    ("U3", [0], [0.1, 0.2], "Invalid number of arguments"),
    ("H", [7], None, "Invalid index"),
])
def test_gate_errors_raise(name, qbits, params, msg):
    c = q1tsim.Circuit(3, 3)
    with pytest.raises(Exception, match=msg):
        c.add_gate(name, qbits, params)


def test_other_errors_raise():
    c = q1tsim.Circuit(2, 2)
    with pytest.raises(Exception, match="Invalid measurement basis"):
        c.measure_basis(0, 0, "Q")
    with pytest.raises(Exception, match="Invalid index"):
        c.measure(0, 5)
    with pytest.raises(Exception, match="not been run"):
        c.cstate()
    with pytest.raises(Exception, match="not been run"):
        c.histogram()
    with pytest.raises(Exception):
        c.reexecute()
    for export in (c.latex, c.open_qasm, c.c_qasm):
        with pytest.raises(Exception):
            export()


@pytest.mark.gpu
def test_binding_example_refparam_reexecute():
    """python/test.py: reexecute() continues from the previous state
    (python/q1tsim.py:483-490).  With the RefParam reassigned to -1.23 the
    second RX undoes the first: every run reads 0.  A plain float bound at
    build time does not change: RX(1.23) twice, P(1) = sin^2(1.23)."""
    shots = 20000
    ang = q1tsim.RefParam(1.23)
    with q1tsim.Circuit(1, 1) as c:
        c.rx(ang, 0)
        c.peek(0, 0)
        c.execute(shots)
        h = c.histogram()
        assert set(h) <= {"0", "1"} and sum(h.values()) == shots
        assert measurement_ok(h.get("1", 0), shots, math.sin(1.23 / 2) ** 2, 1e-6)
        ang.assign(-1.23)
        c.reexecute()
        assert c.histogram() == {"0": shots}
    val = 1.23
    with q1tsim.Circuit(1, 1) as c:
        c.rx(val, 0)
        c.peek(0, 0)
        c.execute(shots)
        val = -1.23     # rebinding the name changes nothing
        c.reexecute()
        assert measurement_ok(c.histogram().get("1", 0), shots, math.sin(1.23) ** 2, 1e-6)


@pytest.mark.gpu
def test_binding_example_cstate():
    """python/test_cstate.py: two H and two measurements."""
    shots = 4000
    with q1tsim.Circuit(2, 2) as c:
        c.h(0)
        c.h(1)
        c.measure(0, 0)
        c.measure(1, 1)
        c.execute(shots)
        cs = c.cstate()
        assert len(cs) == shots and all(isinstance(w, int) and 0 <= w < 4 for w in cs)
        counts = np.bincount(cs, minlength=4)
        for k in range(4):
            assert measurement_ok(int(counts[k]), shots, 0.25, 1e-6)
        h = c.histogram()
        assert {k: h.get(k, 0) for k in ("00", "01", "10", "11")} == {format(k, "02b"): int(counts[k])
                                                                      for k in range(4)}


@pytest.mark.gpu
def test_binding_bases_and_conditional():
    """|+> measured in X is always 0, |+i> in Y always 0; a conditional X
    copies a measured bit (the binding's add_conditional_gate)."""
    shots = 2000
    with q1tsim.Circuit(3, 3) as c:
        c.h(0)
        c.measure_x(0, 0)
        c.h(1)
        c.s(1)
        c.measure_y(1, 1)
        c.h(2)
        c.measure(2, 2)
        c.add_conditional_gate([2], 1, "X", [2])   # flips qubit 2 back to |0> where bit 2 was 1
        c.peek(2, 0)
        c.execute(shots)
        cs = np.array(c.cstate(), dtype=np.uint64)
        assert np.all((cs >> np.uint64(1)) & np.uint64(1) == 0)      # Y measurement of |+i>
        assert np.all(cs & np.uint64(1) == 0)                        # peek of the reset qubit 2
        ones = int(((cs >> np.uint64(2)) & np.uint64(1)).sum())
        assert measurement_ok(ones, shots, 0.5, 1e-6)


def test_segment_matrices_follow_reference_parameters():
    """A circuit keeps each gate run's matrices between executions and
    evaluates them again only when a reference parameter has changed
    (src/gates/parameter.rs:23-75); plain values never change."""
    from q1tsim_gb300 import Circuit as GpuCircuit
    from q1tsim_gb300 import gates as G
    p = q1tsim.RefParam(0.4)
    c = GpuCircuit(2, 0, precision="c128", fusion_width=0)
    c.add_gate(G.RX(p), [0])
    c.add_gate(G.U3(0.1, 0.2, 0.3), [1])
    c.add_gate(G.CRZ(p), [0, 1])
    idx, seq = next((i, op[1]) for i, op in enumerate(c._segments()) if op[0] == "seq")
    first = c._flat_current(idx, seq)
    assert c._flat_current(idx, seq) is first
    p.assign(-1.1)
    second = c._flat_current(idx, seq)
    assert second is not first
    np.testing.assert_allclose(second, c._flat(seq), rtol=0, atol=0)
    np.testing.assert_allclose(second[8:16], first[8:16], rtol=0, atol=0)   # the U3 block is unchanged
    assert not np.array_equal(second[:8], first[:8])


def test_segment_matrices_equal_each_gates_matrix():
    """Circuit._flat evaluates U3 and controlled-U1 gates together and shares
    fixed controlled matrices: the result equals each gate's own matrix(),
    bit for bit, over a mix of gate kinds and reference parameters."""
    from q1tsim_gb300 import Circuit as GpuCircuit
    from q1tsim_gb300 import gates as G
    rng = np.random.default_rng(3)
    p, q = q1tsim.RefParam(0.3), q1tsim.RefParam(1.3)
    make = [lambda: G.U3(*rng.uniform(-7, 7, 3)), G.CX, G.H, lambda: G.RX(rng.uniform(0, 7)),
            lambda: G.CRZ(p), G.Swap, lambda: G.U3(p, 0.2, q), lambda: G.CU1(rng.uniform(-7, 7)),
            lambda: G.CU1(q), G.CZ, lambda: G.U1(rng.uniform(0, 7)), G.T]
    seq = [("gate", make[int(rng.integers(0, len(make)))](), [0]) for _ in range(500)]
    want = np.concatenate([np.ascontiguousarray(op[1].matrix(), dtype=np.complex128).ravel()
                           for op in seq]).view(np.float64)
    got = GpuCircuit._flat(seq)
    assert got.dtype == np.float64 and np.array_equal(got, want)
    p.assign(-2.5)
    want2 = np.concatenate([np.ascontiguousarray(op[1].matrix(), dtype=np.complex128).ravel()
                            for op in seq]).view(np.float64)
    assert np.array_equal(GpuCircuit._flat(seq), want2) and not np.array_equal(want2, want)
