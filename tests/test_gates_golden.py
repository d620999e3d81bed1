"""Gate matrices against the reference's test_matrix known answers (CPU)."""
import numpy as np
import pytest

from q1tsim_gb300 import gates as G
from refcheck import KAT_TOL, dec, kats

K = kats()


@pytest.mark.parametrize("case", K["matrix"], ids=lambda c: c["gate"] + "@" + c["source"])
def test_matrix_kat(case):
    g = G.by_name(case["gate"], case["params"])
    np.testing.assert_allclose(g.matrix(), dec(case["expect"]), rtol=0, atol=KAT_TOL)


def _build(spec):
    if "gate" in spec:
        return G.by_name(spec["gate"], spec["params"])
    if "kron" in spec:
        return G.Kron(_build(spec["kron"][0]), _build(spec["kron"][1]))
    if "loop" in spec:
        return G.Loop("loop", spec["loop"], _build(spec["body"]))
    return G.Composite(spec["composite"], spec["nbits"], [(_build(op), bits) for op, bits in spec["ops"]])


@pytest.mark.parametrize("case", K["compound"], ids=lambda c: c["source"])
def test_compound_matrix_kat(case):
    """Kron, Composite and Loop gates built from parts, against the reference's
    test_matrix known answers."""
    np.testing.assert_allclose(_build(case["spec"]).matrix(), dec(case["expect"]), rtol=0, atol=KAT_TOL)


@pytest.mark.parametrize("case", K["apply"], ids=lambda c: c["gate"] + "@" + c["source"])
def test_apply_matrix_is_reference_gate(case):
    """The matrices the apply KATs use are the ones gates.py builds."""
    g = G.by_name(case["gate"], case["params"])
    np.testing.assert_allclose(g.matrix(), dec(case["mat"]), rtol=0, atol=KAT_TOL)


def test_all_named_gates_unitary():
    rng = np.random.default_rng(1)
    for name, (ctor, npar) in G._BY_NAME.items():
        g = ctor(*rng.uniform(0, 2 * np.pi, npar))
        m = g.matrix()
        assert m.shape == (1 << g.nr_affected_bits(),) * 2
        np.testing.assert_allclose(m @ m.conj().T, np.eye(m.shape[0]), atol=1e-14)


def test_controlled_structure():
    """C<G> puts G in the bottom-right block (src/gates/controlled.rs:62-71)."""
    m = G.CU1(0.3).matrix()
    np.testing.assert_allclose(m, np.diag([1, 1, 1, np.exp(0.3j)]), atol=1e-15)
    m = G.CCX().matrix()
    want = np.eye(8)
    want[6:, 6:] = [[0, 1], [1, 0]]
    np.testing.assert_allclose(m, want, atol=0)


def test_parameter_reference_reevaluates():
    p = G.Parameter(0.5)
    g = G.RX(p)
    m1 = g.matrix()
    p.assign(1.5)
    m2 = g.matrix()
    np.testing.assert_allclose(m2, G.RX(1.5).matrix(), atol=0)
    assert not np.allclose(m1, m2)


def test_by_name_errors():
    with pytest.raises(G.UnknownGate):
        G.by_name("foo")
    with pytest.raises(G.InvalidNrArguments):
        G.by_name("U3", [1.0])


def test_composite_and_loop():
    c = G.Composite("HX", 2, [(G.H(), [0]), (G.CX(), [0, 1])])
    want = G.CX().matrix() @ np.kron(G.H().matrix(), np.eye(2))
    np.testing.assert_allclose(c.matrix(), want, atol=1e-15)
    lp = G.Loop("sq", 2, G.S())
    np.testing.assert_allclose(lp.matrix(), G.Z().matrix(), atol=1e-15)
    k = G.Kron(G.H(), G.X())
    np.testing.assert_allclose(k.matrix(), np.kron(G.H().matrix(), G.X().matrix()), atol=0)
