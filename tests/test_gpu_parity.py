"""Parity of the CUDA engine with the CPU oracle, through the C ABI.

complex128 mode: max |d amp| <= 1e-12 against the oracle and identical shot
outcomes for identical uniforms.  complex64 mode (plain and fused):
max |d amp| <= 2e-6 on normalised states and 1 - fidelity <= 1e-6.
"""
import numpy as np
import pytest

from oracle import oracle as orc
from q1tsim_gb300 import Circuit, Plan, Rng, VectorState, workloads
from q1tsim_gb300 import _lib
from q1tsim_gb300 import gates as G
from refcheck import dec, kats, measurement_ok

pytestmark = pytest.mark.gpu

TOL128 = 1e-12
TOL64 = 2e-6
K = kats()


def rand_state(n, rng):
    a = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    return a / np.linalg.norm(a)


def pair(n, shots, amps=None, prec="c128"):
    if amps is None:
        return orc.OracleState.new(n, shots), VectorState(n, shots, prec)
    return orc.OracleState.from_amplitudes(amps, shots), VectorState.from_amplitudes(amps, shots, prec)


def same(o, g, tol=TOL128):
    assert g.counts == o.counts
    so, sg = o.states(), g.states()
    assert so.shape == sg.shape
    np.testing.assert_allclose(sg, so, rtol=0, atol=tol)


def random_gate(n, rng):
    kinds = ["u3", "h", "x", "y", "z", "s", "t", "rz", "rx", "v", "cx", "cz", "cy", "ch", "cu1",
             "crz", "swap", "ccx", "ccz", "kron", "u3u3", "dense3", "cu3"]
    if n < 3:
        kinds = [k for k in kinds if k not in ("ccx", "ccz", "dense3")]
    if n < 2:
        kinds = [k for k in kinds if k in ("u3", "h", "x", "y", "z", "s", "t", "rz", "rx", "v")]
    k = kinds[rng.integers(len(kinds))]
    ang = rng.uniform(0, 2 * np.pi, 3)
    one = {"u3": G.U3(*ang), "h": G.H(), "x": G.X(), "y": G.Y(), "z": G.Z(), "s": G.S(), "t": G.T(),
           "rz": G.RZ(ang[0]), "rx": G.RX(ang[0]), "v": G.V()}
    if k in one:
        return one[k], [int(rng.integers(n))]
    if k in ("cx", "cz", "cy", "ch", "cu1", "crz", "swap", "kron", "u3u3", "cu3"):
        b = [int(v) for v in rng.choice(n, 2, replace=False)]
        g = {"cx": G.CX(), "cz": G.CZ(), "cy": G.CY(), "ch": G.CH(), "cu1": G.CU1(ang[0]),
             "crz": G.CRZ(ang[1]), "swap": G.Swap(), "kron": G.Kron(G.H(), G.H()),
             "u3u3": G.Kron(G.U3(*ang), G.RY(ang[1])), "cu3": G.CU3(*ang)}[k]
        return g, b
    b = [int(v) for v in rng.choice(n, 3, replace=False)]
    if k == "ccx":
        return G.CCX(), b
    if k == "ccz":
        return G.CCZ(), b
    c = G.Composite("d3", 3, [(G.U3(*ang), [0]), (G.CX(), [0, 1]), (G.U3(*ang[::-1]), [2]),
                              (G.CZ(), [1, 2]), (G.H(), [1])])
    return c, b


# ------------------------------------------------------------------ KATs

# complex128 in FP64 (the reference's rounding) and in the default
# double-float arithmetic (about 47 bits; contract 1e-12)
MODES = [("c128", True, 1e-14), ("c128", False, 1e-13), ("c64", False, TOL64)]


@pytest.mark.parametrize("prec,exact,tol", MODES, ids=["c128-fp64", "c128", "c64"])
@pytest.mark.parametrize("case", K["vectorstate"], ids=lambda c: c["name"])
def test_vectorstate_kats_on_gpu(case, prec, exact, tol):
    init = case["init"]
    if init["kind"] == "new":
        s = VectorState(init["nr_bits"], init["nr_shots"], prec)
    else:
        s = VectorState.from_qubit_coefs(dec(init["coefs"]), init["nr_shots"], prec)
    if exact:
        s.set_fp64_exact()
    for op in case["ops"]:
        if op["op"] == "gate":
            s.apply_gate(dec(op["mat"]), op["bits"])
        elif op["op"] == "cond":
            s.apply_conditional_gate(op["control"], dec(op["mat"]), op["bits"])
        else:
            s.reset_all()
    assert s.counts == case["expect"]["counts"]
    np.testing.assert_allclose(s.states(), dec(case["expect"]["states"]), rtol=0, atol=tol)


@pytest.mark.parametrize("exact,tol", [(True, 1e-14), (False, 1e-13)], ids=["fp64", "df64"])
@pytest.mark.parametrize("case", K["apply"], ids=lambda c: c["gate"] + "@" + c["source"])
def test_gate_apply_kats_on_gpu(case, exact, tol):
    state, expect, mat = dec(case["state"]), dec(case["expect"]), dec(case["mat"])
    for c in range(state.shape[1]):
        s = VectorState.from_amplitudes(state[:, c], 1)
        if exact:
            s.set_fp64_exact()
        s.apply_gate(mat, case["bits"])
        np.testing.assert_allclose(s.states()[:, 0], expect[:, c], rtol=0, atol=tol)


# ------------------------------------------------------ random circuits

@pytest.mark.parametrize("exact", [False, True], ids=["df64", "fp64"])
@pytest.mark.parametrize("n", [1, 2, 3, 5, 8, 11, 13])
def test_random_gates_c128_match_oracle(n, exact):
    rng = np.random.default_rng(100 + n)
    amps = rand_state(n, rng)
    o, g = pair(n, 64, amps)
    if exact:
        g.set_fp64_exact()
    for _ in range(60):
        gate, bits = random_gate(n, rng)
        o.apply_gate(gate.matrix(), bits)
        g.apply_gate(gate, bits)
    same(o, g)


def test_c128_gates_on_extreme_magnitudes():
    """complex128 pair and phase updates run on split double-float pairs;
    amplitudes of 2^126 and more take the FP64 path per pair, those below
    2^-126 are flushed to zero.  All within 1e-12 of the oracle, relative to
    each amplitude's scale, and the oracle's zeros stay zero."""
    rng = np.random.default_rng(77)
    n = 10
    amps = rand_state(n, rng)
    amps[rng.random(1 << n) < 0.2] = 0.0
    tiny = rng.random(1 << n) < 0.1
    amps[tiny] *= 1e-30
    big = rng.random(1 << n) < 0.05
    amps[big] *= 1e140
    o, g = pair(n, 1, amps)
    gates = [(G.U3(0.3, 1.1, -0.4), [2]), (G.H(), [9]), (G.T(), [4]), (G.CU1(0.77), [1, 8]), (G.RX(2.2), [0]),
             (G.X(), [5]), (G.Y(), [3]), (G.CX(), [6, 7]), (G.S(), [2]), (G.Swap(), [0, 9])]
    for gt, b in gates:
        o.apply_gate(gt.matrix(), b)
        g.apply_gate(gt, b)
    so, sg = o.states()[:, 0], g.states()[:, 0]
    err = np.abs(sg - so) / np.maximum(np.abs(so), 1.0)
    assert float(np.max(err)) <= 1e-12, float(np.max(err))
    assert np.all(sg[so == 0] == 0)


def test_c128_unit_matrices_move_amplitudes_exactly():
    """X, Y, CX, CY, Swap, Z, S and controlled forms only move and re-sign
    amplitudes: bit-identical to the oracle."""
    rng = np.random.default_rng(78)
    n = 9
    amps = rand_state(n, rng)
    o, g = pair(n, 1, amps)
    for gt, b in [(G.X(), [0]), (G.Y(), [4]), (G.CX(), [2, 5]), (G.CY(), [8, 1]), (G.Swap(), [3, 6]),
                  (G.Z(), [7]), (G.S(), [2]), (G.Sdg(), [5]), (G.CZ(), [0, 4]), (G.CCX(), [1, 2, 3])]:
        o.apply_gate(gt.matrix(), b)
        g.apply_gate(gt, b)
    assert np.array_equal(o.states(), g.states())


@pytest.mark.parametrize("n", [2, 6, 12])
def test_random_gates_c64_match_oracle(n):
    rng = np.random.default_rng(200 + n)
    amps = rand_state(n, rng)
    o, g = pair(n, 64, amps, "c64")
    for _ in range(40):
        gate, bits = random_gate(n, rng)
        o.apply_gate(gate.matrix(), bits)
        g.apply_gate(gate, bits)
    so, sg = o.states()[:, 0], g.states()[:, 0]
    assert np.max(np.abs(so - sg)) <= TOL64
    assert 1 - abs(np.vdot(so, sg)) ** 2 <= 1e-6


def test_multi_column_gates_and_conditionals():
    """Gates act on every column; conditional gates split columns by run
    (src/vectorstate.rs:193-227)."""
    rng = np.random.default_rng(5)
    n, shots = 7, 40
    o, g = pair(n, shots, rand_state(n, rng))
    for step in range(6):
        control = rng.integers(0, 2, shots).astype(np.uint8)
        gate, bits = random_gate(n, rng)
        o.apply_conditional_gate(control, gate.matrix(), bits)
        g.apply_conditional_gate(control, gate, bits)
        same(o, g)
        gate, bits = random_gate(n, rng)
        o.apply_gate(gate.matrix(), bits)
        g.apply_gate(gate, bits)
        same(o, g)
    assert len(g.counts) > 1


# ---------------------------------------------------------- measurement

@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_measure_into_identical_outcomes(prec):
    rng = np.random.default_rng(9)
    n, shots = 9, 500
    o, g = pair(n, shots, rand_state(n, rng), prec)
    ro = np.zeros(shots, dtype=np.uint64)
    rg = np.zeros(shots, dtype=np.uint64)
    for step in range(8):
        q = int(rng.integers(n))
        cb = int(rng.integers(8))
        u = rng.random(len(o.counts))
        if step % 3 == 2:
            o.peek_into(q, cb, ro, uniforms=u)
            g.peek_into(q, cb, rg, uniforms=u)
        else:
            o.measure_into(q, cb, ro, uniforms=u)
            g.measure_into(q, cb, rg, uniforms=u)
        assert np.array_equal(ro, rg)
        assert g.counts == o.counts
        gate, bits = random_gate(n, rng)
        o.apply_gate(gate.matrix(), bits)
        g.apply_gate(gate, bits)
        if prec == "c128":
            same(o, g)
        else:
            np.testing.assert_allclose(g.states(), o.states(), atol=1e-5)


@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_measure_into_large_state_two_level_weights(prec):
    """23 qubits: the qubit weights reduce 2^14 chunk sums per column in two
    levels; outcomes and collapsed states still match the oracle."""
    rng = np.random.default_rng(23)
    n, shots = 23, 16
    o, g = pair(n, shots, rand_state(n, rng), prec)
    ro = np.zeros(shots, dtype=np.uint64)
    rg = np.zeros(shots, dtype=np.uint64)
    for q in (0, 22):
        u = rng.random(len(o.counts))
        o.measure_into(q, q % 8, ro, uniforms=u)
        g.measure_into(q, q % 8, rg, uniforms=u)
        assert np.array_equal(ro, rg)
        assert g.counts == o.counts
    tol = TOL128 if prec == "c128" else 1e-6
    np.testing.assert_allclose(g.states(), o.states(), rtol=0, atol=tol)


@pytest.mark.parametrize("prec", ["c128", "c64"])
@pytest.mark.parametrize("n", [1, 4, 10, 14])
def test_measure_all_identical_outcomes(prec, n):
    rng = np.random.default_rng(30 + n)
    shots = 3000
    o, g = pair(n, shots, rand_state(n, rng), prec)
    # split into a few columns first
    u0 = rng.random(1)
    ro = np.zeros(shots, dtype=np.uint64)
    rg = np.zeros(shots, dtype=np.uint64)
    o.measure_into(0, 40, ro, uniforms=u0)
    g.measure_into(0, 40, rg, uniforms=u0)
    cbits = [int(c) for c in rng.permutation(n)]
    u = rng.random(shots)
    o.peek_all_into(cbits, ro, uniforms=u)
    g.peek_all_into(cbits, rg, uniforms=u)
    assert np.array_equal(ro, rg)
    o.measure_all_into(cbits, ro, uniforms=u)
    g.measure_all_into(cbits, rg, uniforms=u)
    assert np.array_equal(ro, rg)
    assert g.counts == o.counts
    if (1 << n) * len(o.counts) <= (1 << 22):
        np.testing.assert_allclose(g.states(), o.states(), atol=0)
    # a gate after the collapse densifies the basis columns again
    gate, bits = random_gate(n, rng)
    o.apply_gate(gate.matrix(), bits)
    g.apply_gate(gate, bits)
    if (1 << n) * len(o.counts) <= (1 << 22):
        np.testing.assert_allclose(g.states(), o.states(), atol=1e-12 if prec == "c128" else 1e-6)


@pytest.mark.parametrize("prec", ["c128", "c64"])
@pytest.mark.parametrize("kind", ["sparse", "concentrated", "zero_tail"])
def test_measure_all_on_uneven_mass_matches_oracle(prec, kind):
    """Shots on 18-qubit states whose chunk prefix is mostly flat (a few
    nonzero amplitudes: ties between chunk prefixes and targets), whose mass
    sits in two amplitudes (one merge span takes most shots), or whose upper
    half is zero: the chunk of each shot, found by merging the sorted targets
    with the prefix, is the one the oracle's search finds, so the words are
    identical."""
    n, shots = 18, 40000
    rng = np.random.default_rng(77)
    amps = np.zeros(1 << n, dtype=np.complex128)
    if kind == "sparse":
        idx = rng.choice(1 << n, 24, replace=False)
        amps[idx] = rng.normal(size=24) + 1j * rng.normal(size=24)
    elif kind == "concentrated":
        amps[5] = 0.8
        amps[(1 << n) - 3] = 0.6j
        amps[rng.choice(1 << n, 50, replace=False)] += 1e-4
    else:
        amps[: 1 << (n - 1)] = rng.normal(size=1 << (n - 1)) + 1j * rng.normal(size=1 << (n - 1))
    amps /= np.linalg.norm(amps)
    o, g = pair(n, shots, amps, prec)
    cbits = list(range(n))
    u = rng.random(shots)
    ro = np.zeros(shots, dtype=np.uint64)
    rg = np.zeros(shots, dtype=np.uint64)
    o.peek_all_into(cbits, ro, uniforms=u)
    g.peek_all_into(cbits, rg, uniforms=u)
    if prec == "c128":
        assert np.array_equal(ro, rg)
    else:
        # complex64 probabilities: outcomes may differ only at a boundary
        assert np.mean(ro == rg) >= 0.999


def rand_unitary(d, rng):
    z = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


# qubit lists for 2-4 qubit blocks: the lowest and highest positions, runs and
# scattered sets (qubit q is position n-1-q)
TILE_QUBITS = [[-1, -2], [-4, -1], [0, -2], [3, 8], [-1, -2, -3], [2, 7, 0], [1, 5, -1], [-1, -2, -3, -4],
               [0, 3, 7, -1], [1, 2, 6, 8]]


@pytest.mark.parametrize("prec,tol", [("c128", TOL128), ("c64", TOL64)])
@pytest.mark.parametrize("n", [9, 10, 13])
def test_dense_blocks_in_warp_tiles_match_oracle(prec, tol, n):
    """Uncontrolled dense blocks take the warp-tile kernels: complex64 blocks
    of up to 4 qubits on states of 10+ qubits, complex128 blocks of up to 3
    qubits on double-float pairs on states of 9+ qubits (4-qubit complex128
    blocks keep the per-unit FP64 kernel).  Gate positions include 0 and the
    state's top positions; a second round runs on two columns after a
    measurement."""
    rng = np.random.default_rng(300 + n)
    shots = 64
    o, g = pair(n, shots, rand_state(n, rng), prec)

    def blocks():
        for qs in TILE_QUBITS:
            bits = [q % n for q in qs]
            m = rand_unitary(1 << len(bits), rng)
            o.apply_gate(m, bits)
            g.apply_gate(m, bits)

    blocks()
    np.testing.assert_allclose(g.states(), o.states(), rtol=0, atol=tol)
    u = np.array([0.5])
    ro = np.zeros(shots, dtype=np.uint64)
    rg = np.zeros(shots, dtype=np.uint64)
    o.measure_into(n // 2, 3, ro, uniforms=u)
    g.measure_into(n // 2, 3, rg, uniforms=u)
    assert np.array_equal(ro, rg) and g.counts == o.counts
    blocks()
    assert g.counts == o.counts
    np.testing.assert_allclose(g.states(), o.states(), rtol=0, atol=tol)


def test_c128_dense_blocks_on_extreme_magnitudes():
    """Tiled complex128 blocks: a unit with an amplitude of 2^126 or more is
    done in FP64, amplitudes below 2^-126 are flushed; within 1e-12 of the
    oracle relative to each amplitude's scale."""
    rng = np.random.default_rng(79)
    n = 11
    amps = rand_state(n, rng)
    amps[rng.random(1 << n) < 0.1] *= 1e-30
    amps[rng.random(1 << n) < 0.03] *= 1e140
    o, g = pair(n, 1, amps)
    for qs in ([0, 1], [10, 3, 5], [9, 2]):
        m = rand_unitary(1 << len(qs), rng)
        o.apply_gate(m, qs)
        g.apply_gate(m, qs)
    so, sg = o.states()[:, 0], g.states()[:, 0]
    err = np.abs(sg - so) / np.maximum(np.abs(so), 1.0)
    assert float(np.max(err)) <= 1e-12, float(np.max(err))


def _run_plan(n, gates, width, prec, amps, kinds=True):
    bits = [b for _, b in gates]
    mats = np.concatenate([np.ascontiguousarray(g.matrix()).ravel() for g, _ in gates]).view(np.float64)
    st = VectorState.from_amplitudes(amps, 1, prec)
    st.apply_plan(Plan(n, bits, width, kinds=[g.plan_kind() for g, _ in gates] if kinds else None), mats)
    return st


@pytest.mark.parametrize("n", [10, 13])
def test_qft_phase_runs_match_oracle(n):
    """The QFT with its controlled-phase ladders as phase-run passes (each
    with the next Hadamard), complex64 fused: against the complex128 oracle
    on a random state, as the 28-qubit QFT workload runs it."""
    rng = np.random.default_rng(400 + n)
    amps = rand_state(n, rng)
    q = workloads.qft(n, precision="c64", fusion_width=5, measure=False)
    gates = [(op[1], op[2]) for op in q.ops if op[0] == "gate"]
    o = orc.OracleState.from_amplitudes(amps, 1)
    for g, b in gates:
        o.apply_gate(g.matrix(), b)
    g64 = _run_plan(n, gates, 5, "c64", amps)
    so, sg = o.states()[:, 0], g64.states()[:, 0]
    assert float(np.max(np.abs(sg - so))) <= TOL64
    assert 1.0 - abs(np.vdot(so, sg)) ** 2 <= 1e-6


def test_random_phase_runs_match_oracle():
    """Runs of phases (RZ, T, S, Z, U1) and controlled phases (CU1, CZ, CRZ,
    CS) around a common qubit, between U3 and CX layers; some runs end in a
    1-qubit gate, one has no common qubit and stays fused as usual.
    complex64 against the oracle; complex128 (runs applied gate by gate)
    within 1e-12."""
    n = 12
    rng = np.random.default_rng(401)
    amps = rand_state(n, rng)
    gates = []
    for layer in range(6):
        for q in range(n):
            gates.append((G.U3(*rng.uniform(0, 2 * np.pi, 3)), [q]))
        pivot = int(rng.integers(n))
        for _ in range(int(rng.integers(3, 9))):
            kind = int(rng.integers(6))
            other = int(rng.choice([q for q in range(n) if q != pivot]))
            pair = [pivot, other] if rng.random() < 0.5 else [other, pivot]
            g = [G.CU1(rng.uniform(0, 6.3)), G.CZ(), G.CRZ(rng.uniform(0, 6.3)), G.CS(),
                 G.RZ(rng.uniform(0, 6.3)), G.T()][kind]
            gates.append((g, pair if kind < 4 else [int(rng.integers(n))]))
        if layer % 2:
            gates.append((G.H(), [int(rng.integers(n))]))
        for q in range(layer % 2, n - 1, 2):
            gates.append((G.CX(), [q, q + 1]))
    gates += [(G.CZ(), [q, (q + 1) % n]) for q in range(n)]   # no common qubit
    o = orc.OracleState.from_amplitudes(amps, 1)
    for g, b in gates:
        o.apply_gate(g.matrix(), b)
    so = o.states()[:, 0]
    s64 = _run_plan(n, gates, 5, "c64", amps).states()[:, 0]
    assert float(np.max(np.abs(s64 - so))) <= TOL64
    s128 = _run_plan(n, gates, 3, "c128", amps).states()[:, 0]
    assert float(np.max(np.abs(s128 - so))) <= TOL128


@pytest.mark.parametrize("prec", ["c64", "c128"])
@pytest.mark.parametrize("n", [9, 12, 14])
def test_swap_runs_move_amplitudes_exactly(prec, n):
    """Runs of swaps on disjoint qubit pairs (the QFT's closing reversal, and
    random pairings) as single permutation passes: bit-identical to the
    oracle applying the swaps one by one (9 qubits: the swaps one by one)."""
    rng = np.random.default_rng(500 + n)
    amps = rand_state(n, rng)
    rev = [(G.Swap(), [q, n - 1 - q]) for q in range(n // 2)]
    perm = [int(q) for q in rng.permutation(n)]
    rnd = [(G.Swap(), [perm[2 * k], perm[2 * k + 1]]) for k in range(n // 2 - 1)]
    gates = [(G.U3(0.3, 0.2, 0.1), [0])] + rev + [(G.H(), [n - 1])] + rnd
    o = orc.OracleState.from_amplitudes(amps, 1)
    for g, b in gates:
        o.apply_gate(g.matrix(), b)
    plan_kinds = [g.plan_kind() for g, _ in gates]
    assert plan_kinds.count(2) == len(rev) + len(rnd)
    s = _run_plan(n, gates, 2, prec, amps)
    so, sg = o.states()[:, 0], s.states()[:, 0]
    tol = TOL128 if prec == "c128" else TOL64
    np.testing.assert_allclose(sg, so, rtol=0, atol=tol)
    # the swaps alone move amplitudes without arithmetic
    o2 = orc.OracleState.from_amplitudes(amps, 1)
    for g, b in rev:
        o2.apply_gate(g.matrix(), b)
    s2 = _run_plan(n, rev, 2, prec, amps)
    exp = o2.states()[:, 0]
    if prec == "c64":
        exp = exp.astype(np.complex64).astype(np.complex128)
    assert np.array_equal(s2.states()[:, 0], exp)


def test_gate_wrongly_marked_diagonal_is_an_error():
    """A plan whose diagonal flags mark a non-diagonal gate fails at run time
    with an error, before any launch of that pass."""
    n = 10
    gates = [(G.CU1(0.3), [0, 1]), (G.CU1(0.4), [0, 2]), (G.H(), [0]), (G.CU1(0.5), [0, 3])]
    bits = [b for _, b in gates]
    mats = np.concatenate([np.ascontiguousarray(g.matrix()).ravel() for g, _ in gates]).view(np.float64)
    st = VectorState(n, 1, "c64")
    plan = Plan(n, bits, 5, diagonal=[True, True, True, True])
    with pytest.raises(Exception):
        st.apply_plan(plan, mats)


def _brick(n, depth, seed):
    rng = np.random.default_rng(seed)
    out = []
    for layer in range(depth):
        for q in range(n):
            out.append((G.U3(*rng.uniform(0, 2 * np.pi, 3)), [q]))
        for q in range(layer % 2, n - 1, 2):
            out.append((G.CX(), [q, q + 1]))
    return out


@pytest.mark.parametrize("prec,width", [("c64", 5), ("c64", 4), ("c128", 0), ("c128", 3)])
def test_plan_from_basis_state_runs_its_prefix_compact(prec, width):
    """From a basis state (24 qubits, the smallest size that takes this
    path), a plan's leading blocks touching at most n - 3 positions run on a
    compact state of those positions, scattered into the full one afterwards.
    The result equals the same plan run from a dense copy of |0...0>, which
    takes no prefix (the oracle checks that path elsewhere)."""
    n = 24
    gates = _brick(n, 4, 600 + width)
    bits = [b for _, b in gates]
    mats = np.concatenate([np.ascontiguousarray(g.matrix()).ravel() for g, _ in gates]).view(np.float64)
    plan = Plan(n, bits, width)
    e0 = np.zeros(1 << n, dtype=np.complex128)
    e0[0] = 1.0
    for _ in range(2):      # the second run reuses the plan's prefix and the compact state's buffers
        st = VectorState(n, 1, prec)
        st.apply_plan(plan, mats)
        dense = VectorState.from_amplitudes(e0, 1, prec)
        dense.apply_plan(plan, mats)
        acc = dense.compare(st)
        if prec == "c128":
            assert acc["max_abs_diff"] <= 1e-15, acc
        else:
            assert acc["max_abs_diff"] <= 1e-8 and acc["infidelity"] <= 1e-10, acc
        assert abs(acc["norm_b"] - 1.0) <= (1e-12 if prec == "c128" else 1e-6), acc


def test_prefix_from_a_nonzero_basis_state():
    """After measure_all collapses a 1-run 24-qubit state onto a basis state
    with ones in it, the next plan's compact prefix keeps the untouched
    positions at their measured values (against the oracle)."""
    n = 24
    rng = np.random.default_rng(601)
    amps = rand_state(n, rng)
    o, g = pair(n, 1, amps, "c128")
    u = np.array([0.37])
    ro = np.zeros(1, dtype=np.uint64)
    rg = np.zeros(1, dtype=np.uint64)
    o.measure_all_into(list(range(n)), ro, uniforms=u)
    g.measure_all_into(list(range(n)), rg, uniforms=u)
    assert np.array_equal(ro, rg) and int(ro[0]) != 0
    gates = [(G.U3(*rng.uniform(0, 6, 3)), [q]) for q in range(0, 8)] + [(G.CX(), [q, q + 1]) for q in range(0, 7)]
    for gt, b in gates:
        o.apply_gate(gt.matrix(), b)
    bits = [b for _, b in gates]
    mats = np.concatenate([np.ascontiguousarray(gt.matrix()).ravel() for gt, _ in gates]).view(np.float64)
    g.apply_plan(Plan(n, bits, 3), mats)
    np.testing.assert_allclose(g.states()[:, 0], o.states()[:, 0], rtol=0, atol=TOL128)


def test_rng_stream_matches_oracle():
    """The device-generated sorted uniforms agree with the oracle's host
    generation (same SplitMix64 stream); outcomes then agree except, with
    vanishing probability, at FP rounding boundaries."""
    rng = np.random.default_rng(77)
    n, shots = 12, 20000
    amps = rand_state(n, rng)
    o, g = pair(n, shots, amps)
    ro = np.zeros(shots, dtype=np.uint64)
    rg = np.zeros(shots, dtype=np.uint64)
    r1, r2 = orc.Rng(1234), Rng(1234)
    o.peek_all_into(list(range(n)), ro, rng=r1)
    g.peek_all_into(list(range(n)), rg, rng=r2)
    assert r1.state[1] == r2.counter == shots + 1
    assert np.mean(ro == rg) >= 0.999
    # single-qubit measurement draws one uniform per column on the host
    o.measure_into(3, 50, ro, rng=r1)
    g.measure_into(3, 50, rg, rng=r2)
    assert np.array_equal(ro >> np.uint64(50), rg >> np.uint64(50))


def test_reset_and_reset_all_parity():
    rng = np.random.default_rng(4)
    n, shots = 6, 200
    o, g = pair(n, shots, rand_state(n, rng))
    for q in (0, 3, 5):
        u = rng.random(len(o.counts))
        o.reset(q, uniforms=u)
        g.reset(q, uniforms=u)
        same(o, g)
    g.reset_all()
    o.reset_all()
    same(o, g)


def test_measurement_statistics_large_shot_count():
    """1e6 shots of a 20-qubit state: every qubit's marginal within the
    reference's binomial bounds (src/stats.rs)."""
    rng = np.random.default_rng(8)
    n, shots = 20, 1_000_000
    amps = rand_state(n, rng)
    g = VectorState.from_amplitudes(amps, shots, "c64")
    res = np.zeros(shots, dtype=np.uint64)
    g.peek_all_into(list(range(n)), res, rng=Rng(5))
    p = np.abs(amps) ** 2
    idx = np.arange(1 << n)
    for q in range(n):
        p1 = p[((idx >> (n - 1 - q)) & 1) == 1].sum()
        c1 = int(((res >> np.uint64(q)) & np.uint64(1)).sum())
        assert measurement_ok(c1, shots, p1, 1e-6)


# ------------------------------------------------------------- fusion

@pytest.mark.parametrize("width", [2, 3, 4, 5])
def test_fused_plans_match_plain(width):
    rng = np.random.default_rng(width)
    n = 13
    amps = rand_state(n, rng)
    gl = [random_gate(n, rng) for _ in range(80)]
    mats = np.concatenate([np.ascontiguousarray(gt.matrix()).ravel() for gt, _ in gl]).view(np.float64)
    o = orc.OracleState.from_amplitudes(amps, 1)
    for gt, b in gl:
        o.apply_gate(gt.matrix(), b)
    ref = o.states()[:, 0]
    for prec, tol in (("c128", TOL128), ("c64", TOL64)):
        g = VectorState.from_amplitudes(amps, 1, prec)
        p = Plan(n, [b for _, b in gl], width)
        g.apply_plan(p, mats)
        out = g.states()[:, 0]
        assert np.max(np.abs(out - ref)) <= tol, (prec, np.max(np.abs(out - ref)))
        # fidelity of the normalised states; the tensor cores' FP32
        # accumulation rounds toward zero, so the norm itself may drift by a
        # few 1e-8 per block (sampling divides by the total)
        nrm = np.linalg.norm(out)
        assert abs(nrm - 1.0) <= 1e-5, nrm
        assert 1 - abs(np.vdot(ref, out)) ** 2 / nrm ** 2 <= 1e-9


def test_tensor_core_block_is_exact_on_split_values():
    """A 3-qubit cyclic permutation (entries 0/1) on amplitudes with 20
    fraction bits goes through the tensor-core block kernel; hi + lo recovers
    every amplitude, so the result is exact, not rounded to 11 bits."""
    n = 12
    k = np.arange(1 << n) % 4096
    amps = ((1.0 + k * 2.0 ** -20) / 64.0).astype(np.complex128)
    P = np.zeros((8, 8), dtype=np.complex128)
    for s in range(8):
        P[(s + 1) % 8, s] = 1.0
    g = VectorState.from_amplitudes(amps, 1, "c64")
    g.apply_plan(Plan(n, [[0, 1, 2]], 3), P.ravel().view(np.float64))
    o = orc.OracleState.from_amplitudes(amps, 1)
    o.apply_gate(P, [0, 1, 2])
    out, ref = g.states()[:, 0], o.states()[:, 0]
    assert np.array_equal(out, ref), float(np.max(np.abs(out - ref)))


def cyclic_perm(k, shift):
    d = 1 << k
    P = np.zeros((d, d), dtype=np.complex128)
    for s in range(d):
        P[(s + shift) % d, s] = 1.0
    return P


def split_exact_amps(n):
    k = np.arange(1 << n) % 4096
    return ((1.0 + k * 2.0 ** -20) / 64.0 * (1 + 1j * (k % 3 == 0))).astype(np.complex128)


@pytest.mark.parametrize("n,qubits", [
    (12, [7, 8, 9, 10, 11]),      # lowest positions: gate pairs adjacent, padded stage
    (12, [0, 1, 2, 3, 4]),
    (14, [9, 10, 11, 12, 13]),
    (14, [1, 3, 5, 7, 9]),
    (14, [8, 9, 10, 11]),
    (15, [2, 7, 13]),
    (16, [0, 5, 10, 14, 15]),
])
@pytest.mark.parametrize("pairs", [1, 4])
def test_tensor_core_block_exact_any_layout(n, qubits, pairs):
    """Permutation blocks through the tensor cores on every tile layout (gate
    bits low or high, staged rows padded or not), with A in TMEM (two
    consumer groups) or in shared memory (four): hi + lo recover each
    amplitude, so the result equals the oracle's exactly."""
    amps = split_exact_amps(n)
    P = cyclic_perm(len(qubits), 3)
    g = VectorState.from_amplitudes(amps, 1, "c64")
    g.profile(True)
    plan = Plan(n, [qubits], 5)
    plan.set_tc_tiling(pairs, 8, 2)
    g.apply_plan(plan, P.ravel().view(np.float64))
    assert g.profile_report()["fused_tc_c64"]["launches"] == 1
    o = orc.OracleState.from_amplitudes(amps, 1)
    o.apply_gate(P, qubits)
    out, ref = g.states()[:, 0], o.states()[:, 0]
    assert np.array_equal(out, ref), float(np.max(np.abs(out - ref)))


@pytest.mark.parametrize("pairs,launches", [(1, 2), (4, 2), (5, 1)])
def test_two_blocks_share_one_tensor_core_pass(pairs, launches):
    """Consecutive blocks whose qubits fit one 12-position tile run in one
    pass over the state: two per pass, up to three in the four-group
    kernel's direct chain in pair mode 5; results stay exact."""
    n = 14
    amps = split_exact_amps(n)
    seq = [([0, 1, 2], cyclic_perm(3, 1)), ([11, 12, 13], cyclic_perm(3, 5)), ([5, 6, 7], cyclic_perm(3, 2))]
    mats = np.concatenate([m.ravel() for _, m in seq]).view(np.float64)
    g = VectorState.from_amplitudes(amps, 1, "c64")
    g.profile(True)
    plan = Plan(n, [b for b, _ in seq], 3)
    plan.set_tc_tiling(pairs, 8, 4)
    g.apply_plan(plan, mats)
    o = orc.OracleState.from_amplitudes(amps, 1)
    for b, m in seq:
        o.apply_gate(m, b)
    out, ref = g.states()[:, 0], o.states()[:, 0]
    assert np.array_equal(out, ref), float(np.max(np.abs(out - ref)))
    rep = g.profile_report()
    assert rep["fused_tc_c64"]["launches"] == launches, rep


@pytest.mark.parametrize("n,first,second", [
    (22, [1, 2, 3, 4, 5], [5, 6, 7, 8, 9]),        # tile runs of 8 amplitudes
    (20, [0, 1, 2, 3, 4], [3, 4, 5, 6, 7]),        # tile runs of 8, top position in the tile
])
def test_short_run_pair_goes_as_one_tensor_map_box(n, first, second):
    """Two overlapping 5-qubit blocks on high positions: their tile has short
    contiguous runs, so the pass copies it as one tensor-map box; exact."""
    amps = split_exact_amps(n)
    seq = [(first, cyclic_perm(5, 7)), (second, cyclic_perm(5, 11))]
    mats = np.concatenate([m.ravel() for _, m in seq]).view(np.float64)
    g = VectorState.from_amplitudes(amps, 1, "c64")
    g.profile(True)
    g.apply_plan(Plan(n, [b for b, _ in seq], 5), mats)
    o = orc.OracleState.from_amplitudes(amps, 1)
    for b, m in seq:
        o.apply_gate(m, b)
    out, ref = g.states()[:, 0], o.states()[:, 0]
    assert np.array_equal(out, ref), float(np.max(np.abs(out - ref)))
    assert g.profile_report()["fused_tc_c64"]["launches"] == 1


@pytest.mark.parametrize("n,first,second", [
    (14, [9, 10, 11, 12, 13], [7, 8, 9, 10, 11]),    # low positions, one run
    (16, [3, 4, 5, 6, 7], [1, 2, 3, 4, 5]),          # high positions: brick pair
    (22, [1, 2, 3, 4, 5], [5, 6, 7, 8, 9]),          # tile runs of 8 amplitudes
    (20, [0, 1, 2, 3, 4], [3, 4, 5, 6, 7]),          # top position in the tile
    (16, [0, 5, 10, 14, 15], [2, 3, 4, 5, 12]),      # scattered gate bits
    (18, [13, 14, 15, 16, 17], [4, 5, 6, 7, 8]),     # disjoint blocks
    (14, [4, 5, 6, 7, 8], [9, 10, 11, 12, 13]),      # second block on the lowest positions: 16-byte stores permuted per lane
    (16, [6, 7, 8, 9, 10], [3, 11, 12, 13, 14]),     # 8-byte stores permuted per lane
])
@pytest.mark.parametrize("mode", [3, 4])
def test_direct_pair_is_exact(n, first, second, mode):
    """Pair modes 3 and 4: the first block's write-back stores the second
    block's hi/lo operands in shared memory and its MMAs read them there
    (mode 4: in the four-group kernel, whose first block's operands are in
    shared memory too).  On permutation blocks and amplitudes that split
    exactly, the state equals the oracle's bit for bit, in one pass."""
    amps = split_exact_amps(n)
    seq = [(first, cyclic_perm(5, 7)), (second, cyclic_perm(5, 11))]
    mats = np.concatenate([m.ravel() for _, m in seq]).view(np.float64)
    plan = Plan(n, [b for b, _ in seq], 5)
    plan.set_tc_tiling(mode, 12, 2)
    g = VectorState.from_amplitudes(amps, 1, "c64")
    g.profile(True)
    g.apply_plan(plan, mats)
    o = orc.OracleState.from_amplitudes(amps, 1)
    for b, m in seq:
        o.apply_gate(m, b)
    out, ref = g.states()[:, 0], o.states()[:, 0]
    assert np.array_equal(out, ref), float(np.max(np.abs(out - ref)))
    assert g.profile_report()["fused_tc_c64"]["launches"] == 1


@pytest.mark.parametrize("n,blocks", [
    (16, [[9, 10, 11, 12, 13], [7, 8, 9, 10, 11], [5, 6, 7, 8, 9]]),      # brick windows, one run
    (20, [[3, 4, 5, 6, 7], [1, 2, 3, 4, 5], [0, 1, 2, 3, 4]]),           # high positions
    (22, [[0, 1, 2, 3, 4], [2, 3, 4, 5, 6], [4, 5, 6, 7, 8]]),            # top positions, runs of 8
    (20, [[0, 4, 8, 2, 6], [1, 3, 5, 7, 8], [2, 4, 6, 7, 5]]),           # scattered gate bits, one box
    (16, [[6, 7, 8, 9, 10], [8, 9, 10, 11, 12], [11, 12, 13, 14, 15]]),   # last block on the lowest positions
])
def test_direct_triple_is_exact(n, blocks):
    """Three blocks in one pass of the four-group kernel (pair mode 5):
    block b's write-back stores block b+1's operands in the stage.  On permutation
    blocks and amplitudes that split exactly, the state equals the oracle's
    bit for bit, in one launch."""
    amps = split_exact_amps(n)
    seq = [(b, cyclic_perm(5, 3 + 4 * k)) for k, b in enumerate(blocks)]
    mats = np.concatenate([m.ravel() for _, m in seq]).view(np.float64)
    plan = Plan(n, [b for b, _ in seq], 5)
    plan.set_tc_tiling(5, 12, 4)
    g = VectorState.from_amplitudes(amps, 1, "c64")
    g.profile(True)
    g.apply_plan(plan, mats)
    o = orc.OracleState.from_amplitudes(amps, 1)
    for b, m in seq:
        o.apply_gate(m, b)
    out, ref = g.states()[:, 0], o.states()[:, 0]
    assert np.array_equal(out, ref), float(np.max(np.abs(out - ref)))
    assert g.profile_report()["fused_tc_c64"]["launches"] == 1


def test_two_block_passes_random_circuit():
    """A 16-qubit random circuit fused to 5-qubit blocks (many of them paired
    into one pass) against the oracle."""
    rng = np.random.default_rng(21)
    n = 16
    amps = rand_state(n, rng)
    gl = [random_gate(n, rng) for _ in range(120)]
    mats = np.concatenate([np.ascontiguousarray(gt.matrix()).ravel() for gt, _ in gl]).view(np.float64)
    o = orc.OracleState.from_amplitudes(amps, 1)
    for gt, b in gl:
        o.apply_gate(gt.matrix(), b)
    ref = o.states()[:, 0]
    g = VectorState.from_amplitudes(amps, 1, "c64")
    g.profile(True)
    p = Plan(n, [b for _, b in gl], 5)
    g.apply_plan(p, mats)
    out = g.states()[:, 0]
    assert np.max(np.abs(out - ref)) <= TOL64
    assert 1 - abs(np.vdot(ref, out)) ** 2 / np.linalg.norm(out) ** 2 <= 1e-9
    assert g.profile_report()["fused_tc_c64"]["launches"] < p.nblocks


def test_plan_rerun_with_new_parameters():
    """Matrices are re-read on every run (src/gates/parameter.rs:23-75)."""
    n = 5
    th = G.Parameter(0.3)
    c = Circuit(n, n)
    for q in range(n):
        c.add_gate(G.RX(th), [q])
    c.measure_all(list(range(n)))
    c.execute(1000, Rng(1))
    h0 = c.histogram()
    th.assign(0.0)
    c.execute(1000, Rng(1))
    assert c.histogram() == {0: 1000}
    assert h0 != {0: 1000}


# ------------------------------------------------------------- circuits

def test_circuit_execute_kat():
    """src/circuit.rs:1455-1468"""
    c = Circuit(2, 2)
    c.add_gate(G.X(), [0])
    c.add_gate(G.X(), [1])
    c.add_gate(G.CX(), [0, 1])
    c.measure(0, 0)
    c.measure(1, 1)
    c.execute(5, Rng(0))
    assert list(c.cstate()) == [0b01] * 5


def test_circuit_conditional_kat():
    """src/circuit.rs:1619-1652 (c_state injected before reexecute)."""
    c = Circuit(2, 2)
    c.add_conditional_gate([0, 1], 1, G.X(), [1])
    c.measure_all([0, 1])
    c.execute(5, Rng(0))
    assert list(c.cstate()) == [0] * 5
    for control, target, qb, want in [([0, 1], 1, [1], [0b10, 0, 0, 0, 0]),
                                      ([0, 1], 2, [1], [0, 0b10, 0b10, 0, 0]),
                                      ([1], 1, [0], [0, 0b01, 0b01, 0b01, 0])]:
        c = Circuit(2, 2)
        c.q_state = VectorState(2, 5)
        c.c_state = np.array([0b01, 0b10, 0b10, 0b11, 0b00], dtype=np.uint64)
        c.add_conditional_gate(control, target, G.X(), qb)
        c.measure_all([0, 1])
        c.reexecute(Rng(1))
        assert list(c.cstate()) == want


def test_circuit_measure_all_and_basis_kats():
    """src/circuit.rs:1654-1733"""
    n = 1024
    c = Circuit(2, 2)
    c.x(0)
    c.measure_all([0, 1])
    c.execute(n, Rng(2))
    assert c.histogram_vec() == [0, n, 0, 0]
    c = Circuit(2, 2)
    c.x(0)
    c.measure_all([1, 0])
    c.execute(n, Rng(2))
    assert c.histogram_vec() == [0, 0, n, 0]
    c = Circuit(2, 2)
    c.h(0)
    c.h(1)
    c.measure_all([0, 1])
    c.execute(n, Rng(3))
    assert all(measurement_ok(v, n, 0.25) for v in c.histogram_vec())
    c = Circuit(2, 2)
    c.h(0)
    c.h(1)
    c.measure_all_basis([0, 1], "x")
    c.execute(n, Rng(3))
    assert c.histogram_vec() == [n, 0, 0, 0]
    c = Circuit(2, 2)
    c.x(0)
    c.h(0)
    c.h(1)
    c.s(0)
    c.s(1)
    c.measure_all_basis([0, 1], "y")
    c.execute(n, Rng(3))
    assert c.histogram_vec() == [0, n, 0, 0]


@pytest.mark.parametrize("prec,exact,tol", [("c128", False, 1e-12), ("c128", True, 1e-13), ("c64", False, TOL64)],
                         ids=["c128", "c128-fp64", "c64"])
@pytest.mark.parametrize("n", [3, 11, 14])
def test_unary_gate_all_matches_oracle(n, prec, exact, tol):
    """apply_unary_gate_all (src/vectorstate.rs:180-189) runs the n one-qubit
    gates as fused blocks (one pass per 5 qubits in complex64, per 3 in
    complex128; one by one with FP64 arithmetic): the oracle's amplitudes,
    on a multi-column state."""
    rng = np.random.default_rng(60 + n)
    o, g = pair(n, 16, rand_state(n, rng), prec)
    if exact:
        g.set_fp64_exact()
    for m in (G.H().matrix(), G.U3(*rng.uniform(0, 2 * np.pi, 3)).matrix(), G.Sdg().matrix()):
        o.apply_unary_gate_all(m)
        g.apply_unary_gate_all(m)
    so, sg = o.states(), g.states()
    assert np.max(np.abs(so - sg)) <= tol


@pytest.mark.parametrize("prec", ["c128", "c64"])
@pytest.mark.parametrize("basis", ["x", "y"])
def test_basis_change_and_shots_at_20_qubits(basis, prec):
    """The X- and Y-basis change of measure_all / peek_all
    (src/circuit.rs:692-703) at 20 qubits: apply_unary_gate_all with H, or
    with H Sdg, on a random state.  Amplitudes against the oracle (1e-12 in
    complex128; 2e-6 and 1 - F <= 1e-9 in complex64), then peek_all with the
    same uniforms: identical words in complex128; in complex64, whose
    rounding can move a shot across an outcome boundary, at least 99 %."""
    n, shots = 20, 4096
    rng = np.random.default_rng(70)
    amps = rand_state(n, rng)
    m = G.H().matrix() if basis == "x" else G.H().matrix() @ G.Sdg().matrix()
    o, g = pair(n, shots, amps, prec)
    o.apply_unary_gate_all(m)
    g.apply_unary_gate_all(m)
    so, sg = o.states()[:, 0], g.states()[:, 0]
    err = float(np.max(np.abs(so - sg)))
    infid = 1.0 - abs(np.vdot(so, sg)) ** 2 / np.vdot(sg, sg).real
    u = np.sort(rng.random(shots))
    want = np.zeros(shots, dtype=np.uint64)
    got = np.zeros(shots, dtype=np.uint64)
    o.peek_all_into(list(range(n)), want, uniforms=u)
    g.peek_all_into(list(range(n)), got, uniforms=u)
    same_words = float(np.mean(got == want))
    if prec == "c128":
        assert err <= 1e-12
        assert same_words == 1.0
    else:
        assert err <= TOL64 and infid <= 1e-9, (err, infid)
        assert same_words >= 0.99, (same_words, err, infid)


@pytest.mark.parametrize("prec", ["c128", "c64"])
@pytest.mark.parametrize("basis", ["x", "y"])
def test_basis_measure_all_circuit_matches_oracle(basis, prec):
    """X- and Y-basis measure_all through the Circuit op interpreter: the
    basis change, the collapse onto one basis column per distinct outcome and
    the change back (src/circuit.rs:692-703), against the oracle backend for
    the same seed.  The oracle stores the collapsed columns densely
    (src/vectorstate.rs:150-158), so the case stays small."""
    n, shots = 9, 256
    def build(p, width):
        c = Circuit(n, n, precision=p, fusion_width=width)
        r = np.random.default_rng(99)
        for layer in range(3):
            for q in range(n):
                c.add_gate(G.U3(*r.uniform(0, 2 * np.pi, 3)), [q])
            for q in range(layer % 2, n - 1, 2):
                c.add_gate(G.CX(), [q, q + 1])
        c.measure_all_basis(list(range(n)), basis)
        c.peek_all_basis(list(range(n)), basis)
        return c
    c = build(prec, 5 if prec == "c64" else 3)
    c.execute(shots, Rng(31))
    got = c.cstate().copy()
    ref = build("c128", 0)
    ref.execute_with(shots, Rng(31), orc.OracleState.new(n, shots))
    want = ref.cstate()
    assert float(np.mean(got == want)) >= (1.0 if prec == "c128" else 0.99)


def test_circuit_peek_all_kat():
    """src/circuit.rs:1736-1760"""
    n = 1024
    c = Circuit(1, 3)
    c.h(0)
    c.peek_all([0])
    c.h(0)
    c.peek_all([1])
    c.h(0)
    c.peek_all([2])
    c.execute(n, Rng(4))
    h = c.histogram_vec()
    assert measurement_ok(h[0] + h[2] + h[4] + h[6], n, 0.5)
    assert h[0] + h[1] + h[4] + h[5] == n
    assert measurement_ok(h[0] + h[1] + h[2] + h[3], n, 0.5)


def test_circuit_reset_and_histograms():
    """src/circuit.rs:1851-1986"""
    n = 1024
    c = Circuit(2, 2)
    c.h(0)
    c.z(0)
    c.x(1)
    c.reset(0)
    c.measure(0, 0)
    c.measure(1, 1)
    c.execute(n, Rng(6))
    assert c.histogram_vec() == [0, 0, n, 0]
    c = Circuit(5, 5)
    c.h(0)
    c.z(0)
    c.x(4)
    c.h(3)
    c.reset_all()
    c.measure_all([0, 1, 2, 3, 4])
    c.execute(n, Rng(6))
    h = c.histogram_vec()
    assert h[0] == n and sum(h[1:]) == 0
    c = Circuit(2, 2)
    c.add_gate("H", [0])
    c.add_gate("h", [1])
    c.measure(0, 0)
    c.measure(1, 1)
    c.execute(4096, Rng(7))
    hs = c.histogram_string()
    assert sorted(hs) == ["00", "01", "10", "11"]
    assert sum(hs.values()) == 4096
    assert all(measurement_ok(v, 4096, 0.25) for v in hs.values())


def test_circuit_gpu_equals_oracle_backend():
    """The same Circuit op list executed by the oracle and by the GPU state
    gives identical classical results for the same uniform stream."""
    rng = np.random.default_rng(12)
    n = 8
    c = Circuit(n, n + 2)
    for layer in range(6):
        for q in range(n):
            c.add_gate(G.U3(*rng.uniform(0, 6.28, 3)), [q])
        for q in range(layer % 2, n - 1, 2):
            c.cx(q, q + 1)
        if layer == 2:
            c.measure(3, n)
            c.add_conditional_gate([n], 1, G.X(), [3])
        if layer == 4:
            c.measure(5, n + 1, "x")
    c.measure_all(list(range(n)))
    c.execute_with(2000, Rng(99), VectorState(n, 2000))
    gpu = c.cstate().copy()
    c.execute_with(2000, Rng(99), orc.OracleState.new(n, 2000))
    assert np.array_equal(c.cstate(), gpu)


# --------------------------------------------------------------- errors

def test_error_codes_on_gpu():
    """Status codes and payloads of the reference's Error variants
    (src/vectorstate.rs:112-116, 172, 199, 242-246), so that a binding can
    rebuild e.g. Error::NotEnoughSpace(2, 4) by value."""
    s = VectorState(3, 4)
    cases = [
        (_lib.InvalidNrBits, (1, 2), lambda: s.apply_gate(G.CX(), [0])),
        (_lib.InvalidQBit, (3,), lambda: s.apply_gate(G.H(), [3])),
        (_lib.NotEnoughSpace, (2, 4), lambda: s.measure_into(0, 0, np.zeros(2, dtype=np.uint64), Rng(0))),
        (_lib.NotEnoughSpace, (3, 4), lambda: s.peek_all_into([0, 1, 2], np.zeros(3, dtype=np.uint64), Rng(0))),
        (_lib.InvalidNrMeasurementBits, (2, 3),
         lambda: s.measure_all_into([0, 1], np.zeros(4, dtype=np.uint64), Rng(0))),
        (_lib.InvalidNrControlBits, (3, 4), lambda: s.apply_conditional_gate([1, 0, 1], G.X(), [0])),
        (_lib.InvalidQBit, (5,), lambda: s.measure_into(5, 0, np.zeros(4, dtype=np.uint64), Rng(0))),
        (_lib.InvalidCBit, (70,), lambda: s.measure_into(0, 70, np.zeros(4, dtype=np.uint64), Rng(0))),
    ]
    for cls, payload, call in cases:
        with pytest.raises(cls) as ei:
            call()
        assert ei.value.payload == payload, (cls, ei.value.payload)


def test_autotuned_circuit_matches_oracle():
    """fusion_width="auto": the autotuner times the candidates and the chosen
    plan gives the oracle's state."""
    from q1tsim_gb300 import autotune, workloads
    n = 13
    c = workloads.brick(n, 6, 44, precision="c64", fusion_width="auto", measure=False)
    st = VectorState(n, 1, "c64")
    c.execute_with(1, Rng(1), st)
    o = orc.OracleState.new(n, 1)
    for op in c.ops:
        o.apply_gate(op[1].matrix(), op[2])
    ref, out = o.states()[:, 0], st.states()[:, 0]
    assert 1 - abs(np.vdot(ref, out)) ** 2 / np.linalg.norm(out) ** 2 <= 1e-9
    assert len(autotune.tune.last_timings) >= 5
    assert autotune.tune.last_timings[0]["seconds"] <= autotune.tune.last_timings[-1]["seconds"]
    # the tensor-core tilings were among the candidates timed
    tilings = {(t["pairs"], t["max_high_positions"], t["conflict_slack"]) for t in autotune.tune.last_timings}
    assert set(autotune.TC_TILINGS) <= tilings


@pytest.mark.parametrize("tiling", [(2, 5, 2), (1, 5, 2), (0, 5, 2), (2, 8, 2), (2, 5, 4), (2, 12, 64), (1, 12, 64),
                                    (3, 5, 2), (3, 8, 2), (3, 12, 64), (4, 8, 2), (4, 8, 4), (4, 12, 64),
                                    (5, 8, 4), (5, 12, 64)])
def test_tc_tilings_match_oracle(tiling):
    """Every tensor-core tiling (pairs through registers, through the staged
    tile, as operands the first block stores for the second, or none; pairs
    over more large pages; unpadded tiles kept at more bank conflicts) gives
    the oracle's state."""
    rng = np.random.default_rng(31)
    n = 19
    gl = [random_gate(n, rng) for _ in range(80)]
    bits = [b for _, b in gl]
    mats = np.concatenate([np.ascontiguousarray(gt.matrix()).ravel() for gt, _ in gl]).view(np.float64)
    amps = rand_state(n, rng)
    o = orc.OracleState.from_amplitudes(amps, 1)
    for gt, b in gl:
        o.apply_gate(gt.matrix(), b)
    plan = Plan(n, bits, 5)
    plan.set_tc_tiling(*tiling)
    g = VectorState.from_amplitudes(amps, 1, "c64")
    g.profile(True)
    g.apply_plan(plan, mats)
    assert g.profile_report()["fused_tc_c64"]["launches"] > 0
    want, got = o.states()[:, 0], g.states()[:, 0]
    assert np.max(np.abs(got - want)) <= TOL64
    assert 1 - abs(np.vdot(want, got)) ** 2 <= 1e-6


@pytest.mark.parametrize("pairs", [1, 3, 4])
def test_tensor_core_plan_with_many_tiles_per_sm_matches_oracle(pairs):
    """21 qubits: 512 tiles of 4096 amplitudes, so every SM's CTA takes
    several tiles and both consumer groups of the tensor-core kernel work
    (at 12-16 qubits a CTA has one tile at most).  A brick of U3/CX fused
    into 5-qubit blocks, one- and two-block passes (the second block reading
    the staged tile, or operands stored for it), against the oracle."""
    n = 21
    rng = np.random.default_rng(2101)
    gates = []
    for layer in range(6):
        for q in range(n):
            gates.append((G.U3(*rng.uniform(0, 2 * np.pi, 3)), [q]))
        for q in range(layer % 2, n - 1, 2):
            gates.append((G.CX(), [q, q + 1]))
    amps = rand_state(n, rng)
    o = orc.OracleState.from_amplitudes(amps, 1)
    for gt, b in gates:
        o.apply_gate(gt.matrix(), b)
    ref = o.states()[:, 0]
    mats = np.concatenate([np.ascontiguousarray(gt.matrix()).ravel() for gt, _ in gates]).view(np.float64)
    g = VectorState.from_amplitudes(amps, 1, "c64")
    plan = Plan(n, [b for _, b in gates], 5)
    plan.set_tc_tiling(pairs, 8, 2)
    g.apply_plan(plan, mats)
    out = g.states()[:, 0]
    assert np.max(np.abs(out - ref)) <= TOL64, float(np.max(np.abs(out - ref)))
    assert 1 - abs(np.vdot(ref, out)) ** 2 / np.linalg.norm(out) ** 2 <= 1e-9


@pytest.mark.parametrize("pairs", [1, 3, 4])
def test_tensor_core_stage_reuse_matches_complex128(pairs):
    """24 qubits: 4096 tiles, about 27 per CTA, so each consumer group takes
    several tiles and every shared-memory stage is reused many times, in
    rings of 5 or 6 stages (padded pairs take 5).  A brick of U3/CX fused
    into 5-qubit blocks (pairs of low and high positions among them) in
    each pair mode, against the same circuit gate by gate in complex128 (whose
    kernels the oracle pins)."""
    n = 24
    rng = np.random.default_rng(2402)
    gates = []
    for layer in range(8):
        for q in range(n):
            gates.append((G.U3(*rng.uniform(0, 2 * np.pi, 3)), [q]))
        for q in range(layer % 2, n - 1, 2):
            gates.append((G.CX(), [q, q + 1]))
    bits = [b for _, b in gates]
    mats = np.concatenate([np.ascontiguousarray(gt.matrix()).ravel() for gt, _ in gates]).view(np.float64)
    ref = VectorState(n, 1, "c128")
    ref.apply_plan(Plan(n, bits, 0), mats)
    g = VectorState(n, 1, "c64")
    plan = Plan(n, bits, 5)
    plan.set_tc_tiling(pairs, 8, 2)
    g.profile(True)
    for _ in range(2):
        g.reset_all()
        g.apply_plan(plan, mats)
    assert g.profile_report()["fused_tc_c64"]["launches"] > 0
    acc = ref.compare(g)
    assert acc["max_abs_diff"] <= 1e-6 and acc["infidelity"] <= 1e-9, acc


def test_norm_correction_left_pending_until_needed():
    """A tensor-core plan leaves its norm correction pending: peek_all on the
    unsettled state samples the same outcomes as on a settled copy (sampling
    divides by the column totals), and a single-qubit measurement settles
    first, so both copies end in the same state with the input norm."""
    rng = np.random.default_rng(31)
    n = 14
    amps = rand_state(n, rng)
    gl = [random_gate(n, rng) for _ in range(60)]
    mats = np.concatenate([np.ascontiguousarray(gt.matrix()).ravel() for gt, _ in gl]).view(np.float64)
    plan = Plan(n, [b for _, b in gl], 5)
    shots = 64
    a = VectorState.from_amplitudes(amps, shots, "c64")
    b = VectorState.from_amplitudes(amps, shots, "c64")
    a.apply_plan(plan, mats)
    b.apply_plan(plan, mats)
    b.states()                                   # settles b
    u = np.sort(rng.random(shots))
    ra = np.zeros(shots, dtype=np.uint64)
    rb = np.zeros(shots, dtype=np.uint64)
    a.peek_all_into(list(range(n)), ra, uniforms=u)
    b.peek_all_into(list(range(n)), rb, uniforms=u)
    assert np.array_equal(ra, rb)
    u1 = rng.random(shots)
    ma = np.zeros(shots, dtype=np.uint64)
    mb = np.zeros(shots, dtype=np.uint64)
    a.measure_into(3, 0, ma, uniforms=u1)
    b.measure_into(3, 0, mb, uniforms=u1)
    assert np.array_equal(ma, mb)
    acc = b.compare(a)
    # after the measurement each column (one per outcome) has norm 1
    assert acc["max_abs_diff"] <= 1e-7 and abs(acc["norm_b"] - acc["norm_a"]) <= 1e-6, acc
    assert abs(acc["norm_b"] - round(acc["norm_b"])) <= 1e-6, acc


def test_fused_plan_renormalises_to_the_input_norm():
    """After a tensor-core plan the column norms equal the input norms (an
    unnormalised input keeps its norm)."""
    rng = np.random.default_rng(17)
    n = 14
    amps = 1.7 * rand_state(n, rng)
    gl = [random_gate(n, rng) for _ in range(60)]
    mats = np.concatenate([np.ascontiguousarray(gt.matrix()).ravel() for gt, _ in gl]).view(np.float64)
    g = VectorState.from_amplitudes(amps, 1, "c64")
    g.apply_plan(Plan(n, [b for _, b in gl], 5), mats)
    out = g.states()[:, 0]
    assert abs(np.linalg.norm(out) ** 2 / 1.7 ** 2 - 1.0) <= 2e-6


@pytest.mark.parametrize("n", [14, 21])
def test_fused_plan_on_a_column_of_tiny_norm(n):
    """A column whose squared norm is 2^-20 (as a rare branch would be
    before renormalisation) through tensor-core passes: its amplitudes enter
    the f16 operands scaled by 2^14 / 2^ceil(log2 sqrt(norm)), so the result
    matches the oracle to the same relative accuracy as a unit column."""
    rng = np.random.default_rng(23 + n)
    scale = 2.0 ** -10
    amps = scale * rand_state(n, rng)
    gl = [random_gate(n, rng) for _ in range(40)]
    mats = np.concatenate([np.ascontiguousarray(gt.matrix()).ravel() for gt, _ in gl]).view(np.float64)
    o = orc.OracleState.from_amplitudes(amps, 1)
    for gt, b in gl:
        o.apply_gate(gt.matrix(), b)
    want = o.states()[:, 0]
    g = VectorState.from_amplitudes(amps, 1, "c64")
    g.apply_plan(Plan(n, [b for _, b in gl], 5), mats)
    got = g.states()[:, 0]
    assert np.max(np.abs(got - want)) <= TOL64 * scale
    assert abs(np.linalg.norm(got) ** 2 / scale ** 2 - 1.0) <= 2e-6
    infid = 1.0 - abs(np.vdot(want, got)) ** 2 / (np.vdot(want, want).real * np.vdot(got, got).real)
    assert infid <= 1e-9


def test_tensor_core_wait_limit_expires_then_state_recovers():
    """Tensor-core passes whose waits may last at most 1 ns give up: every
    CTA stops, drains the tile copies and MMAs it still has in flight,
    releases its tensor memory and reports the expiry, so the plan fails with
    DeviceTimeout (the error path of a wait that ran out, taken without any
    fault).  With the default limit restored, the same handle, reset, runs the
    plan again and matches the oracle -- the expired passes left no TMEM
    allocated and nothing in flight -- and so does a new state."""
    rng = np.random.default_rng(90)
    n = 16
    gl = [random_gate(n, rng) for _ in range(60)]
    bits = [b for _, b in gl]
    mats = np.concatenate([np.ascontiguousarray(gt.matrix()).ravel() for gt, _ in gl]).view(np.float64)
    plan = Plan(n, bits, 5)
    g = VectorState.from_amplitudes(rand_state(n, rng), 1, "c64")
    g.set_wait_limit(1e-9)
    g.profile(True)
    with pytest.raises(_lib.DeviceTimeout):
        g.apply_plan(plan, mats)
    assert g.profile_report(reset=True)["fused_tc_c64"]["launches"] > 0
    g.profile(False)
    g.set_wait_limit(0)
    o = orc.OracleState.new(n, 1)
    for gt, b in gl:
        o.apply_gate(gt.matrix(), b)
    want = o.states()[:, 0]
    g.reset_all()
    g.apply_plan(plan, mats)
    fresh = VectorState(n, 1, "c64")
    fresh.apply_plan(plan, mats)
    for st in (g, fresh):
        got = st.states()[:, 0]
        assert np.max(np.abs(got - want)) <= TOL64
        assert 1 - abs(np.vdot(want, got)) ** 2 <= 1e-6


@pytest.mark.parametrize("prec,tol", [("c128", 1e-12), ("c64", 2e-6)])
def test_random_normal_state_matches_oracle(prec, tol):
    """fill_random_normal draws re, im i.i.d. N(0,1) on the device from the
    SplitMix64 stream and normalises each column: the oracle's FP64
    restatement of the same draws (complex64 computes the transform in FP32),
    the same seed the same state, another seed another one."""
    n, seed = 12, 2024
    s = VectorState(n, 8, prec)
    s.fill_random_normal(seed)
    got = s.states()
    want = orc.random_normal_state(n, 1, seed)
    assert got.shape == want.shape
    assert np.max(np.abs(got - want)) <= tol
    assert abs(np.linalg.norm(got) - 1.0) <= (1e-12 if prec == "c128" else 1e-6)
    s.fill_random_normal(seed)
    assert np.array_equal(s.states(), got)
    s.fill_random_normal(seed + 1)
    assert np.max(np.abs(s.states() - got)) > 1e-3


def test_random_normal_state_statistics_at_24_qubits():
    """At 24 qubits the drawn state has the Porter-Thomas statistics of a
    random state: N |a|^2 ~ Exp(1), so its mean is 1 and its second moment 2
    (to 6 standard errors), and it equals the oracle's draws."""
    n = 24
    s = VectorState(n, 1, "c64")
    s.fill_random_normal(77)
    a = s.states()[:, 0].astype(np.complex128)
    x = (1 << n) * np.abs(a) ** 2
    se1, se2 = np.sqrt(1.0 / x.size), np.sqrt(20.0 / x.size)
    assert abs(x.mean() - 1.0) <= 6 * se1
    assert abs((x ** 2).mean() - 2.0) <= 6 * se2
    assert np.max(np.abs(a - orc.random_normal_state(n, 1, 77)[:, 0])) <= 2e-6 / 64


def test_compare_reports_normalised_tv():
    rng = np.random.default_rng(2)
    n = 12
    amps = rand_state(n, rng)
    a = VectorState.from_amplitudes(amps, 1, "c128")
    b = VectorState.from_amplitudes(0.5 * amps, 1, "c64")
    r = a.compare(b)
    assert r["tv"] <= 1e-6 and r["infidelity"] <= 1e-12
    assert abs(r["norm_b"] - 0.25) <= 1e-6
