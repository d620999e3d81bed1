"""The C-ABI library: builds, loads and exports every declared symbol; the
host-only parts of the ABI (plans and the fusion pass) work without a GPU.
No kernel is launched here."""
import ctypes
import itertools

import numpy as np
import pytest

from q1tsim_gb300 import _lib, build
from q1tsim_gb300 import gates as G
from q1tsim_gb300.vectorstate import Plan


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def test_exports_every_declared_symbol(lib):
    declared = _lib.declared_symbols()
    assert len(declared) >= 29
    for name in declared:
        assert hasattr(lib, name), name


def test_version_and_last_error(lib):
    assert lib.q1g_version() >= 100
    assert lib.q1g_last_error() is not None


def test_null_arguments_are_errors_not_crashes(lib):
    assert lib.q1g_state_new(3, 1, 0, None) == _lib.InvalidArgument.code
    assert b"NULL" in lib.q1g_last_error()
    h = ctypes.c_void_p()
    assert lib.q1g_state_new(3, 1, 7, ctypes.byref(h)) == _lib.InvalidArgument.code
    assert lib.q1g_plan_create(4, 1, None, None, 0, ctypes.byref(h)) == _lib.InvalidArgument.code
    with pytest.raises(_lib.InvalidQBit) as ei:
        Plan(3, [[0, 5]])
    assert ei.value.payload == (5,)        # Error::InvalidQBit(5)
    a0, a1 = ctypes.c_uint64(9), ctypes.c_uint64(9)
    lib.q1g_last_error_args(ctypes.byref(a0), ctypes.byref(a1))
    assert (a0.value, a1.value) == (5, 0)
    with pytest.raises(_lib.InvalidArgument) as ei:
        Plan(3, [[0]], fusion_width=7)
    assert ei.value.payload == ()
    p = Plan(3, [[0]], fusion_width=2)
    p.set_tc_tiling(0, 8, 4)
    assert p.tc_tiling == (0, 8, 4)
    for bad in ((2, 13, 2), (2, 5, 0), (2, -1, 2), (6, 5, 2), (-1, 5, 2)):
        with pytest.raises(_lib.InvalidArgument):
            p.set_tc_tiling(*bad)


def _commutes_ok(gate_bits, blocks):
    """Every gate appears once, and two gates sharing a qubit keep their
    relative order in the flattened block sequence."""
    flat = [g for _, gs in blocks for g in gs]
    assert sorted(flat) == list(range(len(gate_bits)))
    pos = {g: i for i, g in enumerate(flat)}
    for a, b in itertools.combinations(range(len(gate_bits)), 2):
        if set(gate_bits[a]) & set(gate_bits[b]):
            assert pos[a] < pos[b], (a, b)
    for qb, gs in blocks:
        assert set(q for g in gs for q in gate_bits[g]) <= set(qb)


def brick(n, depth):
    bits = []
    for layer in range(depth):
        bits += [[q] for q in range(n)]
        start = 0 if layer % 2 == 0 else 1
        bits += [[q, q + 1] for q in range(start, n - 1, 2)]
    return bits


@pytest.mark.parametrize("width", [1, 2, 3, 4, 5])
def test_fusion_respects_order_and_width(lib, width):
    rng = np.random.default_rng(width)
    for n in (4, 9, 16):
        gb = brick(n, 6)
        for _ in range(40):
            k = int(rng.integers(1, 4))
            gb.append([int(q) for q in rng.choice(n, size=k, replace=False)])
        p = Plan(n, gb, fusion_width=width)
        blocks = p.blocks()
        _commutes_ok(gb, blocks)
        for qb, gs in blocks:
            assert len(qb) <= max(width, max(len(gb[g]) for g in gs))
        assert p.nblocks < len(gb)


def test_fusion_product_equals_sequence(lib):
    """The fused blocks, multiplied out on the host, give the same unitary as
    the gate sequence (numpy, 6 qubits)."""
    n = 6
    rng = np.random.default_rng(3)
    gates = []
    for _ in range(60):
        if rng.random() < 0.6:
            q = int(rng.integers(n))
            gates.append((G.U3(*rng.uniform(0, 6.28, 3)), [q]))
        else:
            a, b = (int(v) for v in rng.choice(n, 2, replace=False))
            gates.append((G.CX(), [a, b]))
    seq = np.eye(1 << n, dtype=complex)
    for g, b in gates:
        seq = G.embed(g.matrix(), b, n) @ seq
    p = Plan(n, [b for _, b in gates], fusion_width=4)
    fused = np.eye(1 << n, dtype=complex)
    for qb, gs in p.blocks():
        blk = np.eye(1 << len(qb), dtype=complex)
        for gi in gs:
            g, b = gates[gi]
            local = [qb.index(q) for q in b]
            blk = G.embed(g.matrix(), local, len(qb)) @ blk
        fused = G.embed(blk, qb, n) @ fused
    np.testing.assert_allclose(fused, seq, atol=1e-12)
    assert p.nblocks < len(gates) // 2


@pytest.mark.parametrize("width", [3, 5])
def test_block_matrix_is_the_product_of_its_gates(lib, width):
    """The engine's own fused matrix of every block (q1g_plan_block_matrix)
    equals the numpy product of the block's gates, with 1-, 2- and 3-qubit
    gates, controls and bits in any order."""
    n = 9
    rng = np.random.default_rng(11 + width)
    gates = []
    for _ in range(80):
        r = rng.random()
        if r < 0.45:
            gates.append((G.U3(*rng.uniform(0, 6.28, 3)), [int(rng.integers(n))]))
        elif r < 0.8:
            a, b = (int(v) for v in rng.choice(n, 2, replace=False))
            gates.append((G.Kron(G.U3(*rng.uniform(0, 6.28, 3)), G.RY(rng.uniform(0, 6.28))), [a, b]))
        else:
            bits = [int(v) for v in rng.choice(n, 3, replace=False)]
            gates.append((G.CCX() if r < 0.9 else G.CU3(*rng.uniform(0, 6.28, 3)), bits[:3] if r < 0.9 else bits[:2]))
    mats = np.concatenate([np.ascontiguousarray(g.matrix()).ravel() for g, _ in gates]).view(np.float64)
    p = Plan(n, [b for _, b in gates], fusion_width=width)
    for i, (qb, gs) in enumerate(p.blocks()):
        blk = np.eye(1 << len(qb), dtype=complex)
        for gi in gs:
            g, b = gates[gi]
            blk = G.embed(g.matrix(), [qb.index(q) for q in b], len(qb)) @ blk
        np.testing.assert_allclose(p.block_matrix(i, mats), blk, atol=1e-13)


def test_plain_plan_is_one_pass_per_gate(lib):
    gb = brick(8, 3)
    p = Plan(8, gb, fusion_width=0)
    assert p.nblocks == len(gb)
    assert [gs for _, gs in p.blocks()] == [[i] for i in range(len(gb))]


def _qft_structure(n):
    from q1tsim_gb300 import workloads
    q = workloads.qft(n, precision="c64", fusion_width=5, measure=False)
    seq = [op for op in q.ops if op[0] == "gate"]
    return [op[2] for op in seq], [op[1].is_diagonal() for op in seq]


@pytest.mark.parametrize("n", [6, 12, 28])
def test_phase_runs_group_the_qft_ladders(lib, n):
    """With the diagonal gates marked, each QFT ladder of controlled phases
    (all sharing the target qubit) becomes one phase-run pass together with
    the next Hadamard; every gate appears once, in order."""
    bits, diag = _qft_structure(n)
    plan = Plan(n, bits, 5, diagonal=diag)
    blocks = plan.blocks()
    order = [g for _, gates in blocks for g in gates]
    assert sorted(order) == list(range(len(bits)))
    runs = [(qb, gates) for qb, gates in blocks if len(gates) >= 4 and len(qb) > 5]
    assert len(runs) >= n - 6
    for qb, gates in runs:
        ladder = [g for g in gates if diag[g]]
        assert len(ladder) >= 3
        common = set(bits[ladder[0]])
        for g in ladder:
            common &= set(bits[g])
        assert common   # one qubit shared by the whole ladder
        # the absorbed gate is the non-diagonal 1-qubit gate right after the ladder
        tail = [g for g in gates if not diag[g]]
        assert tail == [] or (tail == [gates[-1]] and len(bits[tail[0]]) == 1 and tail[0] == ladder[-1] + 1)
    assert plan.nblocks < Plan(n, bits, 5).nblocks or n < 8


def test_phase_runs_need_a_common_qubit(lib):
    """A run of diagonal two-qubit gates without a common qubit (a ring of
    controlled phases) stays with the ordinary fusion."""
    n = 8
    bits = [[q, (q + 1) % n] for q in range(n)]
    diag = [True] * n
    plain = Plan(n, bits, 5).blocks()
    marked = Plan(n, bits, 5, diagonal=diag).blocks()
    assert marked == plain


def test_plan_set_gate_kinds_checks_its_arguments(lib):
    plan = Plan(4, [[0], [1, 2]], 3)
    flags = (ctypes.c_ubyte * 1)(1)
    assert lib.q1g_plan_set_gate_kinds(plan.handle, flags, 1) != 0    # one kind for two gates
    assert lib.q1g_plan_set_gate_kinds(None, flags, 1) != 0


def test_swap_runs_group_the_qft_reversal(lib):
    """The QFT's closing swaps (disjoint pairs) become one swap-run pass."""
    from q1tsim_gb300 import workloads
    n = 16
    q = workloads.qft(n, precision="c64", fusion_width=5, measure=False)
    seq = [op for op in q.ops if op[0] == "gate"]
    bits = [op[2] for op in seq]
    kinds = [op[1].plan_kind() for op in seq]
    blocks = Plan(n, bits, 5, kinds=kinds).blocks()
    last = blocks[-1]
    assert [seq[g][1].description() for g in last[1]] == ["Swap"] * (n // 2)
    assert sorted(last[0]) == list(range(n))
    order = [g for _, gates in blocks for g in gates]
    assert sorted(order) == list(range(len(bits)))


def test_plan_gate_kinds_are_checked(lib):
    plan = Plan(4, [[0], [1, 2]], 3)
    kinds = (ctypes.c_ubyte * 2)(2, 0)   # a swap on one qubit
    assert lib.q1g_plan_set_gate_kinds(plan.handle, kinds, 2) != 0
    kinds = (ctypes.c_ubyte * 2)(0, 7)
    assert lib.q1g_plan_set_gate_kinds(plan.handle, kinds, 2) != 0
    kinds = (ctypes.c_ubyte * 2)(1, 2)
    assert lib.q1g_plan_set_gate_kinds(plan.handle, kinds, 2) == 0


def test_window_fusion_on_the_brick_circuit(lib):
    """The 30-qubit brick circuit of the bench (depth 24): window fusion
    takes at most 62 blocks of <= 5 qubits (the greedy fusion alone took 80),
    and the plan's blocks, reordered so that tensor-core-pairable blocks are
    adjacent, still keep every gate once and every dependency in order."""
    n = 30
    gb = brick(n, 24)
    p = Plan(n, gb, fusion_width=5)
    assert p.nblocks <= 62
    blocks = p.blocks()
    for qb, _ in blocks:
        assert len(qb) <= 5
    # dependencies through the flattened order (a sampled check of pairs)
    flat = [g for _, gs in blocks for g in gs]
    assert sorted(flat) == list(range(len(gb)))
    pos = {g: i for i, g in enumerate(flat)}
    last = {}
    for g, bits in enumerate(gb):
        for q in bits:
            if q in last:
                assert pos[last[q]] < pos[g], (last[q], g)
            last[q] = g


def test_reordered_blocks_apply_the_sequence(lib):
    """A 13-qubit random circuit with wide gates (up to 7 qubits) fused to
    5-qubit blocks and reordered: applying the blocks' products to a random
    state equals applying the gates one by one (numpy)."""
    n = 13
    rng = np.random.default_rng(12)
    gates = []
    for _ in range(140):
        r = rng.random()
        if r < 0.5:
            gates.append((G.U3(*rng.uniform(0, 6.28, 3)).matrix(), [int(rng.integers(n))]))
        elif r < 0.95:
            a, b = (int(v) for v in rng.choice(n, 2, replace=False))
            gates.append((np.kron(G.H().matrix(), G.RY(rng.uniform(0, 6)).matrix()) @ G.CX().matrix(), [a, b]))
        else:
            k = int(rng.integers(6, 8))
            bits = [int(v) for v in rng.choice(n, k, replace=False)]
            q, _ = np.linalg.qr(rng.normal(size=(1 << k, 1 << k)) + 1j * rng.normal(size=(1 << k, 1 << k)))
            gates.append((q, bits))
    def apply(psi, m, bits):
        # qubit q is tensor axis q (qubit 0 the most significant index bit)
        k = len(bits)
        t = np.tensordot(m.reshape([2] * (2 * k)), psi.reshape([2] * n), axes=(list(range(k, 2 * k)), bits))
        return np.moveaxis(t, list(range(k)), bits).reshape(-1)
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    seq = psi.copy()
    for m, b in gates:
        seq = apply(seq, m, b)
    p = Plan(n, [b for _, b in gates], fusion_width=5)
    _commutes_ok([b for _, b in gates], p.blocks())
    out = psi.copy()
    for qb, gs in p.blocks():
        for gi in gs:
            m, b = gates[gi]
            out = apply(out, m, b)
    assert np.max(np.abs(out - seq)) <= 1e-9
