"""Pins the CPU oracle to the reference's own known-answer and statistical
tests (CPU only, no GPU)."""
import numpy as np
import pytest

from oracle import oracle as orc
from refcheck import KAT_TOL, dec, get_bounds, kats, measurement_ok

K = kats()


def build_oracle(init):
    if init["kind"] == "new":
        return orc.OracleState.new(init["nr_bits"], init["nr_shots"])
    return orc.OracleState.from_qubit_coefs(dec(init["coefs"]), init["nr_shots"])


def run_ops(s, ops):
    for op in ops:
        if op["op"] == "gate":
            s.apply_gate(dec(op["mat"]), op["bits"])
        elif op["op"] == "cond":
            s.apply_conditional_gate(op["control"], dec(op["mat"]), op["bits"])
        elif op["op"] == "reset_all":
            s.reset_all()


@pytest.mark.parametrize("case", K["vectorstate"], ids=lambda c: c["name"])
def test_vectorstate_kat(case):
    s = build_oracle(case["init"])
    run_ops(s, case["ops"])
    assert s.counts == case["expect"]["counts"]
    np.testing.assert_allclose(s.states(), dec(case["expect"]["states"]), rtol=0, atol=KAT_TOL)


@pytest.mark.parametrize("case", K["apply"], ids=lambda c: c["gate"] + "@" + c["source"])
def test_gate_apply_kat(case):
    state = dec(case["state"])
    expect = dec(case["expect"])
    mat = dec(case["mat"])
    for c in range(state.shape[1]):
        s = orc.OracleState.from_amplitudes(state[:, c], 1)
        s.apply_gate(mat, case["bits"])
        np.testing.assert_allclose(s.states()[:, 0], expect[:, c], rtol=0, atol=KAT_TOL)


def test_support_bits():
    for idx, n, want in K["bits"]["reverse_bits"]:
        assert orc.reverse_bits(idx, n) == want
    for idx, bits, want in K["bits"]["shuffle_bits"]:
        assert orc.shuffle_bits(idx, bits) == want


def test_stats_bounds():
    """src/stats.rs:38-58 (the acceptance rule the statistical tests use)."""
    for n, p, tol, lo, hi in K["stats"]["bounds"]:
        assert get_bounds(n, p, tol) == (lo, hi)
    assert measurement_ok(512, 1024, 0.5, 1e-5)
    assert measurement_ok(444, 1024, 0.5, 1e-5)
    assert not measurement_ok(443, 1024, 0.5, 1e-5)
    assert measurement_ok(580, 1024, 0.5, 1e-5)
    assert not measurement_ok(581, 1024, 0.5, 1e-5)


def test_measure_deterministic():
    """src/vectorstate.rs:519-531"""
    rng = orc.Rng(1)
    s = orc.OracleState.new(1, 3)
    assert list(s.measure(0, rng=rng)) == [0, 0, 0]
    s = orc.OracleState.from_qubit_coefs([1, 0, 1, 0], 3)
    assert list(s.measure(1, rng=rng)) == [0, 0, 0]
    np.testing.assert_allclose(s.states()[:, 0], [1, 0, 0, 0], atol=KAT_TOL)
    assert list(s.measure(0, rng=rng)) == [0, 0, 0]


def test_measure_splits_columns():
    """src/vectorstate.rs:533-590: columns follow the measured bits."""
    x = 1 / np.sqrt(2)
    rng = orc.Rng(7)
    s = orc.OracleState.from_qubit_coefs([1, 1, 1, 1], 1024)
    m0 = s.measure(0, rng=rng)
    st = s.states()
    sc = 0
    for j, b in enumerate(m0):
        if j > 0 and b != m0[j - 1]:
            sc += 1
        want = [x, x, 0, 0] if b == 0 else [0, 0, x, x]
        np.testing.assert_allclose(st[:, sc], want, atol=KAT_TOL)
    assert measurement_ok(int(m0.sum()), 1024, 0.5)
    m0b = s.measure(0, rng=rng)
    assert np.array_equal(m0b, m0)
    m1 = s.measure(1, rng=rng)
    st = s.states()
    sc = 0
    for j in range(1024):
        if j > 0 and (m0[j] != m0[j - 1] or m1[j] != m1[j - 1]):
            sc += 1
        want = np.zeros(4)
        want[2 * int(m0[j]) + int(m1[j])] = 1
        np.testing.assert_allclose(st[:, sc], want, atol=KAT_TOL)


def test_peek_into_statistics():
    """src/vectorstate.rs:593-638"""
    x = 1 / np.sqrt(2)
    n = 1024
    rng = orc.Rng(3)
    res = np.zeros(n, dtype=np.uint64)
    s = orc.OracleState.new(1, n)
    s.peek_into(0, 0, res, rng=rng)
    assert res.sum() == 0
    s = orc.OracleState.from_qubit_coefs([1, 1], n)
    s.peek_into(0, 0, res, rng=rng)
    assert measurement_ok(int(res.sum()), n, 0.5)
    np.testing.assert_allclose(s.states()[:, 0], [x, x], atol=KAT_TOL)
    s = orc.OracleState.from_qubit_coefs([x, x, 0, 1], n)
    res[:] = 0
    s.peek_into(1, 0, res, rng=rng)
    assert int(res.sum()) == n
    np.testing.assert_allclose(s.states()[:, 0], [0, x, 0, x], atol=KAT_TOL)


def test_measure_all_deterministic():
    """src/vectorstate.rs:710-735"""
    rng = orc.Rng(5)
    s = orc.OracleState.from_qubit_coefs([0, 1, 0, 1, 0, 1], 5)
    assert all(int(b) == 0b111 for b in s.measure_all(rng=rng))
    s = orc.OracleState.from_qubit_coefs([0, 1, 0, 1, 1, 0], 5)
    assert all(int(b) == 0b011 for b in s.measure_all(rng=rng))
    s = orc.OracleState.new(3, 5)
    s.apply_gate(np.array([[1, 1], [1, -1]]) / np.sqrt(2), [2])
    assert all((int(b) & 0b011) == 0 for b in s.measure_all(rng=rng))


def test_peek_all_statistics():
    """src/vectorstate.rs:738-771"""
    H = np.array([[1, 1], [1, -1]]) / np.sqrt(2)
    n = 1024
    s = orc.OracleState.from_qubit_coefs([0, 1, 0, 1, 0, 1], n)
    s.apply_gate(H, [0])
    s.apply_gate(H, [2])
    res = np.zeros(n, dtype=np.uint64)
    s.peek_all_into([0, 1, 2], res, rng=orc.Rng(11))
    assert s.counts == [n]
    np.testing.assert_allclose(s.states()[:, 0], [0, 0, .5, -.5, 0, 0, -.5, .5], atol=KAT_TOL)
    cnt = [int(((res >> np.uint64(b)) & np.uint64(1)).sum()) for b in range(3)]
    assert measurement_ok(cnt[0], n, 0.5) and cnt[1] == n and measurement_ok(cnt[2], n, 0.5)


def test_reset():
    """src/vectorstate.rs:774-811"""
    x = 1 / np.sqrt(2)
    rng = orc.Rng(2)
    for coefs, bit, want in [([1, 0], 0, [1, 0]), ([0, 1], 0, [1, 0]), ([0, 1, 0, 1], 0, [0, 1, 0, 0]),
                             ([0, 1, 0, 1], 1, [0, 0, 1, 0]), ([x, -x, 1, 0], 1, [x, 0, -x, 0])]:
        s = orc.OracleState.from_qubit_coefs(coefs, 10)
        s.reset(bit, rng=rng)
        np.testing.assert_allclose(s.states()[:, 0], want, atol=KAT_TOL)
    s = orc.OracleState.from_qubit_coefs([x, -x, 1, 0], 10)
    s.reset(0, rng=rng)
    st = s.states()
    if st.shape[1] == 1:
        np.testing.assert_allclose(st[:, 0], [1, 0, 0, 0], atol=KAT_TOL)
    else:
        np.testing.assert_allclose(st, [[1, -1], [0, 0], [0, 0], [0, 0]], atol=KAT_TOL)


def test_binomial_inverse_matches_distribution():
    """The n0 draw: inverse CDF of Binomial(n, p); its mean and variance."""
    rng = np.random.default_rng(0)
    for n, p in [(1024, 0.5), (1000, 0.03), (50, 0.9), (1_000_000, 0.43)]:
        us = rng.random(400)
        draws = np.array([orc.binomial_inv(n, p, u) for u in us])
        assert abs(draws.mean() - n * p) < 5 * np.sqrt(n * p * (1 - p) / len(us)) + 1
    assert orc.binomial_inv(10, 0.0, 0.5) == 0
    assert orc.binomial_inv(10, 1.0, 0.5) == 10
    assert orc.binomial_inv(0, 0.3, 0.5) == 0


def test_sorted_uniform_stream_is_uniform():
    """Exponential-spacing order statistics from the shared SplitMix64 stream."""
    s = orc.OracleState.new(1, 20000)
    s.apply_gate(np.array([[1, 1], [1, -1]]) / np.sqrt(2), [0])
    res = np.zeros(20000, dtype=np.uint64)
    rng = orc.Rng(99)
    s.peek_all_into([0], res, rng=rng)
    assert rng.state[1] == 20001
    assert measurement_ok(int(res.sum()), 20000, 0.5)
    # outcomes come out grouped in ascending order within the column
    assert np.all(np.diff(res.astype(np.int64)) >= 0)


def test_errors_match_reference():
    s = orc.OracleState.new(2, 4)
    with pytest.raises(orc.OracleError) as e:
        s.apply_gate(np.eye(2), [0, 1])
    assert e.value.code == orc.INVALID_NR_BITS
    with pytest.raises(orc.OracleError) as e:
        s.measure_into(2, 0, np.zeros(4, dtype=np.uint64), rng=orc.Rng(0))
    assert e.value.code == orc.INVALID_QBIT
    with pytest.raises(orc.OracleError) as e:
        s.measure_into(0, 0, np.zeros(3, dtype=np.uint64), rng=orc.Rng(0))
    assert e.value.code == orc.NOT_ENOUGH_SPACE
    with pytest.raises(orc.OracleError) as e:
        s.measure_all_into([0], np.zeros(4, dtype=np.uint64), rng=orc.Rng(0))
    assert e.value.code == orc.INVALID_NR_MEASUREMENT_BITS
    with pytest.raises(orc.OracleError) as e:
        s.apply_conditional_gate([1, 0], np.eye(2), [0])
    assert e.value.code == orc.INVALID_NR_CONTROL_BITS
