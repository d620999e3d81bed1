"""The device histogram of classical words (q1g_histogram), which
Circuit.histogram uses from 2^16 runs on (src/circuit.rs:773-789): the same
counts as numpy's unique, in ascending order, for words that repeat, for all
distinct words, for 0 and the all-ones word (the table's empty mark), and for
an empty array; too small an output array is an error."""
import ctypes

import numpy as np
import pytest

from q1tsim_gb300 import Rng, _lib, workloads
from q1tsim_gb300.vectorstate import device_histogram

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,distinct", [(1, 1), (1000, 7), (1 << 17, 300), (1 << 17, 1 << 40), (1 << 20, 1 << 62)])
def test_histogram_matches_unique(n, distinct):
    rng = np.random.default_rng(n + 3)
    words = rng.integers(0, distinct, size=n, dtype=np.uint64)
    words[::97] = np.uint64(0xFFFFFFFFFFFFFFFF)
    words[::89] = 0
    keys, counts = device_histogram(words)
    want_k, want_c = np.unique(words, return_counts=True)
    assert np.array_equal(keys, want_k) and np.array_equal(counts, want_c.astype(np.uint64))
    assert int(counts.sum()) == n


def test_histogram_of_nothing_and_capacity():
    keys, counts = device_histogram(np.zeros(0, dtype=np.uint64))
    assert len(keys) == 0 and len(counts) == 0
    words = np.arange(10, dtype=np.uint64)
    k = np.empty(4, dtype=np.uint64)
    c = np.empty(4, dtype=np.uint64)
    nk = ctypes.c_size_t(0)
    u64 = ctypes.POINTER(ctypes.c_uint64)
    rc = _lib.load().q1g_histogram(words.ctypes.data_as(u64), 10, k.ctypes.data_as(u64), c.ctypes.data_as(u64), 4,
                                   ctypes.byref(nk), None)
    assert rc == 6 and nk.value == 10     # Q1G_ERR_NOT_ENOUGH_SPACE, with the size needed


def test_circuit_histogram_on_the_device():
    """A 20-qubit GHZ state over 2^17 runs: two words, about half each."""
    n, shots = 20, 1 << 17
    c = workloads.ghz(n, precision="c64", fusion_width=5, measure=True)
    c.execute(shots, Rng(7))
    h = c.histogram()
    assert set(h) == {0, (1 << n) - 1} and sum(h.values()) == shots
    keys, cnt = np.unique(c.cstate(), return_counts=True)
    assert h == dict(zip(keys.tolist(), cnt.tolist()))
