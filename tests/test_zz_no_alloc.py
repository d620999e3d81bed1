"""The sampler entry point that allocates nothing (q1g_sample_shots_noalloc).

It is for callers that cannot call cudaMalloc. One is a framework whose pool
allocator owns all device memory. Another is a latency-critical loop that
must not stall on an allocation's synchronisation. The caller passes the
amplitudes, the sorted uniforms and the outputs in device memory; the scratch
is a fixed device array inside the library.

The test calls it through the C ABI twice in a row on device buffers made
with PyTorch, and checks each call's classical words against the existing
entry point, q1g_peek_all_into, on the same column and uniforms. The two
share their kernels, so the words must be identical (integer outputs: exact
equality).  The cases cover a state smaller than one chunk (3 qubits), the
default classical bits (cbits NULL), and the multi-tile prefix scan inside
the fixed scratch (20 qubits and the 24-qubit maximum).  The file is named to
be collected last.
"""
import ctypes

import numpy as np
import pytest

from q1tsim_gb300 import VectorState, _lib

pytestmark = pytest.mark.gpu


def _noalloc(lib, d_amps, prec, n, d_u, nshots, d_out, d_words, cbits, stream):
    """cbits None passes NULL: the default mapping cbits[q] = q."""
    if cbits is None:
        cb_ptr = None
    else:
        cb = np.ascontiguousarray(np.asarray(cbits, dtype=np.uint64))
        cb_ptr = cb.ctypes.data_as(ctypes.POINTER(ctypes.c_size_t))
    rc = lib.q1g_sample_shots_noalloc(
        ctypes.c_void_p(d_amps), prec, n, ctypes.cast(ctypes.c_void_p(d_u), ctypes.POINTER(ctypes.c_double)),
        nshots, ctypes.cast(ctypes.c_void_p(d_out), ctypes.POINTER(ctypes.c_uint64)),
        ctypes.cast(ctypes.c_void_p(d_words), ctypes.POINTER(ctypes.c_uint64)),
        cb_ptr, ctypes.c_void_p(stream))
    _lib.check(rc, "q1g_sample_shots_noalloc")


@pytest.mark.parametrize("n,explicit_cbits", [(3, True), (3, False), (14, True), (14, False), (20, True),
                                              (24, True)])
@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_noalloc_sampler_matches_peek_all(prec, n, explicit_cbits):
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    rng = np.random.default_rng(41 + n)
    shots = 5000
    a = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    a /= np.linalg.norm(a)
    cbits = [int(c) for c in rng.permutation(n)] if explicit_cbits else list(range(n))
    s = VectorState.from_amplitudes(a, shots, prec)
    tdtype = torch.complex128 if prec == "c128" else torch.complex64
    d_amps = torch.tensor(a, dtype=tdtype, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        u = np.sort(rng.random(shots))
        want = np.zeros(shots, dtype=np.uint64)
        s.peek_all_into(cbits, want, uniforms=u)
        d_u = torch.tensor(u, dtype=torch.float64, device="cuda")
        d_out = torch.zeros(shots, dtype=torch.int64, device="cuda")
        d_words = torch.zeros(shots, dtype=torch.int64, device="cuda")
        _noalloc(lib, d_amps.data_ptr(), _lib.C128 if prec == "c128" else _lib.C64, n, d_u.data_ptr(), shots,
                 d_out.data_ptr(), d_words.data_ptr(), cbits if explicit_cbits else None, stream)
        torch.cuda.synchronize()
        got = d_words.cpu().numpy().view(np.uint64)
        assert np.array_equal(got, want), f"call {call}"
        outc = d_out.cpu().numpy().view(np.uint64)
        assert np.all(outc < (1 << n))


def test_noalloc_sampler_rejects_oversized_states():
    lib = _lib.load()
    rc = lib.q1g_sample_shots_noalloc(ctypes.c_void_p(16), _lib.C64, 25, None, 0, None, None, None, None)
    assert rc == _lib.InvalidArgument.code
    assert b"at most 24 qubits" in lib.q1g_last_error()
