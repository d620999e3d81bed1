"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE).

The oracle (oracle.c) restates q1tsim's complex128 VectorState
(src/vectorstate.rs) in plain C.  Only the tests, the smoke check and the
bench's CPU-baseline leg import this module; the engine never does.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None

_u64 = ctypes.c_uint64
_sz = ctypes.c_size_t
_dp = ctypes.POINTER(ctypes.c_double)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_szp = ctypes.POINTER(ctypes.c_size_t)
_u8p = ctypes.POINTER(ctypes.c_uint8)
_vp = ctypes.c_void_p

OK = 0
INVALID_NR_BITS = 1
INVALID_QBIT = 2
INVALID_CBIT = 3
INVALID_NR_CONTROL_BITS = 4
INVALID_NR_MEASUREMENT_BITS = 5
NOT_ENOUGH_SPACE = 6


def build():
    """Compile liboracle.so beside its source (make, gcc)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        L.oracle_uniform.argtypes = [_u64, _u64]
        L.oracle_uniform.restype = ctypes.c_double
        L.oracle_new.argtypes = [_sz, _sz]
        L.oracle_new.restype = _vp
        L.oracle_from_qubit_coefs.argtypes = [_dp, _sz, _sz]
        L.oracle_from_qubit_coefs.restype = _vp
        L.oracle_from_amplitudes.argtypes = [_dp, _sz, _sz]
        L.oracle_from_amplitudes.restype = _vp
        L.oracle_free.argtypes = [_vp]
        L.oracle_free.restype = None
        L.oracle_nr_cols.argtypes = [_vp]
        L.oracle_nr_cols.restype = _sz
        L.oracle_nr_bits.argtypes = [_vp]
        L.oracle_nr_bits.restype = _sz
        L.oracle_is_sparse.argtypes = [_vp]
        L.oracle_is_sparse.restype = ctypes.c_int
        L.oracle_counts.argtypes = [_vp, _u64p]
        L.oracle_counts.restype = None
        L.oracle_get_states.argtypes = [_vp, _dp, _sz]
        L.oracle_get_states.restype = ctypes.c_int
        L.oracle_apply_gate.argtypes = [_vp, _dp, _sz, _szp, _sz]
        L.oracle_apply_gate.restype = ctypes.c_int
        L.oracle_apply_unary_gate_all.argtypes = [_vp, _dp]
        L.oracle_apply_unary_gate_all.restype = ctypes.c_int
        L.oracle_apply_conditional_gate.argtypes = [_vp, _u8p, _sz, _dp, _sz, _szp, _sz]
        L.oracle_apply_conditional_gate.restype = ctypes.c_int
        for name in ("oracle_measure_into", "oracle_peek_into"):
            f = getattr(L, name)
            f.argtypes = [_vp, _sz, _sz, _u64p, _sz, _dp, _sz, _u64p]
            f.restype = ctypes.c_int
        for name in ("oracle_measure_all_into", "oracle_peek_all_into"):
            f = getattr(L, name)
            f.argtypes = [_vp, _szp, _sz, _u64p, _sz, _dp, _sz, _u64p]
            f.restype = ctypes.c_int
        L.oracle_reset.argtypes = [_vp, _sz, _dp, _sz, _u64p]
        L.oracle_reset.restype = ctypes.c_int
        L.oracle_reset_all.argtypes = [_vp]
        L.oracle_reset_all.restype = None
        L.oracle_reverse_bits.argtypes = [_u64, _sz]
        L.oracle_reverse_bits.restype = _u64
        L.oracle_shuffle_bits.argtypes = [_u64, _szp, _sz]
        L.oracle_shuffle_bits.restype = _u64
        L.oracle_binomial_inv.argtypes = [_u64, ctypes.c_double, ctypes.c_double]
        L.oracle_binomial_inv.restype = _u64
        _lib = L
    return _lib


class OracleError(Exception):
    def __init__(self, code, what):
        super().__init__(f"{what}: oracle status {code}")
        self.code = code


def _dptr(a):
    return a.ctypes.data_as(_dp)


def _szarr(bits):
    a = np.ascontiguousarray(np.asarray(bits, dtype=np.uint64))
    return a, a.ctypes.data_as(_szp)


def _mat(m):
    m = np.ascontiguousarray(np.asarray(m, dtype=np.complex128))
    return m.view(np.float64)


class Rng:
    """SplitMix64 counter stream shared by the oracle and the engine."""

    def __init__(self, seed, counter=0):
        self.state = (ctypes.c_uint64 * 2)(seed & (2**64 - 1), counter)

    @property
    def ptr(self):
        return ctypes.cast(self.state, _u64p)


def _rngp(rng):
    """Pointer to (seed, counter) of an oracle Rng or of the engine's Rng."""
    if rng is None:
        return None
    if hasattr(rng, "as_u64_ptr"):
        return rng.as_u64_ptr()
    return rng.ptr


def uniform(seed, counter):
    return lib().oracle_uniform(seed, counter)


def uniforms(seed, counters):
    """Draws `counters` (a uint64 array) of the SplitMix64 stream `seed`,
    vectorised: mix(seed + (k+1) * gamma) >> 11, over 2^53 (the stream of
    oracle.c's oracle_uniform and of the engine's samplers)."""
    with np.errstate(over="ignore"):
        k = np.asarray(counters, dtype=np.uint64)
        z = np.uint64(seed) + (k + np.uint64(1)) * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def random_normal_state(nr_bits, ncols, seed):
    """The state q1g_state_fill_random_normal makes, in FP64: amplitude i of
    column c has re, im = r (cos 2 pi u2, sin 2 pi u2), r = sqrt(-2 ln(1 -
    u1)), with u1, u2 draws 2(cN+i), 2(cN+i)+1 of the stream `seed`; each
    column then has unit norm.  Shape (2^nr_bits, ncols), as states()."""
    n = 1 << nr_bits
    k = np.arange(n * ncols, dtype=np.uint64)
    u1 = uniforms(seed, 2 * k)
    u2 = uniforms(seed, 2 * k + np.uint64(1))
    r = np.sqrt(-2.0 * np.log1p(-u1))
    a = (r * np.cos(2 * np.pi * u2) + 1j * r * np.sin(2 * np.pi * u2)).reshape(ncols, n).T
    return a / np.linalg.norm(a, axis=0)


class OracleState:
    """Complex128 VectorState restatement (src/vectorstate.rs:24-416)."""

    def __init__(self, handle):
        if not handle:
            raise MemoryError("oracle allocation failed")
        self._h = handle

    @classmethod
    def new(cls, nr_bits, nr_shots):
        return cls(lib().oracle_new(nr_bits, nr_shots))

    @classmethod
    def from_qubit_coefs(cls, coefs, nr_shots):
        c = _mat(coefs)
        return cls(lib().oracle_from_qubit_coefs(_dptr(c), len(coefs) // 2, nr_shots))

    @classmethod
    def from_amplitudes(cls, amps, nr_shots):
        a = _mat(amps)
        n = int(np.log2(len(amps)))
        return cls(lib().oracle_from_amplitudes(_dptr(a), n, nr_shots))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oracle_free(self._h)
            self._h = None

    @property
    def nr_bits(self):
        return lib().oracle_nr_bits(self._h)

    @property
    def ncols(self):
        return lib().oracle_nr_cols(self._h)

    @property
    def counts(self):
        out = np.zeros(self.ncols, dtype=np.uint64)
        lib().oracle_counts(self._h, out.ctypes.data_as(_u64p))
        return [int(x) for x in out]

    def states(self):
        """(2^n, ncols) complex128 matrix, like the reference's CMatrix."""
        n = 1 << self.nr_bits
        out = np.zeros(n * self.ncols * 2, dtype=np.float64)
        rc = lib().oracle_get_states(self._h, _dptr(out), out.size)
        self._check(rc, "get_states")
        return out.view(np.complex128).reshape(self.ncols, n).T.copy()

    def is_sparse(self):
        return bool(lib().oracle_is_sparse(self._h))

    @staticmethod
    def _check(rc, what):
        if rc != OK:
            raise OracleError(rc, what)

    def apply_gate(self, mat, bits, k=None):
        m = _mat(mat)
        k = int(np.log2(np.asarray(mat).shape[0])) if k is None else k
        b, bp = _szarr(bits)
        self._check(lib().oracle_apply_gate(self._h, _dptr(m), k, bp, len(bits)), "apply_gate")

    def apply_unary_gate_all(self, mat):
        m = _mat(mat)
        self._check(lib().oracle_apply_unary_gate_all(self._h, _dptr(m)), "apply_unary_gate_all")

    def apply_conditional_gate(self, control, mat, bits, k=None):
        c = np.ascontiguousarray(np.asarray(control, dtype=np.uint8))
        m = _mat(mat)
        k = int(np.log2(np.asarray(mat).shape[0])) if k is None else k
        b, bp = _szarr(bits)
        self._check(lib().oracle_apply_conditional_gate(
            self._h, c.ctypes.data_as(_u8p), len(c), _dptr(m), k, bp, len(bits)),
            "apply_conditional_gate")

    def _uni(self, uniforms):
        if uniforms is None:
            return None, 0, None
        u = np.ascontiguousarray(np.asarray(uniforms, dtype=np.float64))
        return u, len(u), _dptr(u)

    def measure_into(self, qbit, cbit, res, uniforms=None, rng=None):
        u, nu, up = self._uni(uniforms)
        self._check(lib().oracle_measure_into(
            self._h, qbit, cbit, res.ctypes.data_as(_u64p), len(res), up, nu,
            _rngp(rng)), "measure_into")

    def peek_into(self, qbit, cbit, res, uniforms=None, rng=None):
        u, nu, up = self._uni(uniforms)
        self._check(lib().oracle_peek_into(
            self._h, qbit, cbit, res.ctypes.data_as(_u64p), len(res), up, nu,
            _rngp(rng)), "peek_into")

    def measure_all_into(self, cbits, res, uniforms=None, rng=None):
        u, nu, up = self._uni(uniforms)
        b, bp = _szarr(cbits)
        self._check(lib().oracle_measure_all_into(
            self._h, bp, len(cbits), res.ctypes.data_as(_u64p), len(res), up, nu,
            _rngp(rng)), "measure_all_into")

    def peek_all_into(self, cbits, res, uniforms=None, rng=None):
        u, nu, up = self._uni(uniforms)
        b, bp = _szarr(cbits)
        self._check(lib().oracle_peek_all_into(
            self._h, bp, len(cbits), res.ctypes.data_as(_u64p), len(res), up, nu,
            _rngp(rng)), "peek_all_into")

    def measure(self, qbit, uniforms=None, rng=None):
        res = np.zeros(self._nr_shots(), dtype=np.uint64)
        self.measure_into(qbit, 0, res, uniforms, rng)
        return res

    def measure_all(self, uniforms=None, rng=None):
        res = np.zeros(self._nr_shots(), dtype=np.uint64)
        self.measure_all_into(list(range(self.nr_bits)), res, uniforms, rng)
        return res

    def _nr_shots(self):
        return sum(self.counts)

    def reset(self, bit, uniforms=None, rng=None):
        u, nu, up = self._uni(uniforms)
        self._check(lib().oracle_reset(self._h, bit, up, nu, _rngp(rng)), "reset")

    def reset_all(self):
        lib().oracle_reset_all(self._h)


def reverse_bits(idx, nr_bits):
    return int(lib().oracle_reverse_bits(idx, nr_bits))


def shuffle_bits(idx, bits):
    b, bp = _szarr(bits)
    return int(lib().oracle_shuffle_bits(idx, bp, len(bits)))


def binomial_inv(n, p, u):
    return int(lib().oracle_binomial_inv(n, p, u))
