"""Device-resident VectorState: q1tsim's `QuState` methods over the C ABI.

`VectorState` mirrors the reference's coefficient-vector backend
(src/vectorstate.rs:24-416, trait src/qustate.rs:5-89) method for method;
every call goes through libq1gpu.so and runs as CUDA kernels on the GPU.
Sampling methods take an `Rng` (SplitMix64 stream) in place of
`rng: &mut R`, or explicit uniforms.
"""
import ctypes
import os

import numpy as np

from . import _lib
from ._lib import check

_PREC = {"c128": _lib.C128, "complex128": _lib.C128, _lib.C128: _lib.C128,
         "c64": _lib.C64, "complex64": _lib.C64, _lib.C64: _lib.C64}


def precision_code(p):
    try:
        return _PREC[p]
    except KeyError:
        raise ValueError(f"unknown precision {p!r}: use 'c128' or 'c64'") from None


class Rng:
    """SplitMix64 counter stream (seed, counter) shared with the engine.

    Stands in for the `rng: &mut R` argument of the QuState methods; the
    engine advances `counter` as it draws.
    """

    def __init__(self, seed=None, counter=0):
        if seed is None:
            seed = int.from_bytes(os.urandom(8), "little")
        self.struct = _lib.q1g_rng(seed & (2**64 - 1), counter)

    @property
    def seed(self):
        return self.struct.seed

    @property
    def counter(self):
        return self.struct.counter

    def ptr(self):
        return ctypes.pointer(self.struct)

    def as_u64_ptr(self):
        return ctypes.cast(ctypes.pointer(self.struct), ctypes.POINTER(ctypes.c_uint64))


def _mat(gate):
    m = gate.matrix() if hasattr(gate, "matrix") else gate
    m = np.ascontiguousarray(np.asarray(m, dtype=np.complex128))
    return m


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _sizes(bits):
    a = np.ascontiguousarray(np.asarray(list(bits), dtype=np.uint64))
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_size_t))


def _nr_affected(gate, m):
    if hasattr(gate, "nr_affected_bits"):
        return gate.nr_affected_bits()
    return int(round(np.log2(m.shape[0])))


class VectorState:
    """q1tsim VectorState on the GPU (src/vectorstate.rs:24-416)."""

    def __init__(self, nr_bits, nr_shots, precision="c128", _handle=None):
        L = _lib.load()
        self._prec = precision_code(precision)
        if _handle is None:
            h = ctypes.c_void_p()
            check(L.q1g_state_new(nr_bits, nr_shots, self._prec, ctypes.byref(h)), "VectorState::new")
            _handle = h
        self._h = _handle
        self._nr_bits = nr_bits
        self._nr_shots = nr_shots

    @classmethod
    def from_qubit_coefs(cls, coefs, nr_shots, precision="c128"):
        """src/vectorstate.rs:62-83; coefs = [c0_q0, c1_q0, c0_q1, ...]."""
        L = _lib.load()
        c = np.ascontiguousarray(np.asarray(coefs, dtype=np.complex128)).view(np.float64)
        if len(coefs) % 2:
            raise ValueError("Length of coefficient array is not even")
        n = len(coefs) // 2
        h = ctypes.c_void_p()
        check(L.q1g_state_from_qubit_coefs(_dptr(c), n, nr_shots, precision_code(precision),
                                           ctypes.byref(h)), "from_qubit_coefs")
        return cls(n, nr_shots, precision, _handle=h)

    @classmethod
    def from_amplitudes(cls, amps, nr_shots, precision="c128"):
        """Arbitrary initial state of 2^n complex amplitudes (no reference
        counterpart: the reference API builds only product states)."""
        L = _lib.load()
        a = np.ascontiguousarray(np.asarray(amps, dtype=np.complex128)).view(np.float64)
        n = int(round(np.log2(len(amps))))
        if 1 << n != len(amps):
            raise ValueError("amplitude count must be a power of two")
        h = ctypes.c_void_p()
        check(L.q1g_state_from_amplitudes(_dptr(a), n, nr_shots, precision_code(precision),
                                          ctypes.byref(h)), "from_amplitudes")
        return cls(n, nr_shots, precision, _handle=h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib._lib is not None:
            _lib._lib.q1g_state_free(h)
            self._h = None

    # ---- introspection
    def nr_bits(self):
        return self._nr_bits

    @property
    def nr_shots(self):
        return self._nr_shots

    @property
    def precision(self):
        return "c128" if self._prec == _lib.C128 else "c64"

    @property
    def handle(self):
        return self._h

    @property
    def ncols(self):
        nc = ctypes.c_size_t()
        check(_lib.load().q1g_state_info(self._h, None, None, ctypes.byref(nc), None))
        return nc.value

    @property
    def counts(self):
        out = np.zeros(self.ncols, dtype=np.uint64)
        check(_lib.load().q1g_state_counts(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                           len(out)))
        return [int(x) for x in out]

    def states(self):
        """The state as a (2^n, ncols) complex128 matrix, like the CMatrix."""
        n = 1 << self._nr_bits
        nc = self.ncols
        out = np.zeros(2 * n * nc, dtype=np.float64)
        check(_lib.load().q1g_state_download(self._h, _dptr(out), out.size), "download")
        return out.view(np.complex128).reshape(nc, n).T.copy()

    def compare(self, other):
        """Accuracy of `other` against this state, computed on the device:
        {max_abs_diff, infidelity, tv, norm_a, norm_b}."""
        out = np.zeros(5, dtype=np.float64)
        check(_lib.load().q1g_state_compare(self._h, other._h, _dptr(out)), "compare")
        return {"max_abs_diff": float(out[0]), "infidelity": float(out[1]), "tv": float(out[2]),
                "norm_a": float(out[3]), "norm_b": float(out[4])}

    def set_fp64_exact(self, exact=True):
        """complex128: FP64 arithmetic (the reference's rounding) instead of
        the default double-float pairs (within the 1e-12 contract)."""
        check(_lib.load().q1g_state_set_fp64_exact(self._h, 1 if exact else 0))

    def set_stream(self, stream):
        """Run on a caller-owned cudaStream_t (an int handle), None = own."""
        check(_lib.load().q1g_state_set_stream(self._h, ctypes.c_void_p(stream) if stream else None))

    def synchronize(self):
        check(_lib.load().q1g_state_synchronize(self._h))

    # ---- QuState methods (src/qustate.rs:5-89)
    def apply_gate(self, gate, bits):
        m = _mat(gate)
        k = _nr_affected(gate, m)
        b, bp = _sizes(bits)
        check(_lib.load().q1g_apply_gate(self._h, _dptr(m.view(np.float64)), k, bp, len(b)), "apply_gate")

    def apply_unary_gate_all(self, gate):
        m = _mat(gate)
        check(_lib.load().q1g_apply_unary_gate_all(self._h, _dptr(m.view(np.float64))), "apply_unary_gate_all")

    def apply_conditional_gate(self, control, gate, bits):
        c = np.ascontiguousarray(np.asarray(control, dtype=np.uint8))
        m = _mat(gate)
        k = _nr_affected(gate, m)
        b, bp = _sizes(bits)
        check(_lib.load().q1g_apply_conditional_gate(
            self._h, c.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), len(c),
            _dptr(m.view(np.float64)), k, bp, len(b)), "apply_conditional_gate")

    @staticmethod
    def _uni(uniforms):
        if uniforms is None:
            return None, None, 0
        u = np.ascontiguousarray(np.asarray(uniforms, dtype=np.float64))
        return u, _dptr(u), len(u)

    @staticmethod
    def _rng(rng):
        return rng.ptr() if rng is not None else None

    @staticmethod
    def _res(res):
        if res.dtype != np.uint64 or not res.flags["C_CONTIGUOUS"]:
            raise TypeError("res must be a contiguous uint64 array")
        return res.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))

    def measure_into(self, qbit, cbit, res, rng=None, uniforms=None):
        u, up, nu = self._uni(uniforms)
        check(_lib.load().q1g_measure_into(self._h, qbit, cbit, self._res(res), len(res), up, nu,
                                           self._rng(rng)), "measure_into")

    def peek_into(self, qbit, cbit, res, rng=None, uniforms=None):
        u, up, nu = self._uni(uniforms)
        check(_lib.load().q1g_peek_into(self._h, qbit, cbit, self._res(res), len(res), up, nu,
                                        self._rng(rng)), "peek_into")

    def measure_all_into(self, cbits, res, rng=None, uniforms=None):
        u, up, nu = self._uni(uniforms)
        b, bp = _sizes(cbits)
        check(_lib.load().q1g_measure_all_into(self._h, bp, len(b), self._res(res), len(res), up, nu,
                                               self._rng(rng)), "measure_all_into")

    def peek_all_into(self, cbits, res, rng=None, uniforms=None):
        u, up, nu = self._uni(uniforms)
        b, bp = _sizes(cbits)
        check(_lib.load().q1g_peek_all_into(self._h, bp, len(b), self._res(res), len(res), up, nu,
                                            self._rng(rng)), "peek_all_into")

    def measure(self, qbit, rng=None, uniforms=None):
        res = np.zeros(self._nr_shots, dtype=np.uint64)
        self.measure_into(qbit, 0, res, rng, uniforms)
        return res

    def measure_all(self, rng=None, uniforms=None):
        res = np.zeros(self._nr_shots, dtype=np.uint64)
        self.measure_all_into(list(range(self._nr_bits)), res, rng, uniforms)
        return res

    def reset(self, bit, rng=None, uniforms=None):
        u, up, nu = self._uni(uniforms)
        check(_lib.load().q1g_reset(self._h, bit, up, nu, self._rng(rng)), "reset")

    def reset_all(self):
        check(_lib.load().q1g_reset_all(self._h), "reset_all")

    # ---- gate sequences
    def apply_plan(self, plan, mats_flat):
        m = np.ascontiguousarray(mats_flat, dtype=np.float64)
        check(_lib.load().q1g_plan_run(plan.handle, self._h, _dptr(m), m.size), "plan_run")

    # ---- profiling
    def profile(self, enable=True):
        check(_lib.load().q1g_profile_enable(self._h, 1 if enable else 0))

    def profile_report(self, reset=False):
        L = _lib.load()
        cap = 64
        names = ctypes.create_string_buffer(32 * cap)
        launches = np.zeros(cap, dtype=np.uint64)
        ms = np.zeros(cap, dtype=np.float64)
        by = np.zeros(cap, dtype=np.float64)
        n = ctypes.c_size_t(cap)
        check(L.q1g_profile_report(self._h, names, launches.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                   _dptr(ms), _dptr(by), ctypes.byref(n)))
        out = {}
        raw = names.raw
        for i in range(n.value):
            nm = raw[32 * i:32 * i + 32].split(b"\0", 1)[0].decode()
            out[nm] = {"launches": int(launches[i]), "ms": float(ms[i]), "bytes": float(by[i])}
        if reset:
            check(L.q1g_profile_reset(self._h))
        return out

    def fill_random_normal(self, seed):
        """Every column a random unit vector drawn on the device (re, im
        i.i.d. N(0,1) from the SplitMix64 stream `seed`, then normalised)."""
        check(_lib.load().q1g_state_fill_random_normal(self._h, int(seed) & (2 ** 64 - 1)))

    def set_wait_limit(self, seconds=0.0):
        """Longest wait inside a tensor-core pass before the pass gives up
        with DeviceTimeout (amplitudes then undefined); 0 = default (60 s)."""
        check(_lib.load().q1g_state_set_wait_limit(self._h, float(seconds)))

    def transfer_bytes(self, reset=False):
        """(host->device, device->host) bytes copied by this state's calls
        since it was made or last reset."""
        h2d, d2h = ctypes.c_uint64(0), ctypes.c_uint64(0)
        check(_lib.load().q1g_state_transfer_bytes(self._h, ctypes.byref(h2d), ctypes.byref(d2h),
                                                   1 if reset else 0))
        return int(h2d.value), int(d2h.value)


class Plan:
    """A gate sequence lowered once: structure, fusion grouping, passes."""

    KIND_GENERAL, KIND_DIAGONAL, KIND_SWAP = 0, 1, 2
    # (pairs of blocks per pass: 0 none, 1 through the staged tile, 2 through
    # registers; tile positions at >= 2 MB strides a pair may have;
    # bank-conflict slack of an unpadded tile)
    DEFAULT_TC_TILING = (4, 8, 4)

    def __init__(self, nr_bits, gate_bits, fusion_width=0, tensor_cores=True, diagonal=None, kinds=None):
        """kinds: per gate, KIND_DIAGONAL for gates whose matrix is always
        diagonal (phases, controlled phases) and KIND_SWAP for swaps; runs of
        them then become single phase or permutation passes
        (q1g_plan_set_gate_kinds).  diagonal: per gate, True for diagonal
        gates (the same as kinds with only KIND_DIAGONAL)."""
        L = _lib.load()
        ks = np.asarray([len(b) for b in gate_bits], dtype=np.uint64)
        flat = np.asarray([q for b in gate_bits for q in b], dtype=np.uint64)
        h = ctypes.c_void_p()
        check(L.q1g_plan_create(nr_bits, len(ks), ks.ctypes.data_as(ctypes.POINTER(ctypes.c_size_t)),
                                flat.ctypes.data_as(ctypes.POINTER(ctypes.c_size_t)), int(fusion_width),
                                ctypes.byref(h)), "plan_create")
        self._h = h
        self.nr_bits = nr_bits
        self.fusion_width = fusion_width
        self.ngates = len(ks)
        self.tensor_cores = bool(tensor_cores)
        check(L.q1g_plan_set_tensor_cores(h, 1 if tensor_cores else 0), "plan_set_tensor_cores")
        self.tc_tiling = self.DEFAULT_TC_TILING
        if kinds is None and diagonal is not None:
            kinds = [self.KIND_DIAGONAL if d else self.KIND_GENERAL for d in diagonal]
        if kinds is not None and any(kinds):
            flags = np.asarray(kinds, dtype=np.uint8)
            check(L.q1g_plan_set_gate_kinds(h, flags.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)), len(flags)),
                  "plan_set_gate_kinds")

    @property
    def handle(self):
        return self._h

    def set_tc_tiling(self, allow_pairs=4, max_high_positions=8, conflict_slack=4):
        """Tiling of the tensor-core passes (q1g_plan_set_tc_tiling)."""
        check(_lib.load().q1g_plan_set_tc_tiling(self.handle, int(allow_pairs), int(max_high_positions),
                                                 int(conflict_slack)), "plan_set_tc_tiling")
        self.tc_tiling = (int(allow_pairs), int(max_high_positions), int(conflict_slack))

    @property
    def nblocks(self):
        nb = ctypes.c_size_t()
        check(_lib.load().q1g_plan_info(self._h, None, ctypes.byref(nb)))
        return nb.value

    def block_matrix(self, i, mats_flat):
        """The fused matrix of block i for these gate matrices (host only)."""
        L = _lib.load()
        mats = np.ascontiguousarray(mats_flat, dtype=np.float64)
        out = np.zeros(2 * 32 * 32, dtype=np.float64)
        n = ctypes.c_size_t(out.size)
        check(L.q1g_plan_block_matrix(self._h, i, _dptr(mats), mats.size, _dptr(out), ctypes.byref(n)),
              "plan_block_matrix")
        dim = int(round((n.value // 2) ** 0.5))
        return out[:n.value].view(np.complex128).reshape(dim, dim)

    def blocks(self):
        """[(qubits, gate indices)] of every pass, in launch order."""
        L = _lib.load()
        out = []
        for i in range(self.nblocks):
            qb = np.zeros(64, dtype=np.uint64)
            gb = np.zeros(max(self.ngates, 1), dtype=np.uint64)
            nq = ctypes.c_size_t(len(qb))
            ng = ctypes.c_size_t(len(gb))
            check(L.q1g_plan_block(self._h, i, qb.ctypes.data_as(ctypes.POINTER(ctypes.c_size_t)), ctypes.byref(nq),
                                   gb.ctypes.data_as(ctypes.POINTER(ctypes.c_size_t)), ctypes.byref(ng)))
            out.append(([int(q) for q in qb[:nq.value]], [int(g) for g in gb[:ng.value]]))
        return out

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib._lib is not None:
            _lib._lib.q1g_plan_free(h)
            self._h = None


def device_info():
    L = _lib.load()
    sm = ctypes.c_int()
    free = ctypes.c_size_t()
    total = ctypes.c_size_t()
    check(L.q1g_device_info(ctypes.byref(sm), ctypes.byref(free), ctypes.byref(total)))
    return {"sm_count": sm.value, "free_bytes": free.value, "total_bytes": total.value}


def device_histogram(words, stream=None, sort=True):
    """Distinct values of a uint64 array and their counts, counted on the
    GPU (q1g_histogram): the classical-word histogram of a circuit with many
    runs.  Ascending with sort, else in the device table's order."""
    w = np.ascontiguousarray(words, dtype=np.uint64)
    n = len(w)
    keys = np.empty(max(n, 1), dtype=np.uint64)
    counts = np.empty(max(n, 1), dtype=np.uint64)
    nk = ctypes.c_size_t(0)
    u64 = ctypes.POINTER(ctypes.c_uint64)
    check(_lib.load().q1g_histogram(w.ctypes.data_as(u64), n, keys.ctypes.data_as(u64), counts.ctypes.data_as(u64),
                                    len(keys), ctypes.byref(nk), stream), "histogram")
    keys, counts = keys[:nk.value], counts[:nk.value]
    if sort and len(keys) > 1:
        order = np.argsort(keys)     # distinct keys: any sort order is the same
        keys, counts = keys[order], counts[order]
    return keys, counts
