"""Many independent circuits in one persistent GPU launch.

`Batch` lowers `Circuit` programs of gates, up to four mid-circuit Z
measurements, gates conditioned on one classical bit and a final
`measure_all` into the engine's
batch op list (include/q1gpu.h, q1g_batch_*), then runs them all in one
persistent kernel launch replayed from a CUDA graph.  Each circuit's
classical words equal what `Circuit.execute` with the same `Rng(seed)` gives
(src/circuit.rs:643-762 per circuit).
"""
import ctypes

import numpy as np

from . import _lib
from . import gates as G
from ._lib import check

OP_GATE, OP_MEASURE, OP_CONDITIONAL, OP_MEASURE_ALL = 0, 1, 2, 3

_szp = ctypes.POINTER(ctypes.c_size_t)
_dp = ctypes.POINTER(ctypes.c_double)


def _protos(L):
    if getattr(L, "_batch_protos", False):
        return
    L.q1g_batch_create.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
    L.q1g_batch_create.restype = ctypes.c_int
    L.q1g_batch_free.argtypes = [ctypes.c_void_p]
    L.q1g_batch_free.restype = None
    L.q1g_batch_add_circuit.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_uint64,
                                        ctypes.c_size_t, ctypes.POINTER(ctypes.c_int), _szp, _szp, _dp, _szp]
    L.q1g_batch_add_circuit.restype = ctypes.c_int
    L.q1g_batch_run.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64), ctypes.c_size_t]
    L.q1g_batch_run.restype = ctypes.c_int
    L.q1g_batch_info.argtypes = [ctypes.c_void_p, _szp, _szp, _szp, _szp, _dp]
    L.q1g_batch_info.restype = ctypes.c_int
    L.q1g_batch_traffic.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]
    L.q1g_batch_traffic.restype = ctypes.c_int
    L._batch_protos = True


def lower(circuit):
    """Op arrays of a Circuit for q1g_batch_add_circuit."""
    kinds, nbits, bits, mats, args = [], [], [], [], []
    H = G.H().matrix()
    Sdg, S = G.Sdg().matrix(), G.S().matrix()

    def gate(m, b):
        kinds.append(OP_GATE)
        nbits.append(len(b))
        bits.extend(b)
        mats.append(np.ascontiguousarray(m, dtype=np.complex128).ravel())
        args.extend([0, 0])

    for op in circuit.ops:
        kind = op[0]
        if kind == "gate":
            gate(op[1].matrix(), op[2])
        elif kind == "measure":
            _, q, cbit, basis = op
            if basis == "x":
                gate(H, [q])
            elif basis == "y":
                gate(Sdg, [q])
                gate(H, [q])
            kinds.append(OP_MEASURE)
            nbits.append(0)
            args.extend([q, cbit])
            if basis == "x":
                gate(H, [q])
            elif basis == "y":
                gate(H, [q])
                gate(S, [q])
        elif kind == "cgate":
            _, control, target, g, b = op
            if len(control) != 1:
                raise ValueError("a batched conditional gate tests one classical bit")
            kinds.append(OP_CONDITIONAL)
            nbits.append(len(b))
            bits.extend(b)
            mats.append(np.ascontiguousarray(g.matrix(), dtype=np.complex128).ravel())
            args.extend([control[0], target])
        elif kind == "measure_all":
            _, cbits, basis = op
            for q in range(circuit.nr_qbits):
                if basis == "x":
                    gate(H, [q])
                elif basis == "y":
                    gate(Sdg, [q])
                    gate(H, [q])
            kinds.append(OP_MEASURE_ALL)
            nbits.append(len(cbits))
            bits.extend(cbits)
            args.extend([0, 0])
        elif kind == "barrier":
            continue
        else:
            raise ValueError(f"op {kind!r} is not supported in a batch")
    flat = np.concatenate(mats).view(np.float64) if mats else np.zeros(0)
    return (np.asarray(kinds, dtype=np.int32), np.asarray(nbits, dtype=np.uint64),
            np.asarray(bits, dtype=np.uint64), np.ascontiguousarray(flat), np.asarray(args, dtype=np.uint64))


class Batch:
    def __init__(self, fusion_width=4):
        L = _lib.load()
        _protos(L)
        h = ctypes.c_void_p()
        check(L.q1g_batch_create(int(fusion_width), ctypes.byref(h)), "batch_create")
        self._h = h
        self._shots = []

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib._lib is not None:
            _lib._lib.q1g_batch_free(h)
            self._h = None

    def add(self, circuit, nr_shots, seed):
        """Add a circuit; returns its index."""
        kinds, nbits, bits, mats, args = lower(circuit)
        L = _lib.load()
        check(L.q1g_batch_add_circuit(
            self._h, circuit.nr_qbits, nr_shots, seed & (2**64 - 1), len(kinds),
            kinds.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), nbits.ctypes.data_as(_szp),
            bits.ctypes.data_as(_szp), mats.ctypes.data_as(_dp), args.ctypes.data_as(_szp)), "batch_add")
        self._shots.append(nr_shots)
        return len(self._shots) - 1

    def run(self):
        """Run all circuits; returns one uint64 c_state array per circuit."""
        total = sum(self._shots)
        out = np.zeros(max(total, 1), dtype=np.uint64)
        check(_lib.load().q1g_batch_run(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), len(out)),
              "batch_run")
        res, off = [], 0
        for s in self._shots:
            res.append(out[off:off + s])
            off += s
        return res

    def info(self):
        nc, runs, arena, nops = (ctypes.c_size_t() for _ in range(4))
        ms = ctypes.c_double()
        check(_lib.load().q1g_batch_info(self._h, ctypes.byref(nc), ctypes.byref(runs), ctypes.byref(arena),
                                         ctypes.byref(nops), ctypes.byref(ms)))
        moved = ctypes.c_uint64()
        check(_lib.load().q1g_batch_traffic(self._h, ctypes.byref(moved)))
        return {"circuits": nc.value, "runs": runs.value, "arena_bytes": arena.value, "ops": nops.value,
                "last_ms": ms.value, "traffic_bytes": moved.value}
