"""ctypes binding of libq1gpu.so (the engine's C ABI, include/q1gpu.h).

The library is built in-tree (q1tsim_gb300/build.py).  There is no CPU
fallback: if the shared library is missing or cannot be loaded, importing
the engine raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libq1gpu.so")
HEADER = os.path.join(HERE, "..", "include", "q1gpu.h")

C128 = 0
C64 = 1

_sz = ctypes.c_size_t
_szp = ctypes.POINTER(ctypes.c_size_t)
_dp = ctypes.POINTER(ctypes.c_double)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_u8p = ctypes.POINTER(ctypes.c_uint8)
_vp = ctypes.c_void_p
_int = ctypes.c_int


class q1g_rng(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_uint64), ("counter", ctypes.c_uint64)]


_rngp = ctypes.POINTER(q1g_rng)


# ---------------------------------------------------------------- errors
# Status codes 1..7 mirror crate::error::Error (src/error.rs:135-152).

class Q1Error(Exception):
    """payload: the reference error variant's values, e.g. (q,) for
    InvalidQBit(q) or (len, runs) for NotEnoughSpace(len, runs)."""
    code = -1
    payload = ()

    def __init__(self, msg, code=None, payload=()):
        super().__init__(msg)
        if code is not None:
            self.code = code
        self.payload = tuple(payload)


class InvalidNrBits(Q1Error):
    code = 1


class InvalidQBit(Q1Error):
    code = 2


class InvalidCBit(Q1Error):
    code = 3


class InvalidNrControlBits(Q1Error):
    code = 4


class InvalidNrMeasurementBits(Q1Error):
    code = 5


class NotEnoughSpace(Q1Error):
    code = 6


class NotExecuted(Q1Error):
    code = 7


class InvalidArgument(Q1Error):
    code = 8


class OutOfMemory(Q1Error):
    code = 9


class DeviceError(Q1Error):
    code = 10


class DeviceTimeout(Q1Error):
    code = 11


_BY_CODE = {c.code: c for c in (InvalidNrBits, InvalidQBit, InvalidCBit, InvalidNrControlBits,
                                 InvalidNrMeasurementBits, NotEnoughSpace, NotExecuted,
                                 InvalidArgument, OutOfMemory, DeviceError, DeviceTimeout)}

_lib = None


def _proto(L, name, res, args):
    f = getattr(L, name)
    f.restype = res
    f.argtypes = args


def load():
    """Load libq1gpu.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is missing: build the CUDA engine first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    L = ctypes.CDLL(LIB_PATH)
    _proto(L, "q1g_last_error", ctypes.c_char_p, [])
    _proto(L, "q1g_last_error_args", None, [_u64p, _u64p])
    _proto(L, "q1g_version", _int, [])
    _proto(L, "q1g_device_info", _int, [ctypes.POINTER(_int), _szp, _szp])
    _proto(L, "q1g_state_new", _int, [_sz, _sz, _int, ctypes.POINTER(_vp)])
    _proto(L, "q1g_state_from_qubit_coefs", _int, [_dp, _sz, _sz, _int, ctypes.POINTER(_vp)])
    _proto(L, "q1g_state_from_amplitudes", _int, [_dp, _sz, _sz, _int, ctypes.POINTER(_vp)])
    _proto(L, "q1g_state_free", None, [_vp])
    _proto(L, "q1g_state_set_stream", _int, [_vp, _vp])
    _proto(L, "q1g_state_set_fp64_exact", _int, [_vp, _int])
    _proto(L, "q1g_state_synchronize", _int, [_vp])
    _proto(L, "q1g_state_info", _int, [_vp, _szp, _szp, _szp, ctypes.POINTER(_int)])
    _proto(L, "q1g_state_counts", _int, [_vp, _u64p, _sz])
    _proto(L, "q1g_state_download", _int, [_vp, _dp, _sz])
    _proto(L, "q1g_state_compare", _int, [_vp, _vp, _dp])
    _proto(L, "q1g_apply_gate", _int, [_vp, _dp, _sz, _szp, _sz])
    _proto(L, "q1g_apply_unary_gate_all", _int, [_vp, _dp])
    _proto(L, "q1g_apply_conditional_gate", _int, [_vp, _u8p, _sz, _dp, _sz, _szp, _sz])
    for n in ("q1g_measure_into", "q1g_peek_into"):
        _proto(L, n, _int, [_vp, _sz, _sz, _u64p, _sz, _dp, _sz, _rngp])
    for n in ("q1g_measure_all_into", "q1g_peek_all_into"):
        _proto(L, n, _int, [_vp, _szp, _sz, _u64p, _sz, _dp, _sz, _rngp])
    _proto(L, "q1g_reset", _int, [_vp, _sz, _dp, _sz, _rngp])
    _proto(L, "q1g_reset_all", _int, [_vp])
    _proto(L, "q1g_plan_create", _int, [_sz, _sz, _szp, _szp, _int, ctypes.POINTER(_vp)])
    _proto(L, "q1g_plan_free", None, [_vp])
    _proto(L, "q1g_plan_info", _int, [_vp, _szp, _szp])
    _proto(L, "q1g_plan_block", _int, [_vp, _sz, _szp, _szp, _szp, _szp])
    _proto(L, "q1g_plan_block_matrix", _int, [_vp, _sz, _dp, _sz, _dp, _szp])
    _proto(L, "q1g_plan_run", _int, [_vp, _vp, _dp, _sz])
    _proto(L, "q1g_plan_set_tensor_cores", _int, [_vp, _int])
    _proto(L, "q1g_plan_set_tc_tiling", _int, [_vp, _int, _int, _int])
    _proto(L, "q1g_plan_set_gate_kinds", _int, [_vp, ctypes.POINTER(ctypes.c_ubyte), _sz])
    _proto(L, "q1g_profile_enable", _int, [_vp, _int])
    _proto(L, "q1g_profile_report", _int, [_vp, ctypes.c_char_p, _u64p, _dp, _dp, _szp])
    _proto(L, "q1g_profile_reset", _int, [_vp])
    _proto(L, "q1g_state_transfer_bytes", _int, [_vp, _u64p, _u64p, _int])
    _proto(L, "q1g_state_set_wait_limit", _int, [_vp, ctypes.c_double])
    _proto(L, "q1g_state_fill_random_normal", _int, [_vp, ctypes.c_uint64])
    _proto(L, "q1g_state_column_norms", _int, [_vp, _dp, _sz])
    _proto(L, "q1g_state_device_amplitudes", _int, [_vp, ctypes.POINTER(_vp), _szp])
    _proto(L, "q1g_state_amplitudes_written", _int, [_vp])
    _proto(L, "q1g_sample_shots_noalloc", _int, [_vp, _int, _sz, _dp, _sz, _u64p, _u64p, _szp, _vp])
    _proto(L, "q1g_histogram", _int, [_u64p, _sz, _u64p, _u64p, _sz, _szp, _vp])
    _lib = L
    return L


# how many payload values each variant carries (src/error.rs:135-152)
_PAYLOAD_LEN = {1: 2, 2: 1, 3: 1, 4: 2, 5: 2, 6: 2}


def check(rc, what=""):
    if rc != 0:
        L = load()
        msg = L.q1g_last_error().decode("utf-8", "replace")
        a0, a1 = ctypes.c_uint64(0), ctypes.c_uint64(0)
        L.q1g_last_error_args(ctypes.byref(a0), ctypes.byref(a1))
        payload = (int(a0.value), int(a1.value))[:_PAYLOAD_LEN.get(rc, 0)]
        cls = _BY_CODE.get(rc, Q1Error)
        raise cls(f"{what}: {msg}" if what else msg, rc, payload)


def declared_symbols(header=HEADER):
    """Function names declared in include/q1gpu.h."""
    import re
    txt = open(header).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(q1g_\w+)\s*\(", txt)))
