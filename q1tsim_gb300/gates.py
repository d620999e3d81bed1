"""Gate matrices of q1tsim, evaluated on the host in FP64.

Each gate mirrors the reference gate of the same name: `description()`,
`nr_affected_bits()` and `matrix()` (src/gates.rs:154-175).  The engine only
needs the matrix and the bits, exactly as the reference's VectorState path
does through `apply_gate_mat_slice` (src/gates.rs:121-152).  Angles may be
`Parameter`s whose value changes between executions
(src/gates/parameter.rs:23-75); matrices are therefore re-evaluated on every
execute.  Gate trigonometry stays on the host in FP64.
"""
import math

import numpy as np

_HS2 = 1.0 / math.sqrt(2.0)   # COMPLEX_HSQRT2, src/cmatrix.rs:17


class Parameter:
    """A gate angle that can be changed between executions.

    Mirrors `Parameter::Reference` / the Python binding's `RefParam`
    (src/gates/parameter.rs:23-31, python/q1tsim.py:5-38).
    """

    def __init__(self, value):
        self.value = float(value)

    def assign(self, value):
        self.value = float(value)

    def __float__(self):
        return self.value


def _val(p):
    return float(p)


def _polar(r, theta):
    return complex(r * math.cos(theta), r * math.sin(theta))


class Gate:
    """Base class: a unitary on `nr_affected_bits()` qubits."""

    desc = "?"
    nbits = 1

    def description(self):
        return self.desc

    def nr_affected_bits(self):
        return self.nbits

    def matrix(self):
        raise NotImplementedError

    def param_key(self):
        """Current values of the gate's reference parameters (Parameter
        objects); () for a gate whose matrix cannot change."""
        return ()

    def is_diagonal(self):
        """True when the matrix is diagonal for every parameter value."""
        return False

    def is_swap(self):
        """True for the swap of two qubits."""
        return False

    def plan_kind(self):
        """What a gate plan may assume about this gate: 1 always diagonal, 2
        a swap, 0 anything else (q1g_plan_set_gate_kinds)."""
        if self.is_diagonal():
            return 1
        return 2 if self.is_swap() else 0

    def is_stabilizer(self):
        return False

    def __repr__(self):
        return f"{self.description()}"


_SWAP = np.array([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]], dtype=np.complex128)


class _Fixed(Gate):
    def __init__(self, desc, mat, stabilizer=False):
        self.desc = desc
        self._m = np.asarray(mat, dtype=np.complex128)
        self.nbits = int(round(math.log2(self._m.shape[0])))
        self._stab = stabilizer

    def matrix(self):
        return self._m.copy()

    def _shared_matrix(self):
        """The matrix itself, not a copy (read by Circuit._flat only)."""
        return self._m

    def is_diagonal(self):
        return bool(np.count_nonzero(self._m - np.diag(np.diag(self._m))) == 0)

    def is_swap(self):
        return self._m.shape == (4, 4) and bool(np.array_equal(self._m, _SWAP))

    def is_stabilizer(self):
        return self._stab


def H():
    """src/gates/hadamard.rs:89-93"""
    return _Fixed("H", [[_HS2, _HS2], [_HS2, -_HS2]], True)


def X():
    """src/gates/x.rs:79-84"""
    return _Fixed("X", [[0, 1], [1, 0]], True)


def Y():
    """src/gates/y.rs:53-58"""
    return _Fixed("Y", [[0, -1j], [1j, 0]], True)


def Z():
    """src/gates/z.rs:53-58"""
    return _Fixed("Z", [[1, 0], [0, -1]], True)


def I():
    """src/gates/identity.rs:52-55"""
    return _Fixed("I", np.eye(2), True)


def S():
    """src/gates/s.rs:60-66"""
    return _Fixed("S", [[1, 0], [0, 1j]], True)


def Sdg():
    """src/gates/s.rs:186-192"""
    return _Fixed("Sdg", [[1, 0], [0, -1j]], True)


def T():
    """src/gates/t.rs:52-59"""
    return _Fixed("T", [[1, 0], [0, complex(_HS2, _HS2)]])


def Tdg():
    """src/gates/t.rs:153-160"""
    return _Fixed("Tdg", [[1, 0], [0, complex(_HS2, -_HS2)]])


def V():
    """src/gates/v.rs:58-63"""
    return _Fixed("V", [[0.5 + 0.5j, 0.5 - 0.5j], [0.5 - 0.5j, 0.5 + 0.5j]], True)


def Vdg():
    """src/gates/v.rs:157-162"""
    return _Fixed("Vdg", [[0.5 - 0.5j, 0.5 + 0.5j], [0.5 + 0.5j, 0.5 - 0.5j]], True)


def Swap():
    """src/gates/swap.rs:78-88"""
    return _Fixed("Swap", [[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]], True)


class _Param(Gate):
    def __init__(self, desc, fn, params, nbits=1, diagonal=False):
        self.desc = desc
        self._fn = fn
        self.params = list(params)
        self.nbits = nbits
        self._diagonal = diagonal
        self._refs = [p for p in self.params if isinstance(p, Parameter)]

    def matrix(self):
        return np.asarray(self._fn(*[_val(p) for p in self.params]), dtype=np.complex128)

    def param_key(self):
        return tuple(p.value for p in self._refs) if self._refs else ()

    def is_diagonal(self):
        return self._diagonal


def _rx(theta):
    h = 0.5 * theta
    c, si = complex(math.cos(h), 0.0), complex(0.0, math.sin(h))
    return [[c, -si], [-si, c]]


def _ry(theta):
    h = 0.5 * theta
    c, s = math.cos(h), math.sin(h)
    return [[c, -s], [s, c]]


def _rz(lmb):
    p = _polar(1.0, 0.5 * lmb)
    return [[p.conjugate(), 0], [0, p]]


def _u1(lmb):
    return [[1, 0], [0, _polar(1.0, lmb)]]


def _u2(phi, lmb):
    x = _HS2
    return [[complex(x, 0.0), -_polar(x, lmb)], [_polar(x, phi), _polar(x, phi + lmb)]]


def _u3(theta, phi, lmb):
    h = 0.5 * theta
    c, s = math.cos(h), math.sin(h)
    return [[complex(c, 0.0), -_polar(s, lmb)], [_polar(s, phi), _polar(c, phi + lmb)]]


def RX(theta):
    """src/gates/rx.rs:64-70"""
    return _Param("RX", _rx, [theta])


def RY(theta):
    """src/gates/ry.rs:64-70"""
    return _Param("RY", _ry, [theta])


def RZ(lmb):
    """src/gates/rz.rs:65-70"""
    return _Param("RZ", _rz, [lmb], diagonal=True)


def U1(lmb):
    """src/gates/u1.rs:69-75"""
    return _Param("U1", _u1, [lmb], diagonal=True)


def U2(phi, lmb):
    """src/gates/u2.rs:70-79"""
    return _Param("U2", _u2, [phi, lmb])


def U3(theta, phi, lmb):
    """src/gates/u3.rs:74-84"""
    return _Param("U3", _u3, [theta, phi, lmb])


_CONTROLLED_FIXED = {}


class C(Gate):
    """Controlled gate: identity, with `gate` in the bottom-right block
    (src/gates/controlled.rs:62-71); the control is the first bit."""

    def __init__(self, gate, desc=None):
        self.gate = gate
        self.desc = desc if desc is not None else "C" + gate.description()
        self.nbits = 1 + gate.nr_affected_bits()

    def matrix(self):
        gm = self.gate.matrix()
        g = gm.shape[0]
        res = np.eye(2 * g, dtype=np.complex128)
        res[g:, g:] = gm
        return res

    def _shared_matrix(self):
        """For a fixed inner gate, one matrix shared by every instance with
        that inner matrix (a CX per gate of a circuit would otherwise build
        its 4x4 each time); None otherwise.  Read by Circuit._flat only."""
        if not isinstance(self.gate, _Fixed):
            return None
        key = (self.gate._m.shape[0], self.gate._m.tobytes())
        m = _CONTROLLED_FIXED.get(key)
        if m is None:
            m = self.matrix()
            m.setflags(write=False)
            _CONTROLLED_FIXED[key] = m
        return m

    def param_key(self):
        return self.gate.param_key()

    def is_diagonal(self):
        return self.gate.is_diagonal()

    def is_stabilizer(self):
        return self.desc in ("CX", "CY", "CZ")


class Kron(Gate):
    """g0 (x) g1 on the concatenated bits (src/gates/kron.rs:50-62)."""

    def __init__(self, g0, g1):
        self.g0, self.g1 = g0, g1
        self.desc = f"{g0.description()}⊗{g1.description()}"
        self.nbits = g0.nr_affected_bits() + g1.nr_affected_bits()

    def matrix(self):
        return np.kron(self.g0.matrix(), self.g1.matrix())

    def param_key(self):
        return self.g0.param_key() + self.g1.param_key()

    def is_diagonal(self):
        return self.g0.is_diagonal() and self.g1.is_diagonal()


class Loop(Gate):
    """`gate` applied `count` times (src/gates/staticloop.rs:60-92)."""

    def __init__(self, label, count, gate):
        self.gate, self.count = gate, int(count)
        self.desc = f"{label}({gate.description()})"
        self.nbits = gate.nr_affected_bits()

    def matrix(self):
        return np.linalg.matrix_power(self.gate.matrix(), self.count)

    def param_key(self):
        return self.gate.param_key()

    def is_diagonal(self):
        return self.gate.is_diagonal()


class Composite(Gate):
    """A sequence of (gate, bits) on `nr_bits` local qubits, replayed in
    order (src/gates/composite.rs:463-501); the matrix is their product."""

    def __init__(self, name, nr_bits, ops=()):
        self.desc = name
        self.nbits = int(nr_bits)
        self.ops = [(g, list(b)) for g, b in ops]

    def add_gate(self, gate, bits):
        self.ops.append((gate, list(bits)))

    def matrix(self):
        dim = 1 << self.nbits
        m = np.eye(dim, dtype=np.complex128)
        for g, bits in self.ops:
            m = embed(g.matrix(), bits, self.nbits) @ m
        return m

    def param_key(self):
        return tuple(v for g, _ in self.ops for v in g.param_key())

    def is_diagonal(self):
        return all(g.is_diagonal() for g, _ in self.ops)


def embed(mat, bits, nr_bits):
    """Full 2^nr_bits matrix of `mat` acting on `bits` (bit 0 = MSB)."""
    k = len(bits)
    dim = 1 << nr_bits
    full = np.zeros((dim, dim), dtype=np.complex128)
    pos = [nr_bits - 1 - b for b in bits]
    for col in range(dim):
        gin = 0
        for m, p in enumerate(pos):
            gin |= ((col >> p) & 1) << (k - 1 - m)
        base = col
        for p in pos:
            base &= ~(1 << p)
        for gout in range(1 << k):
            row = base
            for m, p in enumerate(pos):
                row |= ((gout >> (k - 1 - m)) & 1) << p
            full[row, col] += mat[gout, gin]
    return full


def _controlled(name, inner):
    return C(inner, desc=name)


def CX():
    """src/gates/cx.rs"""
    return _controlled("CX", X())


def CY():
    """src/gates/cy.rs"""
    return _controlled("CY", Y())


def CZ():
    """src/gates/cz.rs"""
    return _controlled("CZ", Z())


def CH():
    """src/gates/controlled.rs:402-405"""
    return _controlled("CH", H())


def CRX(theta):
    return _controlled("CRX", RX(theta))


def CRY(theta):
    return _controlled("CRY", RY(theta))


def CRZ(lmb):
    return _controlled("CRZ", RZ(lmb))


def CS():
    return _controlled("CS", S())


def CSdg():
    return _controlled("CSdg", Sdg())


def CT():
    return _controlled("CT", T())


def CTdg():
    return _controlled("CTdg", Tdg())


def CU1(lmb):
    """Controlled phase CP(lambda) (src/gates/controlled.rs:454-459)."""
    return _controlled("CU1", U1(lmb))


def CU2(phi, lmb):
    return _controlled("CU2", U2(phi, lmb))


def CU3(theta, phi, lmb):
    return _controlled("CU3", U3(theta, phi, lmb))


def CV():
    return _controlled("CV", V())


def CVdg():
    return _controlled("CVdg", Vdg())


def CCRX(theta):
    return _controlled("CCRX", CRX(theta))


def CCRY(theta):
    return _controlled("CCRY", CRY(theta))


def CCRZ(lmb):
    return _controlled("CCRZ", CRZ(lmb))


def CCX():
    return _controlled("CCX", CX())


def CCZ():
    return _controlled("CCZ", CZ())


# Gate names accepted by Circuit.add_gate(name, ...), as in src/ffi.rs:350-395.
_BY_NAME = {
    "ch": (CH, 0), "crx": (CRX, 1), "cry": (CRY, 1), "crz": (CRZ, 1),
    "cx": (CX, 0), "cy": (CY, 0), "cz": (CZ, 0), "h": (H, 0), "i": (I, 0),
    "rx": (RX, 1), "ry": (RY, 1), "rz": (RZ, 1), "s": (S, 0), "sdg": (Sdg, 0),
    "swap": (Swap, 0), "t": (T, 0), "tdg": (Tdg, 0), "u1": (U1, 1),
    "u2": (U2, 2), "u3": (U3, 3), "v": (V, 0), "vdg": (Vdg, 0), "x": (X, 0),
    "y": (Y, 0), "z": (Z, 0),
    # controlled gates reachable through the Rust API
    "cs": (CS, 0), "csdg": (CSdg, 0), "ct": (CT, 0), "ctdg": (CTdg, 0),
    "cu1": (CU1, 1), "cu2": (CU2, 2), "cu3": (CU3, 3), "cv": (CV, 0),
    "cvdg": (CVdg, 0), "ccrx": (CCRX, 1), "ccry": (CCRY, 1), "ccrz": (CCRZ, 1),
    "ccx": (CCX, 0), "ccz": (CCZ, 0),
}


class UnknownGate(ValueError):
    pass


class InvalidNrArguments(ValueError):
    pass


def by_name(name, params=None):
    """Construct a gate from its name (case-insensitive) and parameters."""
    key = name.lower()
    if key not in _BY_NAME:
        raise UnknownGate(f"Unknown gate \"{name}\"")
    ctor, nparams = _BY_NAME[key]
    params = list(params or [])
    if len(params) != nparams:
        raise InvalidNrArguments(
            f"Invalid number of arguments for \"{name}\": expected {nparams}, got {len(params)}")
    return ctor(*params)
