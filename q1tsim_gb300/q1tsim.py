"""The reference's Python binding API (python/q1tsim.py) on the GPU engine.

`from q1tsim_gb300 import q1tsim` gives the module a user of the reference's
cffi binding imports as `q1tsim`: `Circuit(nr_qbits, nr_cbits)` used as a
context manager, gates added by name or through the shortcuts, `RefParam`
parameters changed between executions, `execute(nr_shots)`, `reexecute()`,
`cstate()` and `histogram()` (bit-string keys, classical bit 0 last).  It
runs in the complex128 drop-in mode.

Semantics follow the binding's C entry points (src/ffi.rs): the gate names
and parameter counts of `circuit_add_gate` (src/ffi.rs:308-380), the
measurement bases 'X', 'Y', 'Z' in either case (src/ffi.rs:495-557), and
every failure raised as an exception carrying the message
(python/q1tsimffi.py:85-108).  `latex`, `open_qasm` and `c_qasm` export the
circuit to text formats, which is outside this engine's scope: they raise.
"""
from . import gates as G
from .circuit import Circuit as _Circuit

# gate names and parameter counts accepted by circuit_add_gate (src/ffi.rs:334-358)
_FFI_GATES = {"ch": 0, "crx": 1, "cry": 1, "crz": 1, "cx": 0, "cy": 0, "cz": 0, "h": 0, "i": 0, "rx": 1,
              "ry": 1, "rz": 1, "s": 0, "sdg": 0, "swap": 0, "t": 0, "tdg": 0, "u1": 1, "u2": 2, "u3": 3,
              "v": 0, "vdg": 0, "x": 0, "y": 0, "z": 0}


class RefParam(G.Parameter):
    """A gate parameter passed by reference (python/q1tsim.py:5-38): assign()
    a new value and the next execution of the circuit uses it."""

    def pointer(self):
        """The parameter object itself (the binding hands the engine a
        pointer to the value; here the engine holds the object)."""
        return self


def _gate(name, params):
    key = str(name).lower()
    if key not in _FFI_GATES:
        raise Exception(f"Unknown gate \"{name}\"")
    params = [] if params is None else list(params)
    if len(params) != _FFI_GATES[key]:
        raise Exception(f"Invalid number of arguments for \"{name.upper()}\": expected "
                        f"{_FFI_GATES[key]}, got {len(params)}")
    return G.by_name(key, params)


def _basis(basis):
    b = str(basis)
    if len(b) != 1 or b.lower() not in ("x", "y", "z"):
        raise Exception(f"Invalid measurement basis '{b}'")
    return b.lower()


class Circuit(object):
    """A quantum circuit (python/q1tsim.py:39-529), executed on the GPU."""

    def __init__(self, nr_qbits, nr_cbits=0):
        self._c = _Circuit(nr_qbits, nr_cbits, precision="c128", fusion_width=0)

    def __enter__(self):
        return self

    def __exit__(self, exc_type, exc_value, traceback):
        self._c.q_state = None

    def nr_qbits(self):
        return self._c.nr_qbits

    def nr_cbits(self):
        return self._c.nr_cbits

    def cstate(self):
        """The measurement words of every run (a list of unsigned 64-bit
        integers, one per shot)."""
        if self._c.c_state is None:
            raise Exception("Circuit has not been run yet")
        return [int(w) for w in self._c.cstate()]

    def add_gate(self, name, qbits, params=None):
        self._c.add_gate(_gate(name, params), list(qbits))

    def add_conditional_gate(self, control, target, name, qbits, params=None):
        self._c.add_conditional_gate(list(control), int(target), _gate(name, params), list(qbits))

    # gate shortcuts (python/q1tsim.py:118-306)
    def ch(self, control, target): return self.add_gate('CH', [control, target])
    def crx(self, theta, control, target): return self.add_gate('CRX', [control, target], [theta])
    def cry(self, theta, control, target): return self.add_gate('CRY', [control, target], [theta])
    def crz(self, lmb, control, target): return self.add_gate('CRZ', [control, target], [lmb])
    def cx(self, control, target): return self.add_gate('CX', [control, target])
    def cy(self, control, target): return self.add_gate('CY', [control, target])
    def cz(self, control, target): return self.add_gate('CZ', [control, target])
    def h(self, qbit): return self.add_gate('H', [qbit])
    def i(self, qbit): return self.add_gate('I', [qbit])
    def rx(self, theta, qbit): return self.add_gate('RX', [qbit], [theta])
    def ry(self, theta, qbit): return self.add_gate('RY', [qbit], [theta])
    def rz(self, lmb, qbit): return self.add_gate('RZ', [qbit], [lmb])
    def s(self, qbit): return self.add_gate('S', [qbit])
    def sdg(self, qbit): return self.add_gate('Sdg', [qbit])
    def swap(self, qbit0, qbit1): return self.add_gate('Swap', [qbit0, qbit1])
    def t(self, qbit): return self.add_gate('T', [qbit])
    def tdg(self, qbit): return self.add_gate('Tdg', [qbit])
    def u1(self, lmb, qbit): return self.add_gate('U1', [qbit], [lmb])
    def u2(self, phi, lmb, qbit): return self.add_gate('U2', [qbit], [phi, lmb])
    def u3(self, theta, phi, lmb, qbit): return self.add_gate('U3', [qbit], [theta, phi, lmb])
    def v(self, qbit): return self.add_gate('V', [qbit])
    def vdg(self, qbit): return self.add_gate('Vdg', [qbit])
    def x(self, qbit): return self.add_gate('X', [qbit])
    def y(self, qbit): return self.add_gate('Y', [qbit])
    def z(self, qbit): return self.add_gate('Z', [qbit])

    # measurement (python/q1tsim.py:308-452)
    def measure_basis(self, qbit, cbit, basis):
        self._c.measure_basis(qbit, cbit, _basis(basis))

    def measure_x(self, qbit, cbit): return self.measure_basis(qbit, cbit, 'X')
    def measure_y(self, qbit, cbit): return self.measure_basis(qbit, cbit, 'Y')
    def measure_z(self, qbit, cbit): return self.measure_basis(qbit, cbit, 'Z')
    def measure(self, qbit, cbit): return self.measure_basis(qbit, cbit, 'Z')

    def measure_all_basis(self, cbits, basis):
        self._c.measure_all_basis(list(cbits), _basis(basis))

    def measure_all(self, cbits): return self.measure_all_basis(cbits, 'Z')

    def peek_basis(self, qbit, cbit, basis):
        self._c.peek_basis(qbit, cbit, _basis(basis))

    def peek_x(self, qbit, cbit): return self.peek_basis(qbit, cbit, 'X')
    def peek_y(self, qbit, cbit): return self.peek_basis(qbit, cbit, 'Y')
    def peek_z(self, qbit, cbit): return self.peek_basis(qbit, cbit, 'Z')
    def peek(self, qbit, cbit): return self.peek_basis(qbit, cbit, 'Z')

    def peek_all_basis(self, cbits, basis):
        self._c.peek_all_basis(list(cbits), _basis(basis))

    def peek_all(self, cbits): return self.peek_all_basis(cbits, 'Z')

    def reset(self, qbit):
        self._c.reset(qbit)

    def reset_all(self):
        self._c.reset_all()

    # execution and results (python/q1tsim.py:473-502)
    def execute(self, nr_shots):
        self._c.execute(nr_shots)

    def reexecute(self):
        self._c.reexecute()

    def histogram(self):
        """{bit string: count}; the last character is classical bit 0."""
        if self._c.c_state is None:
            raise Exception("Circuit has not been run yet")
        return self._c.histogram_string()

    def latex(self):
        raise Exception("LaTeX export is not provided by the GPU engine")

    def open_qasm(self):
        raise Exception("OpenQasm export is not provided by the GPU engine")

    def c_qasm(self):
        raise Exception("c-Qasm export is not provided by the GPU engine")
