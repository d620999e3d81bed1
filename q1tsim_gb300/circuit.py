"""Circuit: q1tsim's circuit API executing on the GPU VectorState.

Mirrors `Circuit` (src/circuit.rs:97-1282) and the Python binding
(python/q1tsim.py): gates are added by object or by name, then `execute`
runs the op list (src/circuit.rs:643-762) on a device-resident state and
`histogram*` count the classical results (src/circuit.rs:773-841).

Runs of consecutive gates are lowered to one `Plan` per run: in the plain
complex128 mode (fusion_width 0) each gate is its own pass, exactly as
`apply_gate` would run it; with fusion_width k (complex64 fused mode) the
plan groups gates into blocks of at most k qubits.  Matrices are evaluated
again on every execute, since gate parameters may change between runs
(src/gates/parameter.rs:23-75).
"""
import numpy as np

from . import gates as G
from ._lib import InvalidCBit, InvalidQBit, NotExecuted
from .vectorstate import Plan, Rng, VectorState

BASES = ("x", "y", "z")


class Circuit:
    def __init__(self, nr_qbits, nr_cbits=0, precision="c128", fusion_width=0):
        """fusion_width: qubits per fused block (0 = one pass per gate, the
        plain drop-in mode) or "auto" to let the autotuner choose the width
        and the dense-block kernel on the first execution."""
        self.nr_qbits = int(nr_qbits)
        self.nr_cbits = int(nr_cbits)
        self.precision = precision
        self.fusion_width = fusion_width if fusion_width == "auto" else int(fusion_width)
        self.ops = []
        self.q_state = None
        self.c_state = None
        self.rng = None
        self._plans = {}
        self._frozen = None
        self._segs = None
        self._flats = {}    # segment index -> (gates with reference parameters, their values, matrices)

    # ------------------------------------------------------------ building
    def _check_qbits(self, qbits):
        for b in qbits:
            if b >= self.nr_qbits or b < 0:
                raise InvalidQBit(f"Invalid index {b} for a quantum bit")

    def _check_cbits(self, cbits):
        for b in cbits:
            if b >= self.nr_cbits or b < 0:
                raise InvalidCBit(f"Invalid index {b} for a classical bit")

    def _push(self, op):
        self.ops.append(op)
        self._plans.clear()
        self._frozen = None
        self._segs = None
        self._flats = {}

    def freeze(self):
        """Evaluate every gate matrix now and reuse them on later executions
        (a request handed to a server arrives with its matrices evaluated).
        Parameters changed afterwards take effect only after unfreeze()."""
        self._frozen = {}
        for idx, op in enumerate(self._segments()):
            if op[0] == "seq":
                self._frozen[idx] = self._flat(op[1])
        return self

    def unfreeze(self):
        self._frozen = None

    @staticmethod
    def _flat(seq):
        """The segment's gate matrices, concatenated row-major as (re, im)
        doubles.  Fixed gates contribute their stored matrices; U3 gates (most
        of a random circuit) are evaluated together with numpy, with the
        formulas of gates._u3 (src/gates/u3.rs:74-84).  A server builds these
        for every request, under the interpreter lock."""
        n = len(seq)
        if n == 0:
            return np.zeros(0)
        sizes = np.empty(n, dtype=np.int64)
        parts = [None] * n
        u3_rows, u3_par, cu1_rows, cu1_par = [], [], [], []
        for i, op in enumerate(seq):
            g = op[1]
            sizes[i] = 1 << (2 * g.nr_affected_bits())
            tg = type(g)
            if tg is G._Param and g._fn is G._u3:
                u3_rows.append(i)
                u3_par.append([float(p) for p in g.params])
                continue
            if tg is G.C and type(g.gate) is G._Param and g.gate._fn is G._u1:
                cu1_rows.append(i)
                cu1_par.append(float(g.gate.params[0]))
                continue
            shared = getattr(g, "_shared_matrix", None)
            m = shared() if shared is not None else None
            parts[i] = m if m is not None else np.asarray(g.matrix(), dtype=np.complex128)
        offs = np.zeros(n + 1, dtype=np.int64)
        np.cumsum(sizes, out=offs[1:])
        out = np.empty(int(offs[-1]), dtype=np.complex128)
        for i, m in enumerate(parts):
            if m is not None:
                out[offs[i]:offs[i + 1]] = m.ravel()
        if u3_rows:
            p = np.asarray(u3_par)
            theta, phi, lmb = p[:, 0], p[:, 1], p[:, 2]
            c, s = np.cos(0.5 * theta), np.sin(0.5 * theta)
            pl = phi + lmb
            m = np.empty((len(u3_rows), 4), dtype=np.complex128)
            m.real[:, 0], m.imag[:, 0] = c, 0.0
            m.real[:, 1], m.imag[:, 1] = -(s * np.cos(lmb)), -(s * np.sin(lmb))
            m.real[:, 2], m.imag[:, 2] = s * np.cos(phi), s * np.sin(phi)
            m.real[:, 3], m.imag[:, 3] = c * np.cos(pl), c * np.sin(pl)
            out[offs[np.asarray(u3_rows)][:, None] + np.arange(4)] = m
        if cu1_rows:
            # C(U1(lmb)) = diag(1, 1, 1, e^(i lmb)) (src/gates/u1.rs:69-84)
            lmb = np.asarray(cu1_par)
            m = np.zeros((len(cu1_rows), 16), dtype=np.complex128)
            m[:, 0] = m[:, 5] = m[:, 10] = 1.0
            m.real[:, 15], m.imag[:, 15] = np.cos(lmb), np.sin(lmb)
            out[offs[np.asarray(cu1_rows)][:, None] + np.arange(16)] = m
        return out.view(np.float64)

    def _flat_current(self, idx, seq):
        """The segment's matrices for this execution.  They are evaluated
        again only when a reference parameter of one of its gates has changed
        (src/gates/parameter.rs:23-75); gates with plain values keep theirs."""
        ent = self._flats.get(idx)
        if ent is not None:
            dyn, key, flat = ent
            now = tuple(v for i in dyn for v in seq[i][1].param_key())
            if now == key:
                return flat
        dyn = [i for i, op in enumerate(seq) if op[1].param_key()]
        flat = self._flat(seq)
        self._flats[idx] = (dyn, tuple(v for i in dyn for v in seq[i][1].param_key()), flat)
        return flat

    @staticmethod
    def _gate(gate, params):
        if isinstance(gate, str):
            return G.by_name(gate, params)
        return gate

    def add_gate(self, gate, qbits, params=None):
        """src/circuit.rs:161-175 (object) / python/q1tsim.py add_gate (name)."""
        g = self._gate(gate, params)
        qbits = list(qbits)
        self._check_qbits(qbits)
        self._push(("gate", g, qbits))

    def add_conditional_gate(self, control, target, gate, qbits, params=None):
        """src/circuit.rs:182-204: apply when the classical bits `control`
        (first = least significant) form the word `target`."""
        g = self._gate(gate, params)
        control, qbits = list(control), list(qbits)
        self._check_cbits(control)
        self._check_qbits(qbits)
        self._push(("cgate", control, int(target), g, qbits))

    def measure_basis(self, qbit, cbit, basis):
        self._check_qbits([qbit])
        self._check_cbits([cbit])
        self._push(("measure", qbit, cbit, basis.lower()))

    def measure(self, qbit, cbit, basis="z"):
        self.measure_basis(qbit, cbit, basis)

    def measure_x(self, qbit, cbit):
        self.measure_basis(qbit, cbit, "x")

    def measure_y(self, qbit, cbit):
        self.measure_basis(qbit, cbit, "y")

    def measure_z(self, qbit, cbit):
        self.measure_basis(qbit, cbit, "z")

    def measure_all_basis(self, cbits, basis):
        cbits = list(cbits)
        self._check_cbits(cbits)
        self._push(("measure_all", cbits, basis.lower()))

    def measure_all(self, cbits=None, basis="z"):
        if cbits is None:
            cbits = list(range(self.nr_qbits))
        self.measure_all_basis(cbits, basis)

    def peek_basis(self, qbit, cbit, basis):
        self._check_qbits([qbit])
        self._check_cbits([cbit])
        self._push(("peek", qbit, cbit, basis.lower()))

    def peek(self, qbit, cbit, basis="z"):
        self.peek_basis(qbit, cbit, basis)

    def peek_all_basis(self, cbits, basis):
        cbits = list(cbits)
        self._check_cbits(cbits)
        self._push(("peek_all", cbits, basis.lower()))

    def peek_all(self, cbits=None, basis="z"):
        if cbits is None:
            cbits = list(range(self.nr_qbits))
        self.peek_all_basis(cbits, basis)

    def reset(self, qbit):
        self._check_qbits([qbit])
        self._push(("reset", qbit))

    def reset_all(self):
        self._push(("reset_all",))

    def barrier(self, qbits):
        self._check_qbits(list(qbits))
        self._push(("barrier", list(qbits)))

    # gate shortcuts of src/circuit.rs:430-541 and python/q1tsim.py
    def h(self, q): self.add_gate(G.H(), [q])
    def x(self, q): self.add_gate(G.X(), [q])
    def y(self, q): self.add_gate(G.Y(), [q])
    def z(self, q): self.add_gate(G.Z(), [q])
    def s(self, q): self.add_gate(G.S(), [q])
    def sdg(self, q): self.add_gate(G.Sdg(), [q])
    def t(self, q): self.add_gate(G.T(), [q])
    def tdg(self, q): self.add_gate(G.Tdg(), [q])
    def v(self, q): self.add_gate(G.V(), [q])
    def vdg(self, q): self.add_gate(G.Vdg(), [q])
    def i(self, q): self.add_gate(G.I(), [q])
    def rx(self, theta, q): self.add_gate(G.RX(theta), [q])
    def ry(self, theta, q): self.add_gate(G.RY(theta), [q])
    def rz(self, lmb, q): self.add_gate(G.RZ(lmb), [q])
    def u1(self, lmb, q): self.add_gate(G.U1(lmb), [q])
    def u2(self, phi, lmb, q): self.add_gate(G.U2(phi, lmb), [q])
    def u3(self, theta, phi, lmb, q): self.add_gate(G.U3(theta, phi, lmb), [q])
    def cx(self, c, t): self.add_gate(G.CX(), [c, t])
    def cy(self, c, t): self.add_gate(G.CY(), [c, t])
    def cz(self, c, t): self.add_gate(G.CZ(), [c, t])
    def ch(self, c, t): self.add_gate(G.CH(), [c, t])
    def crx(self, theta, c, t): self.add_gate(G.CRX(theta), [c, t])
    def cry(self, theta, c, t): self.add_gate(G.CRY(theta), [c, t])
    def crz(self, lmb, c, t): self.add_gate(G.CRZ(lmb), [c, t])
    def swap(self, a, b): self.add_gate(G.Swap(), [a, b])

    def is_stabilizer_circuit(self):
        return all(op[0] != "gate" or op[1].is_stabilizer() for op in self.ops) and \
            all(op[0] != "cgate" or op[3].is_stabilizer() for op in self.ops)

    # ----------------------------------------------------------- execution
    def new_state(self, nr_shots):
        return VectorState(self.nr_qbits, nr_shots, self.precision)

    def execute(self, nr_shots, rng=None):
        """Run the circuit from |0...0> over nr_shots runs on the GPU vector
        backend (src/circuit.rs:562-585; the stabilizer choice of the
        reference is not made here: every circuit runs on the vector state,
        as execute_with(QuStateRepr::vector(..)) does)."""
        if isinstance(self.q_state, VectorState) and self.q_state.nr_shots == nr_shots \
                and self.q_state.precision == self.precision:
            self.q_state.reset_all()
            q_state = self.q_state
        else:
            q_state = self.new_state(nr_shots)
        self.execute_with(nr_shots, rng if rng is not None else Rng(), q_state)

    def execute_with(self, nr_shots, rng, q_state):
        """src/circuit.rs:594-600"""
        self.q_state = q_state
        self.c_state = np.zeros(nr_shots, dtype=np.uint64)
        self.rng = rng
        self.reexecute_with_rng(rng)

    def reexecute(self, rng=None):
        """src/circuit.rs:608-611: run again from the previous state."""
        self.reexecute_with_rng(rng if rng is not None else (self.rng or Rng()))

    def reexecute_with_rng(self, rng):
        if self.c_state is None or self.q_state is None:
            raise NotExecuted("Circuit has not been run yet")
        self.rng = rng
        self._do_execute(self.q_state, self.c_state, rng)

    def _segments(self):
        """Op list with runs of consecutive gates grouped: ("seq", [ops])."""
        if self._segs is not None:
            return self._segs
        out = []
        for op in self.ops:
            if op[0] == "gate":
                if out and out[-1][0] == "seq":
                    out[-1][1].append(op)
                else:
                    out.append(("seq", [op]))
            else:
                out.append(op)
        self._segs = out
        return out

    def _run_seq(self, q_state, idx, seq):
        if hasattr(q_state, "apply_plan"):
            flat = self._frozen[idx] if self._frozen is not None else self._flat_current(idx, seq)
            key = (idx, q_state.precision)
            plan = self._plans.get(key)
            if plan is None:
                bits = [op[2] for op in seq]
                kinds = [op[1].plan_kind() for op in seq]
                width, tc, tiling = self.fusion_width, True, None
                if width == "auto":
                    from . import autotune
                    width, tc, tiling = autotune.tune(self.nr_qbits, q_state.precision, bits, flat, kinds=kinds)
                if q_state.precision == "c128" and width > 3:
                    # complex128 blocks of up to 3 qubits run on double-float
                    # pairs in warp tiles; larger ones would take the FP64 pipe
                    width = 3
                plan = Plan(self.nr_qbits, bits, width, tensor_cores=tc, kinds=kinds)
                if tiling is not None and tiling != Plan.DEFAULT_TC_TILING:
                    plan.set_tc_tiling(*tiling)
                self._plans[key] = plan
            q_state.apply_plan(plan, flat)
        else:
            for op in seq:
                q_state.apply_gate(op[1].matrix(), op[2])

    def _do_execute(self, q_state, c_state, rng):
        """src/circuit.rs:643-762"""
        H, S, Sdg = G.H().matrix(), G.S().matrix(), G.Sdg().matrix()
        # Y basis: Sdg then H before the measurement, H then S after it
        # (src/circuit.rs:692-703), each pair as one matrix
        to_y, from_y = H @ Sdg, S @ H
        for idx, op in enumerate(self._segments()):
            kind = op[0]
            if kind == "seq":
                self._run_seq(q_state, idx, op[1])
            elif kind == "cgate":
                _, control, target, gate, bits = op
                word = np.zeros(len(c_state), dtype=np.uint64)
                for dst, src in enumerate(control):
                    word |= ((c_state >> np.uint64(src)) & np.uint64(1)) << np.uint64(dst)
                apply = (word == np.uint64(target)).astype(np.uint8)
                q_state.apply_conditional_gate(apply, gate.matrix(), bits)
            elif kind in ("measure", "peek"):
                _, qbit, cbit, basis = op
                fn = q_state.measure_into if kind == "measure" else q_state.peek_into
                if basis == "x":
                    q_state.apply_gate(H, [qbit])
                    fn(qbit, cbit, c_state, rng=rng)
                    q_state.apply_gate(H, [qbit])
                elif basis == "y":
                    q_state.apply_gate(to_y, [qbit])
                    fn(qbit, cbit, c_state, rng=rng)
                    q_state.apply_gate(from_y, [qbit])
                else:
                    fn(qbit, cbit, c_state, rng=rng)
            elif kind in ("measure_all", "peek_all"):
                _, cbits, basis = op
                fn = q_state.measure_all_into if kind == "measure_all" else q_state.peek_all_into
                if basis == "x":
                    q_state.apply_unary_gate_all(H)
                    fn(cbits, c_state, rng=rng)
                    q_state.apply_unary_gate_all(H)
                elif basis == "y":
                    q_state.apply_unary_gate_all(to_y)
                    fn(cbits, c_state, rng=rng)
                    q_state.apply_unary_gate_all(from_y)
                else:
                    fn(cbits, c_state, rng=rng)
            elif kind == "reset":
                q_state.reset(op[1], rng=rng)
            elif kind == "reset_all":
                q_state.reset_all()
            elif kind == "barrier":
                pass

    # ----------------------------------------------------------- results
    def cstate(self):
        return self.c_state

    # from this many runs the words are counted on the GPU (q1g_histogram)
    # rather than sorted on the host
    DEVICE_HISTOGRAM_RUNS = 1 << 16

    def histogram(self):
        """src/circuit.rs:773-789: {u64 key: count}, cbit 0 = LSB."""
        if self.c_state is None:
            raise NotExecuted("Circuit has not been run yet")
        if len(self.c_state) >= self.DEVICE_HISTOGRAM_RUNS:
            from .vectorstate import device_histogram
            keys, cnt = device_histogram(self.c_state, sort=False)
        else:
            keys, cnt = np.unique(self.c_state, return_counts=True)
        return dict(zip(keys.tolist(), cnt.tolist()))

    def histogram_vec(self):
        """src/circuit.rs:800-815"""
        if self.c_state is None:
            raise NotExecuted("Circuit has not been run yet")
        return np.bincount(self.c_state.astype(np.int64), minlength=1 << self.nr_cbits).tolist()

    def histogram_string(self):
        """src/circuit.rs:823-841: keys are binary strings, cbit 0 last."""
        return {format(k, f"0{self.nr_cbits}b"): c for k, c in self.histogram().items()}
