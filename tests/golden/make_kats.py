"""Writes vectorstate_kats.json: the reference's known-answer tests for the
statevector path, transcribed from its Rust unit tests (each case cites the
test it comes from).  The reference is Rust and cannot run here, so the
expected values are the literal arrays of those tests; gate matrices are
restated from the reference's `matrix()` definitions.

Run:  python tests/golden/make_kats.py
"""
import json
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

z = 0j
o = 1 + 0j
i = 1j
x = complex(1 / math.sqrt(2), 0)      # COMPLEX_HSQRT2, src/cmatrix.rs:17
h = 0.5 * o


def polar(r, t):
    return complex(r * math.cos(t), r * math.sin(t))


# gate matrices, src/gates/*.rs matrix()
MATS = {
    "H": [[x, x], [x, -x]],
    "X": [[z, o], [o, z]],
    "Y": [[z, -i], [i, z]],
    "CX": [[o, z, z, z], [z, o, z, z], [z, z, z, o], [z, z, o, z]],
    "CCX": None,  # filled below
    "HH": None,   # Kron(H, H)
}
ccx = np.eye(8, dtype=complex)
ccx[6:, 6:] = [[0, 1], [1, 0]]
MATS["CCX"] = ccx.tolist()
MATS["HH"] = np.kron(np.array(MATS["H"]), np.array(MATS["H"])).tolist()


def u3(theta, phi, lmb):
    c, s = math.cos(theta / 2), math.sin(theta / 2)
    return [[complex(c, 0), -polar(s, lmb)], [polar(s, phi), polar(c, phi + lmb)]]


def u2(phi, lmb):
    return [[complex(x.real, 0), -polar(x.real, lmb)], [polar(x.real, phi), polar(x.real, phi + lmb)]]


def rx(t):
    c, si = complex(math.cos(t / 2), 0), complex(0, math.sin(t / 2))
    return [[c, -si], [-si, c]]


def rz(l):
    p = polar(1.0, l / 2)
    return [[p.conjugate(), z], [z, p]]


def ch():
    m = np.eye(4, dtype=complex)
    m[2:, 2:] = MATS["H"]
    return m.tolist()


def enc(m):
    """complex nested list -> [[re, im], ...] nested"""
    a = np.asarray(m, dtype=complex)
    return np.stack([a.real, a.imag], axis=-1).tolist()


def col(*vals):
    return [[v] for v in vals]


def main():
    vs = []

    def case(name, source, init, ops, counts, states):
        vs.append({"name": name, "source": source, "init": init, "ops": ops,
                   "expect": {"counts": counts, "states": enc(states)}})

    def new(n, shots):
        return {"kind": "new", "nr_bits": n, "nr_shots": shots}

    def coefs(vals, shots):
        return {"kind": "coefs", "coefs": enc(vals), "nr_shots": shots}

    def gate(name, bits):
        return {"op": "gate", "mat": enc(MATS[name]), "bits": bits, "name": name}

    def cond(control, name, bits):
        return {"op": "cond", "control": control, "mat": enc(MATS[name]), "bits": bits, "name": name}

    src = "src/vectorstate.rs"
    # test_new, src/vectorstate.rs:426-443
    case("new_1", f"{src}:431-435", new(1, 1024), [], [1024], col(o, z))
    case("new_3", f"{src}:437-442", new(3, 1500), [], [1500], col(o, z, z, z, z, z, z, z))
    # test_from_qubit_coefs, src/vectorstate.rs:446-470
    case("coefs_01", f"{src}:453-457", coefs([o, z, z, o], 1), [], [1], col(z, o, z, z))
    case("coefs_10", f"{src}:459-463", coefs([z, o, o, z], 13), [], [13], col(z, z, o, z))
    case("coefs_unnormalised", f"{src}:465-470", coefs([o, o, -i, z], 9), [], [9],
         col(-x * i, z, -x * i, z))
    # test_apply_conditional_gate, src/vectorstate.rs:473-509
    case("cond_x1", f"{src}:479-482", new(2, 5), [cond([0, 0, 1, 1, 0], "X", [1])], [2, 2, 1],
         [[o, z, o], [z, o, z], [z, z, z], [z, z, z]])
    case("cond_x0", f"{src}:484-487", new(2, 5), [cond([0, 0, 1, 1, 1], "X", [0])], [2, 3],
         [[o, z], [z, z], [z, o], [z, z]])
    case("cond_h1", f"{src}:489-493", new(2, 5), [cond([1, 0, 1, 1, 0], "H", [1])], [1, 1, 2, 1],
         [[x, o, x, o], [x, z, x, z], [z, z, z, z], [z, z, z, z]])
    case("cond_cx", f"{src}:495-499", coefs([o, z, x, x], 5), [cond([1, 0, 1, 1, 0], "CX", [1, 0])],
         [1, 1, 2, 1], [[x, x, x, x], [z, x, z, x], [z, z, z, z], [x, z, x, z]])
    case("cond_h0_twice", f"{src}:501-508", new(2, 5),
         [cond([1, 1, 1, 0, 0], "H", [0]), cond([0, 0, 1, 1, 1], "H", [0])], [2, 1, 2],
         [[x, o, x], [z, z, z], [x, z, x], [z, z, z]])
    # test_apply_unary_gate, src/vectorstate.rs:641-658
    case("unary_h0", f"{src}:647-649", new(3, 1), [gate("H", [0])], [1], col(x, z, z, z, x, z, z, z))
    case("unary_h1", f"{src}:651-653", new(3, 1), [gate("H", [1])], [1], col(x, z, x, z, z, z, z, z))
    case("unary_y2", f"{src}:655-657", new(3, 1), [gate("Y", [2])], [1], col(z, i, z, z, z, z, z, z))
    # test_apply_binary_gate, src/vectorstate.rs:661-683
    case("binary_cx01_zero", f"{src}:667-669", new(3, 1), [gate("CX", [0, 1])], [1],
         col(o, z, z, z, z, z, z, z))
    case("binary_cx01", f"{src}:671-673", coefs([z, o, o, z, o, z], 1), [gate("CX", [0, 1])], [1],
         col(z, z, z, z, z, z, o, z))
    case("binary_cx02", f"{src}:675-677", coefs([z, o, o, z, o, z], 1), [gate("CX", [0, 2])], [1],
         col(z, z, z, z, z, o, z, z))
    case("binary_hh12", f"{src}:679-682", coefs([z, o, o, z, o, z], 1), [gate("HH", [1, 2])], [1],
         col(z, z, z, z, h, h, h, h))
    # test_apply_n_ary_gate, src/vectorstate.rs:686-707
    case("ccx_zero", f"{src}:693-695", new(3, 1), [gate("CCX", [0, 1, 2])], [1],
         col(o, z, z, z, z, z, z, z))
    case("ccx_021_then_012", f"{src}:697-701", coefs([z, o, z, o, o, z], 1),
         [gate("CCX", [0, 2, 1]), gate("CCX", [0, 1, 2])], [1], col(z, z, z, z, z, z, z, o))
    case("ccx_superposed", f"{src}:703-706", coefs([x, -x, x, -x, x, -x], 1), [gate("CCX", [0, 2, 1])],
         [1], col(0.5 * x, -0.5 * x, -0.5 * x, 0.5 * x, -0.5 * x, -0.5 * x, 0.5 * x, 0.5 * x))
    # test_reset_all, src/vectorstate.rs:814-829
    e0 = [[o]] + [[z]] * 31
    case("reset_all", f"{src}:814-829", new(5, 100),
         [gate("H", [2]), gate("X", [0]), gate("H", [4]), {"op": "reset_all"}], [100], e0)

    # gate matrix KATs (test_matrix of src/gates/*.rs)
    mk = []

    def mat_case(gate_name, params, expect, source):
        mk.append({"gate": gate_name, "params": params, "expect": enc(expect), "source": source})

    mat_case("U3", [0.32, math.pi / 4, math.log(2)],
             [[complex(0.9872272833756269, 0.0), complex(-0.1225537622232209, -0.1017981646382380)],
              [complex(0.1126549842634128, 0.1126549842634128), complex(0.09094356700076842, 0.9830294892130130)]],
             "src/gates/u3.rs:148-155")
    mat_case("U2", [math.pi / 4, math.log(2)],
             [[complex(0.7071067811865476, 0.0), complex(-0.5439340435069544, -0.4518138513969824)],
              [complex(0.5, 0.5), complex(0.06513881252516862, 0.7041000888388035)]],
             "src/gates/u2.rs:156-163")
    mat_case("RX", [math.pi / 2], [[x, -x * i], [-x * i, x]], "src/gates/rx.rs:187-188")
    mat_case("RX", [math.pi], [[z, -i], [-i, z]], "src/gates/rx.rs:190-191")
    mat_case("RZ", [math.pi], [[-i, z], [z, i]], "src/gates/rz.rs:173-176")
    mat_case("V", [], [[h + 0.5 * i, h - 0.5 * i], [h - 0.5 * i, h + 0.5 * i]], "src/gates/v.rs:255-256")
    mat_case("Vdg", [], [[h - 0.5 * i, h + 0.5 * i], [h + 0.5 * i, h - 0.5 * i]], "src/gates/v.rs:258-259")
    mat_case("CX", [], MATS["CX"], "src/gates/cx.rs:150-160")
    mat_case("CH", [], [[o, z, z, z], [z, o, z, z], [z, z, x, x], [z, z, x, -x]],
             "src/gates/controlled.rs:591-597")
    ccrz = np.eye(8, dtype=complex)
    ccrz[6, 6], ccrz[7, 7] = -i, i
    mat_case("CCRZ", [math.pi], ccrz.tolist(), "src/gates/controlled.rs:599-609")
    t4 = polar(1.0, math.pi / 4)
    mat_case("H", [], [[x, x], [x, -x]], "src/gates/hadamard.rs:186-191")
    mat_case("X", [], [[z, o], [o, z]], "src/gates/x.rs:164-170")
    mat_case("Y", [], [[z, -i], [i, z]], "src/gates/y.rs:161-167")
    mat_case("Z", [], [[o, z], [z, -o]], "src/gates/z.rs:152-158")
    mat_case("I", [], [[o, z], [z, o]], "src/gates/identity.rs:142-148")
    mat_case("S", [], [[o, z], [z, i]], "src/gates/s.rs:297-308")
    mat_case("Sdg", [], [[o, z], [z, -i]], "src/gates/s.rs:297-308")
    mat_case("T", [], [[o, z], [z, t4]], "src/gates/t.rs:246-257")
    mat_case("Tdg", [], [[o, z], [z, t4.conjugate()]], "src/gates/t.rs:246-257")
    mat_case("U1", [math.pi / 2], [[o, z], [z, i]], "src/gates/u1.rs:154-161")
    mat_case("RY", [math.pi / 2], [[x, -x], [x, x]], "src/gates/ry.rs:184-195")
    mat_case("RY", [math.pi], [[z, -o], [o, z]], "src/gates/ry.rs:184-195")
    mat_case("Swap", [], [[o, z, z, z], [z, z, o, z], [z, o, z, z], [z, z, z, o]], "src/gates/swap.rs:189-200")
    mat_case("CY", [], [[o, z, z, z], [z, o, z, z], [z, z, z, -i], [z, z, i, z]], "src/gates/cy.rs:146-159")
    mat_case("CZ", [], [[o, z, z, z], [z, o, z, z], [z, z, o, z], [z, z, z, -o]], "src/gates/cz.rs:144-156")

    # compound gates (test_matrix of kron.rs, composite.rs, staticloop.rs):
    # a spec is {"gate", "params"}, {"kron": [a, b]}, {"composite": name,
    # "nbits", "ops": [[spec, bits], ...]} or {"loop": count, "body": spec}
    ck = []

    def g(name, params=()):
        return {"gate": name, "params": list(params)}

    def compound(spec, expect, source):
        ck.append({"spec": spec, "expect": enc(expect), "source": source})

    compound({"kron": [g("I"), g("H")]}, [[x, x, z, z], [x, -x, z, z], [z, z, x, x], [z, z, x, -x]],
             "src/gates/kron.rs:202-235")
    compound({"kron": [g("H"), g("H")]}, [[h, h, h, h], [h, -h, h, -h], [h, h, -h, -h], [h, -h, -h, h]],
             "src/gates/kron.rs:202-235")
    compound({"kron": [g("H"), {"kron": [g("I"), g("H")]}]},
             [[h, h, z, z, h, h, z, z], [h, -h, z, z, h, -h, z, z], [z, z, h, h, z, z, h, h],
              [z, z, h, -h, z, z, h, -h], [h, h, z, z, -h, -h, z, z], [h, -h, z, z, -h, h, z, z],
              [z, z, h, h, z, z, -h, -h], [z, z, h, -h, z, z, -h, h]],
             "src/gates/kron.rs:202-235")
    compound({"composite": "CZ", "nbits": 2, "ops": [[g("H"), [1]], [g("CX"), [0, 1]], [g("H"), [1]]]},
             [[o, z, z, z], [z, o, z, z], [z, z, o, z], [z, z, z, -o]], "src/gates/composite.rs:665-717")
    compound({"composite": "Inc", "nbits": 2,
              "ops": [[g("H"), [0]], [g("H"), [1]], [g("CX"), [0, 1]], [g("H"), [1]], [g("H"), [0]],
                      [g("X"), [1]]]},
             [[z, z, z, o], [o, z, z, z], [z, o, z, z], [z, z, o, z]], "src/gates/composite.rs:665-717")
    inc3 = np.roll(np.eye(8, dtype=complex), 1, axis=0)
    compound({"composite": "Inc", "nbits": 3,
              "ops": [[g("H"), [0]], [g("H"), [2]], [g("CCX"), [0, 1, 2]], [g("H"), [2]], [g("H"), [1]],
                      [g("H"), [2]], [g("CX"), [1, 2]], [g("H"), [2]], [g("H"), [0]], [g("H"), [1]],
                      [g("X"), [2]]]},
             inc3.tolist(), "src/gates/composite.rs:665-717")
    compound({"loop": 3, "body": {"composite": "body", "nbits": 1, "ops": [[g("RX", [1.0471975511965976]), [0]]]}},
             [[z, -i], [-i, z]], "src/gates/staticloop.rs:265-272")

    # gate_test KATs: the gate applied to every column of a k-qubit state
    ak = []

    def apply_case(gate_name, params, mat, state, result, source):
        k = int(round(math.log2(len(mat))))
        ak.append({"gate": gate_name, "params": params, "mat": enc(mat), "bits": list(range(k)),
                   "state": enc(state), "expect": enc(result), "source": source})

    apply_case("U3", [3 * math.pi / 2, math.pi / 4, math.pi / 2], u3(3 * math.pi / 2, math.pi / 4, math.pi / 2),
               [[x, x], [z, -x], [x, z], [z, z]],
               (np.array([[-o - i, -o], [z, o], [2 * x, (o + i) * x], [z, -(o + i) * x]]) * 0.5).tolist(),
               "src/gates/u3.rs:158-173")
    apply_case("U2", [math.pi / 4, math.pi / 2], u2(math.pi / 4, math.pi / 2),
               [[x, x], [z, -x], [x, z], [z, z]],
               (np.array([[o - i, o], [z, -o], [2 * i * x, (o + i) * x], [z, -(o + i) * x]]) * 0.5).tolist(),
               "src/gates/u2.rs:166-183")
    apply_case("RZ", [math.pi / 2], rz(math.pi / 2),
               [[o, z, x, x], [z, o, x, -x]],
               [[x * (o - i), z, 0.5 * (o - i), 0.5 * (o - i)], [z, x * (o + i), 0.5 * (o + i), -0.5 * (o + i)]],
               "src/gates/rz.rs:180-196")
    apply_case("CX", [], MATS["CX"],
               [[o, z, h, z], [z, z, -h, z], [z, o, h, x], [z, z, -h, -x]],
               [[o, z, h, z], [z, z, -h, z], [z, z, -h, -x], [z, o, h, x]],
               "src/gates/cx.rs:163-177")
    apply_case("CH", [], ch(),
               [[o, z, h, z], [z, z, -h, z], [z, o, h, x], [z, z, -h, -x]],
               [[o, z, h, z], [z, z, -h, z], [z, x, z, z], [z, x, x, o]],
               "src/gates/controlled.rs:611-645")
    # the one-qubit gates on the 2-row state [[1, 0, x, x], [0, 1, x, -x]]
    one = [[o, z, x, x], [z, o, x, -x]]
    apply_case("H", [], MATS["H"], one, [[x, x, o, z], [x, -x, z, o]], "src/gates/hadamard.rs:194-202")
    apply_case("X", [], MATS["X"], one, [[z, o, x, -x], [o, z, x, x]], "src/gates/x.rs:173-181")
    apply_case("Y", [], MATS["Y"], one, [[z, -i, -i * x, i * x], [i, z, i * x, i * x]], "src/gates/y.rs:170-179")
    apply_case("Z", [], [[o, z], [z, -o]], one, [[o, z, x, x], [z, -o, -x, x]], "src/gates/z.rs:161-169")
    apply_case("S", [], [[o, z], [z, i]], one, [[o, z, x, x], [z, i, x * i, -x * i]], "src/gates/s.rs:311-337")
    apply_case("Sdg", [], [[o, z], [z, -i]], one, [[o, z, x, x], [z, -i, -x * i, x * i]], "src/gates/s.rs:311-337")
    apply_case("U1", [math.pi / 4], [[o, z], [z, polar(1.0, math.pi / 4)]], one,
               [[o, z, x, x], [z, x * (o + i), 0.5 * (o + i), -0.5 * (o + i)]], "src/gates/u1.rs:164-174")
    apply_case("RY", [math.pi / 2], [[x, -x], [x, x]], one, [[x, -x, z, o], [x, x, o, z]],
               "src/gates/ry.rs:198-213")
    # T and Tdg on the top qubit of a 4-row state
    tq = polar(1.0, math.pi / 4)
    four = [[o, z, x, h], [z, o, z, -h], [z, z, x, h], [z, z, z, -h]]
    four = [row + [e] for row, e in zip(four, [z, z, z, o])]
    apply_case("T", [], [[o, z], [z, tq]], four,
               [[o, z, x, h, z], [z, o, z, -h, z], [z, z, tq * x, tq * h, z], [z, z, z, -tq * h, tq]],
               "src/gates/t.rs:260-296")
    td = tq.conjugate()
    apply_case("Tdg", [], [[o, z], [z, td]], four,
               [[o, z, x, h, z], [z, o, z, -h, z], [z, z, td * x, td * h, z], [z, z, z, -td * h, td]],
               "src/gates/t.rs:260-296")
    apply_case("Swap", [], [[o, z, z, z], [z, z, o, z], [z, o, z, z], [z, z, z, o]],
               [[o, z, x, x, x, h, z], [z, o, x, -x, z, -h, z], [z, z, z, z, x, h, o], [z, z, z, z, z, -h, z]],
               [[o, z, x, x, x, h, z], [z, z, z, z, x, h, o], [z, o, x, -x, z, -h, z], [z, z, z, z, z, -h, z]],
               "src/gates/swap.rs:203-222")
    two = [[o, z, h, z], [z, z, -h, z], [z, o, h, x], [z, z, -h, -x]]
    apply_case("CY", [], [[o, z, z, z], [z, o, z, z], [z, z, z, -i], [z, z, i, z]], two,
               [[o, z, h, z], [z, z, -h, z], [z, z, h * i, x * i], [z, i, h * i, x * i]], "src/gates/cy.rs:162-183")
    apply_case("CZ", [], [[o, z, z, z], [z, o, z, z], [z, z, o, z], [z, z, z, -o]], two,
               [[o, z, h, z], [z, z, -h, z], [z, o, h, x], [z, z, h, x]], "src/gates/cz.rs:159-179")
    apply_case("CCX", [], MATS["CCX"],
               [[o, z, z], [z, z, z], [z, z, z], [z, x, z], [z, z, z], [z, z, z], [z, z, -x], [z, -x, x]],
               [[o, z, z], [z, z, z], [z, z, z], [z, x, z], [z, z, z], [z, z, z], [z, -x, x], [z, z, -x]],
               "src/gates/controlled.rs:647-676")

    # support helpers, src/support.rs:100-118
    bits = {
        "reverse_bits": [[1, 1, 1], [1, 4, 8], [10, 4, 5], [26, 4, 5], [0xfffffffffffffffa, 4, 0x5],
                         [0xffffffffffffaaaa, 32, 0x5555ffff], [0x1ffffffffffffffa, 64, 0x5ffffffffffffff8]],
        "shuffle_bits": [[0xc, [0, 3, 1, 2], 0x6], [0xfffffffffffffffa, [8, 9, 10, 11], 0xa00],
                         [0xf555555555555555, [63, 62, 61, 60], 0xa000000000000000], [0x3, [3, 2, 1, 0], 0xc]],
        "source": "src/support.rs:100-118",
    }
    # binomial acceptance bounds, src/stats.rs:38-45
    stats = {"bounds": [[1024, 0.5, 1e-5, 443, 581], [1234, 0.25, 1e-5, 243, 374], [1234, 0.75, 1e-5, 860, 991],
                        [1234, 0.75, 1e-10, 828, 1023], [1_000_000, 0.43, 1e-4, 428158, 431842]],
             "source": "src/stats.rs:38-45"}

    out = {"vectorstate": vs, "matrix": mk, "compound": ck, "apply": ak, "bits": bits, "stats": stats}
    path = os.path.join(HERE, "vectorstate_kats.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print(path, len(vs), len(mk), len(ck), len(ak))


if __name__ == "__main__":
    main()
