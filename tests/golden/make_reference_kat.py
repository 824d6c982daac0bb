"""Write reference_kat.json: the known answers of the reference's own tests.

Every case restates one assertion block of arrayfire/afQuantumSim
test/tests.cpp (line ranges cited per case): the initial per-qubit QState
amplitudes (before QState's normalisation), the gates, and the amplitudes,
indices or matrix equalities the reference asserts.  Composite builders
(ControlGate, Gate, NControl_Gate, Control_Group_Gate, Group_Gate,
Rewire_Gate) appear in their lowered form: each sub-gate with the extra
control the builder adds.  Angles are evaluated in float32 as the C++
expressions do (std::atan(0.75f), aqs::pi / 2.f, std::acos(0.6f) * 2.f).

Run:  python tests/golden/make_reference_kat.py   (writes next to itself)
"""
import json
from pathlib import Path

import numpy as np

f32 = np.float32
PI = f32(3.14159265358979323846)          # aqs::pi, include/quantum.h:121
ATAN075 = float(np.arctan(f32(0.75)))
ATAN1 = float(np.arctan(f32(1.0)))
PI_2 = float(PI / f32(2))
PI_3 = float(PI / f32(3))
PI_4 = float(PI / f32(4))
ACOS06x2 = float(f32(np.arccos(f32(0.6))) * f32(2))
S8 = 0.3535533906                          # invsqrt8, tests.cpp:747
R2 = float(np.sqrt(f32(0.5)))              # std::sqrt(1.0f / 2.0f), tests.cpp:986

ZERO = [1, 0, 0, 0]
ONE = [0, 0, 1, 0]
PLUS = [0.70710678118, 0, 0.70710678118, 0]
MINUS = [0.70710678118, 0, -0.70710678118, 0]
Q68 = [0.6, 0, 0, 0.8]                     # QState({0.6f,0},{0,0.8f})
Q86 = [0, 0.8, 0.6, 0]                     # QState({0,0.8f},{0.6f,0})


def g(name, *q, a=None, c=None, cv=None):
    d = {"g": name, "q": list(q)}
    if a is not None:
        d["a"] = float(a)
    if c:
        d["c"] = list(c)
        if cv is not None:
            d["cv"] = cv
    return d


cases = []


def amp(name, lines, init, gates, expect, cmp="fequal", tol=1e-4):
    cases.append({"type": "amplitudes", "name": name, "lines": lines, "n": len(init),
                  "init": init, "gates": gates, "expect": expect, "cmp": cmp, "tol": tol})


def mat(name, lines, n, ga, gb, cmp="exact", tol=0.0):
    cases.append({"type": "matrix_equal", "name": name, "lines": lines, "n": n,
                  "a": ga, "b": gb, "cmp": cmp, "tol": tol})


def peek(name, lines, init, gates, expect):
    cases.append({"type": "peek_measure_all", "name": name, "lines": lines, "n": len(init),
                  "init": init, "gates": gates, "expect": expect})


def marg(name, lines, init, expect, cmp="fequal", tol=1e-4):
    cases.append({"type": "marginals", "name": name, "lines": lines, "n": len(init),
                  "init": init, "expect": expect, "cmp": cmp, "tol": tol})


def sveq(name, lines, init_a, init_b, gates_b, tol):
    # tests.cpp asserts exact equality; whether QState{r, r} renormalises to
    # r depends on FMA contraction of the norm (with it: 1.0f; without it:
    # 0.99999994f), so the comparison carries an absolute tolerance.
    cases.append({"type": "statevector_equal", "name": name, "lines": lines,
                  "n": len(init_a), "init_a": init_a, "init_b": init_b, "gates": gates_b,
                  "tol": tol})


# ---- test_qsim_gates, tests.cpp:414-1005 (4 qubits) -------------------------
S0001 = [ZERO, ZERO, ZERO, ONE]
amp("X", "424-439", S0001, [g("X", 2), g("X", 3)], [[0b0010, 1, 0]], "exact")
amp("Y", "441-459", S0001, [g("Y", 2), g("Y", 3)], [[0b0010, 1, 0]], "exact")
amp("Z", "461-479", S0001, [g("Z", 2), g("Z", 3)], [[0b0001, -1, 0]], "exact")
amp("Not", "481-491", S0001, [g("X", 2), g("X", 3)], [[0b0010, 1, 0]], "exact")
amp("H", "493-519", S0001, [g("H", 2), g("H", 3)],
    [[0, .5, 0], [1, -.5, 0], [2, .5, 0], [3, -.5, 0]])
amp("Phase", "521-547", [ZERO, ZERO, Q68, ZERO],
    [g("Phase", 2, a=ATAN075), g("Phase", 3, a=ATAN1)],
    [[0, .6, 0], [1, 0, 0], [2, -.48, .64], [3, 0, 0]])
amp("RotX", "549-565", [ZERO, ZERO, MINUS, ZERO], [g("RotX", 2, a=PI_2)],
    [[0, .5, .5], [1, 0, 0], [2, -.5, -.5], [3, 0, 0]])
amp("RotY", "567-583", [ZERO, ZERO, ONE, ZERO], [g("RotY", 2, a=ACOS06x2)],
    [[0, -.8, 0], [1, 0, 0], [2, .6, 0], [3, 0, 0]])
amp("RotZ", "585-601", [ZERO, ZERO, MINUS, ZERO], [g("RotZ", 2, a=-PI_2)],
    [[0, .5, .5], [1, 0, 0], [2, -.5, .5], [3, 0, 0]])
S01qq = [ZERO, ONE, Q68, Q68]
CXEXP = [[0b0100, 0, .48], [0b0101, .36, 0], [0b0110, -.64, 0], [0b0111, 0, .48]]
amp("Xor", "603-619", S01qq, [g("CX", 0, 2), g("CX", 1, 3)], CXEXP)
amp("Swap", "621-637", [ZERO, ONE, Q68, Q86], [g("Swap", 0, 2), g("Swap", 1, 3)],
    [[0b0001, 0, .48], [0b0101, .36, 0], [0b1001, -.64, 0], [0b1101, 0, .48]])
amp("CNOT", "639-655", S01qq, [g("CX", 0, 2), g("CX", 1, 3)], CXEXP)
amp("CX", "657-671", [[1, 0, 0, 0], [0, 0, 1, 0], Q68, Q68],
    [g("CX", 0, 2), g("CX", 1, 3)], CXEXP)
amp("CY", "687-703", S01qq, [g("CY", 0, 2), g("CY", 1, 3)],
    [[0b0100, .48, 0], [0b0101, 0, .36], [0b0110, 0, .64], [0b0111, -.48, 0]])
amp("CZ", "705-720", S01qq, [g("CZ", 0, 2), g("CZ", 1, 3)],
    [[0b0100, .36, 0], [0b0101, 0, -.48], [0b0110, 0, .48], [0b0111, .64, 0]])
amp("CPhase", "722-738", S01qq,
    [g("CPhase", 0, 2, a=ATAN075), g("CPhase", 1, 3, a=ATAN075)],
    [[0b0100, .36, 0], [0b0101, -.288, .384], [0b0110, 0, .48], [0b0111, -.512, -.384]])
amp("CRotX", "740-760", [ZERO, ONE, MINUS, MINUS],
    [g("CRotX", 0, 2, a=PI_2), g("CRotX", 1, 3, a=PI_2)],
    [[0b0100, S8, S8], [0b0101, -S8, -S8], [0b0110, -S8, -S8], [0b0111, S8, S8]])
amp("CRotY", "762-779", [ZERO, ONE, ONE, ONE],
    [g("CRotY", 0, 2, a=ACOS06x2), g("CRotY", 1, 3, a=ACOS06x2)],
    [[0b0100, 0, 0], [0b0101, 0, 0], [0b0110, -.8, 0], [0b0111, .6, 0]])
amp("CRotZ", "781-798", [ZERO, ONE, MINUS, MINUS],
    [g("CRotZ", 0, 2, a=-PI_2), g("CRotZ", 1, 3, a=-PI_2)],
    [[0b0100, S8, S8], [0b0101, -S8, S8], [0b0110, -S8, -S8], [0b0111, S8, -S8]])
OR = [g("Or", 0, 1, 2), g("Or", 1, 0, 3)]
amp("Or/1", "800-813", [ZERO, ONE, ZERO, ZERO], OR, [[0b0111, 1, 0]])
amp("Or/2", "815-819", [ONE, ONE, ZERO, ZERO], OR, [[0b1111, 1, 0]])
amp("Or/3", "821-825", [ZERO, ZERO, ZERO, ZERO], OR, [[0b0000, 1, 0]])
AND = [g("CCNot", 0, 1, 2), g("CCNot", 1, 0, 3)]
amp("And/1", "827-840", [ZERO, ONE, ZERO, ZERO], AND, [[0b0100, 1, 0]])
amp("And/2", "842-846", [ONE, ONE, ZERO, ZERO], AND, [[0b1111, 1, 0]])
amp("And/3", "848-852", [ZERO, ZERO, ZERO, ZERO], AND, [[0b0000, 1, 0]])
amp("CSwap/1", "854-869", [ZERO, ONE, Q68, Q86], [g("CSwap", 0, 2, 3)],
    [[0b0100, 0, .48], [0b0101, .36, 0], [0b0110, -.64, 0], [0b0111, 0, .48]])
amp("CSwap/2", "871-880", [ZERO, ONE, Q68, Q86], [g("CSwap", 1, 2, 3)],
    [[0b0100, 0, .48], [0b0101, -.64, 0], [0b0110, .36, 0], [0b0111, 0, .48]])
amp("CCNot/1", "882-895", [ZERO, ONE, ZERO, ZERO], AND, [[0b0100, 1, 0]])
amp("CCNot/2", "897-901", [ONE, ONE, ZERO, ZERO], AND, [[0b1111, 1, 0]])
amp("CCNot/3", "903-907", [ZERO, ZERO, ZERO, ZERO], AND, [[0b0000, 1, 0]])

# ControlGate(temp{H(0), CNot(0,1), Z(0), Swap(0,1)}, control, begin)
mat("ControlGate/0->2", "909-926", 4,
    [g("H", 2, c=[0]), g("CX", 2, 3, c=[0]), g("Z", 2, c=[0]), g("Swap", 2, 3, c=[0])],
    [g("CH", 0, 2), g("CCNot", 0, 2, 3), g("CZ", 0, 2), g("CSwap", 0, 2, 3)])
mat("ControlGate/2->0", "928-941", 4,
    [g("H", 0, c=[2]), g("CX", 0, 1, c=[2]), g("Z", 0, c=[2]), g("Swap", 0, 1, c=[2])],
    [g("CH", 2, 0), g("CCNot", 0, 2, 1), g("CZ", 2, 0), g("CSwap", 2, 0, 1)])
# Gate(temp{H(0), CPhase(0,1,1.0), X(1), Swap(0,1)}, 1)
mat("Gate", "943-961", 4,
    [g("H", 1), g("CPhase", 1, 2, a=1.0), g("X", 2), g("Swap", 1, 2)],
    [g("H", 1), g("CPhase", 1, 2, a=1.0), g("X", 2), g("Swap", 1, 2)])
sveq("CHadamard/1", "963-983", [ZERO, ZERO, ONE, ZERO], [ZERO, ZERO, ONE, ZERO],
     [g("CH", 0, 1), g("CH", 3, 2)], 0.0)
sveq("CHadamard/2", "985-1002", [ONE, [R2, 0, R2, 0], [R2, 0, -R2, 0], ONE],
     [ONE, ZERO, ONE, ONE], [g("CH", 0, 1), g("CH", 3, 2)], 2e-7)

# ---- test_special_gates, tests.cpp:1011-1135 --------------------------------
NC = [g("X", 3, c=[0, 2, 4, 5])]           # NControl_Gate(6, {0,2,4,5}, 3, X)
peek("NControl/1", "1015-1029", [ONE] * 6, NC, 0b111011)
peek("NControl/2", "1031-1034", [ONE, ONE, ONE, ZERO, ONE, ONE], NC, 0b111111)
peek("NControl/3", "1036-1040", [ONE, ZERO, ONE, ZERO, ONE, ONE], NC, 0b101111)
peek("NControl/4", "1042-1046", [ONE, ZERO, ONE, ONE, ONE, ONE], NC, 0b101011)
mat("NControl/CX", "1049-1058", 4, [g("X", 0, c=[3])], [g("CX", 3, 0)])
mat("NControl/CCNot", "1060-1070", 4, [g("X", 2, c=[0, 3])], [g("CCNot", 0, 3, 2)])
mat("Control_Group_Gate", "1073-1084", 4,
    [g("X", 0, c=[1]), g("X", 2, c=[1]), g("X", 3, c=[1])],
    [g("CX", 1, 0), g("CX", 1, 2), g("CX", 1, 3)])
mat("Group_Gate", "1086-1094", 4, [g("X", 0), g("X", 2), g("X", 3)],
    [g("X", 0), g("X", 2), g("X", 3)])
# Rewire_Gate(4, {2,1,3,0}, circuit{H0, CX(0,2), H1, Z3}): swap network, the
# gate, and the swaps undone (quantum_gates.cpp:184-231)
mat("Rewire_Gate", "1096-1108", 4,
    [g("Swap", 0, 2), g("Swap", 2, 3), g("H", 0), g("CX", 0, 2), g("H", 1), g("Z", 3),
     g("Swap", 2, 3), g("Swap", 0, 2)],
    [g("H", 2), g("CX", 2, 3), g("H", 1), g("Z", 0)])
# Adjoint_Gate (quantum_gates.cpp:233-338): the adjoint of `circuit`'s matrix
# equals `ref`'s within 1e-5 absolute (tests.cpp:1110-1132)
cases.append({"type": "matrix_adjoint", "name": "Adjoint_Gate", "lines": "1110-1132", "n": 4,
              "a": [g("Swap", 1, 2), g("CPhase", 2, 1, a=float(-PI / f32(3))),
                    g("CRotX", 1, 3, a=float(PI / f32(4))), g("X", 0),
                    g("CRotY", 3, 0, a=float(-PI / f32(2)))],
              "b": [g("CRotY", 3, 0, a=float(PI / f32(2))), g("X", 0),
                    g("CRotX", 1, 3, a=float(-PI / f32(4))), g("CPhase", 2, 1, a=float(PI / f32(3))),
                    g("Swap", 1, 2)],
              "cmp": "abs", "tol": 1e-5})

# ---- test_qsim_measurement, tests.cpp:274-336 (3 qubits) --------------------
peek("measure/zero", "281-286", [ZERO] * 3, [], 0)
peek("measure/101", "292-300", [ONE, ZERO, ONE], [], 0b101)
cases.append({"type": "collapse", "name": "measure/q0", "lines": "313-333", "n": 3,
              "init": [[0, 1, -1, 0], ZERO, Q68], "qubit": 0,
              "branches": {"1": [[0b100, -.6, 0], [0b101, 0, -.8]],
                           "0": [[0b000, 0, .6], [0b001, -.8, 0]]}, "tol": 1e-4})

# ---- test_qsim_probability, tests.cpp:1141-1194 (4 qubits) -------------------
marg("probability/zero", "1148-1155", [ZERO] * 4, [0, 0, 0, 0], "exact")
marg("probability/q3=1", "1157-1169", [ZERO, ZERO, ZERO, [0, 0, 1, 0]], [0, 0, 0, 1], "exact")
marg("probability/q3=+", "1171-1181", [ZERO, ZERO, ZERO, [1, 0, 1, 0]], [0, 0, 0, .5])
marg("probability/q0", "1183-1194", [Q68, ZERO, ZERO, [1, 0, 1, 0]], [.64, 0, 0, .5])

out = Path(__file__).with_name("reference_kat.json")
out.write_text(json.dumps({"source": "arrayfire/afQuantumSim test/tests.cpp",
                           "cases": cases}, indent=1))
print(f"wrote {len(cases)} cases to {out}")
