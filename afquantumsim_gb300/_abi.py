"""ctypes mirror of include/aqsg.h (structs and constants only, no loading)."""
from __future__ import annotations

import ctypes as C

MAX_QUBITS = 34
MAX_UNITARY_QUBITS = 5
OP_MAX_QUBITS = 5
OP_MAX_CONTROLS = 16

# aqsg_status
OK = 0
ERR_OUT_OF_RANGE = -1
ERR_INVALID_ARGUMENT = -2
ERR_DOMAIN = -3
ERR_RUNTIME = -4
ERR_CUDA = -5
ERR_OUT_OF_MEMORY = -6
ERR_TIMEOUT = -7
ERR_NULL = -8

# aqsg_dtype
C64 = 0
C128 = 1

# aqsg_op_kind (values 0..20 follow QGate::GateTypes, include/quantum.h:776-800)
BARRIER, X, Y, Z, H, PHASE, SWAP, RX, RY, RZ = range(10)
CX, CY, CZ, CH, CPHASE, CSWAP, CRX, CRY, CRZ, CCX, OR = range(10, 21)
UNITARY = 32

KIND_NAMES = {
    BARRIER: "Barrier", X: "X", Y: "Y", Z: "Z", H: "H", PHASE: "Phase",
    SWAP: "Swap", RX: "RotX", RY: "RotY", RZ: "RotZ", CX: "CX", CY: "CY",
    CZ: "CZ", CH: "CH", CPHASE: "CPhase", CSWAP: "CSwap", CRX: "CRotX",
    CRY: "CRotY", CRZ: "CRotZ", CCX: "CCNot", OR: "Or", UNITARY: "Unitary",
}

ARITY = {BARRIER: 0, X: 1, Y: 1, Z: 1, H: 1, PHASE: 1, RX: 1, RY: 1, RZ: 1,
         SWAP: 2, CX: 2, CY: 2, CZ: 2, CH: 2, CPHASE: 2, CRX: 2, CRY: 2,
         CRZ: 2, CSWAP: 3, CCX: 3, OR: 3}

# aqsg_exec_mode
EXEC_AUTO = 0
EXEC_PER_GATE = 1
EXEC_TILED = 2

# aqsg_sample_rule
SAMPLE_REFERENCE = 0
SAMPLE_CLAMP = 1


class Op(C.Structure):
    """struct aqsg_op"""
    _fields_ = [
        ("kind", C.c_int32),
        ("num_qubits", C.c_int32),
        ("num_controls", C.c_int32),
        ("control_values", C.c_uint32),
        ("angle", C.c_float),
        ("qubits", C.c_int32 * OP_MAX_QUBITS),
        ("controls", C.c_int32 * OP_MAX_CONTROLS),
        ("matrix", C.POINTER(C.c_double)),
    ]


def make_op(kind: int, qubits=(), angle: float = 0.0, controls=(),
            control_values=None, matrix=None, keep=None) -> Op:
    """Build one aqsg_op.  `matrix` (UNITARY) is a complex (2^k, 2^k) array;
    its storage is appended to `keep` (a list) so it outlives the call."""
    op = Op()
    op.kind = kind
    qubits = list(qubits)
    op.num_qubits = len(qubits)
    for i, q in enumerate(qubits):
        op.qubits[i] = int(q)
    op.angle = float(angle)
    controls = list(controls)
    op.num_controls = len(controls)
    for i, c in enumerate(controls):
        op.controls[i] = int(c)
    if control_values is None:
        control_values = (1 << len(controls)) - 1
    op.control_values = int(control_values)
    if matrix is not None:
        import numpy as np
        m = np.ascontiguousarray(np.asarray(matrix, dtype=np.complex128))
        buf = m.view(np.float64).copy()
        if keep is not None:
            keep.append(buf)
        op.matrix = buf.ctypes.data_as(C.POINTER(C.c_double))
        op._buf = buf  # keep alive with the struct
    return op


def op_array(ops) -> "C.Array":
    arr = (Op * len(ops))()
    for i, o in enumerate(ops):
        arr[i] = o
    arr._keep = [getattr(o, "_buf", None) for o in ops]
    return arr
