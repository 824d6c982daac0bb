"""ctypes binding of the CPU oracle (oracle/aqs_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py: GPU results are compared with it, and the
CPU-baseline leg times it as the CPU arm; it is never the product measured
or shipped.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from afquantumsim_gb300._abi import Op, op_array

ORACLE_DIR = Path(__file__).resolve().parent
LIB_PATH = ORACLE_DIR / "_build" / "libaqs_oracle.so"
_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            from afquantumsim_gb300.build import build_oracle
            build_oracle()
        L = C.CDLL(str(LIB_PATH))
        P = C.c_void_p
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_get_threads.restype = C.c_int
        L.orc_apply_ops_f64.argtypes = [P, C.c_int, C.POINTER(Op), C.c_int]
        L.orc_apply_ops_f32.argtypes = [P, C.c_int, C.POINTER(Op), C.c_int]
        L.orc_probs_f64.argtypes = [P, C.c_int, P]
        L.orc_probs_f32.argtypes = [P, C.c_int, P]
        L.orc_first_index.argtypes = [P, C.c_int, C.c_double]
        L.orc_first_index.restype = C.c_int64
        L.orc_qubit_prob_f64.argtypes = [P, C.c_int, C.c_int]
        L.orc_qubit_prob_f64.restype = C.c_double
        L.ref32_product_state.argtypes = [C.c_int, P, P]
        L.ref32_qstate_normalize.argtypes = [P]
        L.ref32_apply_ops.argtypes = [P, C.c_int, C.c_int, C.POINTER(Op), C.c_int]
        L.ref32_peek_measure_all.argtypes = [P, C.c_int, C.c_float]
        L.ref32_peek_measure_all.restype = C.c_uint32
        L.ref32_profile_measure_all.argtypes = [P, C.c_int, C.c_uint32, P, P, P]
        L.ref32_qubit_probability_true.argtypes = [P, C.c_int, C.c_int]
        L.ref32_qubit_probability_true.restype = C.c_float
        L.ref32_basis_matrix_f.argtypes = [C.c_int, C.c_int, P]
        L.ref32_set_basis.argtypes = [P, C.c_int, C.c_int, C.c_int]
        L.orc_set_basis_f64.argtypes = [P, C.c_int, C.c_int, C.c_int]
        _lib = L
    return _lib


def set_threads(t: int) -> None:
    lib().orc_set_threads(int(t))


def threads() -> int:
    return lib().orc_get_threads()


def _n_of(sv) -> int:
    n = int(sv.size).bit_length() - 1
    assert 1 << n == sv.size
    return n


def apply_f64(sv: np.ndarray, ops) -> np.ndarray:
    """Per-gate FP64 oracle, in place on a complex128 vector."""
    assert sv.dtype == np.complex128 and sv.flags.c_contiguous
    arr = op_array(list(ops))
    rc = lib().orc_apply_ops_f64(sv.ctypes.data, _n_of(sv), arr, len(arr))
    assert rc == 0, rc
    return sv


def apply_f32(sv: np.ndarray, ops) -> np.ndarray:
    """Per-gate oracle in float (reference coefficients), in place."""
    assert sv.dtype == np.complex64 and sv.flags.c_contiguous
    arr = op_array(list(ops))
    rc = lib().orc_apply_ops_f32(sv.ctypes.data, _n_of(sv), arr, len(arr))
    assert rc == 0, rc
    return sv


def ref32_apply(x: np.ndarray, n: int, ops) -> np.ndarray:
    """Faithful restatement of the reference algorithm: X <- G X with each
    gate's full 2^n x 2^n operator.  x: complex64 (2^n,) or (2^n, cols)."""
    assert x.dtype == np.complex64 and x.flags.c_contiguous
    cols = 1 if x.ndim == 1 else x.shape[1]
    arr = op_array(list(ops))
    rc = lib().ref32_apply_ops(x.ctypes.data, n, cols, arr, len(arr))
    assert rc == 0, rc
    return x


def ref32_compile(n: int, ops) -> np.ndarray:
    """QCircuit::compile (quantum.cpp:199-210): the circuit matrix, identity
    multiplied by every gate's operator."""
    m = np.eye(1 << n, dtype=np.complex64)
    return ref32_apply(np.ascontiguousarray(m), n, ops)


def ref32_product_state(qubit_amps) -> np.ndarray:
    q = np.ascontiguousarray(np.asarray(qubit_amps, dtype=np.float32).reshape(-1))
    n = q.size // 4
    sv = np.empty(1 << n, dtype=np.complex64)
    lib().ref32_product_state(n, q.ctypes.data, sv.ctypes.data)
    return sv


def ref32_qstate(zero, one) -> np.ndarray:
    z, o = complex(zero), complex(one)
    q = np.array([z.real, z.imag, o.real, o.imag], dtype=np.float32)
    if lib().ref32_qstate_normalize(q.ctypes.data) != 0:
        raise ValueError("Cannot normalize a null state")
    return q


def probs(sv: np.ndarray) -> np.ndarray:
    out = np.empty(sv.size, dtype=np.float64)
    if sv.dtype == np.complex128:
        lib().orc_probs_f64(sv.ctypes.data, _n_of(sv), out.ctypes.data)
    else:
        lib().orc_probs_f32(np.ascontiguousarray(sv, dtype=np.complex64).ctypes.data,
                            _n_of(sv), out.ctypes.data)
    return out


def first_index(p: np.ndarray, u: float) -> int:
    p = np.ascontiguousarray(p, dtype=np.float64)
    return int(lib().orc_first_index(p.ctypes.data, _n_of(p), float(u)))


def qubit_prob_f64(sv: np.ndarray, q: int) -> float:
    sv = np.ascontiguousarray(sv, dtype=np.complex128)
    return float(lib().orc_qubit_prob_f64(sv.ctypes.data, _n_of(sv), q))


def ref32_peek_measure_all(sv: np.ndarray, u: float) -> int:
    sv = np.ascontiguousarray(sv, dtype=np.complex64)
    return int(lib().ref32_peek_measure_all(sv.ctypes.data, _n_of(sv), float(u)))


def ref32_profile_measure_all(sv: np.ndarray, u) -> tuple[np.ndarray, int]:
    sv = np.ascontiguousarray(sv, dtype=np.complex64)
    u = np.ascontiguousarray(np.asarray(u, dtype=np.float32))
    counts = np.zeros(sv.size, dtype=np.uint32)
    un = np.zeros(1, dtype=np.uint32)
    lib().ref32_profile_measure_all(sv.ctypes.data, _n_of(sv), u.size, u.ctypes.data,
                                    counts.ctypes.data, un.ctypes.data)
    return counts, int(un[0])


def ref32_qubit_probability_true(sv: np.ndarray, q: int) -> float:
    sv = np.ascontiguousarray(sv, dtype=np.complex64)
    return float(lib().ref32_qubit_probability_true(sv.ctypes.data, _n_of(sv), q))


BASIS_Z, BASIS_Y, BASIS_X = 0, 1, 2  # QSimulator::Basis (include/quantum.h:489-500)


def ref32_basis_matrix(frm: int, to: int) -> np.ndarray:
    """The 2x2 change of basis set_basis applies to every qubit (float, with
    the reference's fall-through: leaving Y uses X-to-Z)."""
    out = np.zeros(4, dtype=np.complex64)
    lib().ref32_basis_matrix_f(frm, to, out.ctypes.data)
    return out.reshape(2, 2)


def ref32_set_basis(sv: np.ndarray, frm: int, to: int) -> np.ndarray:
    """set_basis as the reference computes it (dense Kronecker operator in
    float), in place on a complex64 vector of at most 12 qubits."""
    assert sv.dtype == np.complex64 and sv.flags.c_contiguous
    rc = lib().ref32_set_basis(sv.ctypes.data, _n_of(sv), frm, to)
    assert rc == 0, rc
    return sv


def set_basis_f64(sv: np.ndarray, frm: int, to: int) -> np.ndarray:
    """The same change of basis in FP64, in place on a complex128 vector."""
    assert sv.dtype == np.complex128 and sv.flags.c_contiguous
    lib().orc_set_basis_f64(sv.ctypes.data, _n_of(sv), frm, to)
    return sv
