"""afquantumsim_gb300 — GB300-native state-vector engine (Python binding).

The engine is ``libaqsg.so`` (CUDA, sm_103a, C ABI declared in
include/aqsg.h).  This module binds it with ctypes for tests, benchmarks and
scripting.  There is no CPU fallback: importing works without a GPU (so the
ABI can be inspected), but every call that needs the device fails loudly
when the library or the GPU is missing.

Gate constructors mirror the reference's gate classes (include/quantum.h):
``X(t)``, ``CX(c, t)``, ``CPhase(c, t, angle)``, ... each returning an
``aqsg_op``; ``Simulator`` mirrors QSimulator's state/measure members.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import _abi
from . import _abi as kinds  # op kind constants: kinds.X, kinds.CPHASE, ...
from ._abi import (C64, C128, EXEC_AUTO, EXEC_PER_GATE, EXEC_TILED, SAMPLE_CLAMP,
                   SAMPLE_REFERENCE, Op, make_op, op_array)

PKG_DIR = Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "_build" / "libaqsg.so"

EXPORTS = [
    "aqsg_version", "aqsg_last_error", "aqsg_init", "aqsg_shutdown",
    "aqsg_set_exec_mode", "aqsg_set_tensor_cores", "aqsg_set_whole_tile_max", "aqsg_synchronize", "aqsg_ctx_after", "aqsg_ctx_stream",
    "aqsg_launch_count",
    "aqsg_state_alloc", "aqsg_state_free", "aqsg_state_info",
    "aqsg_state_set_basis_index", "aqsg_state_set_product", "aqsg_state_upload",
    "aqsg_state_download", "aqsg_state_download_range", "aqsg_state_copy",
    "aqsg_check_ops", "aqsg_apply_ops", "aqsg_qubit_prob", "aqsg_state_prob",
    "aqsg_probs", "aqsg_norm2", "aqsg_sample", "aqsg_sample_seeded",
    "aqsg_collapse_qubit", "aqsg_collapse_all", "aqsg_expect_z", "aqsg_sample_noalloc",
    "aqsg_state_compare", "aqsg_compile", "aqsg_program_info", "aqsg_run_program", "aqsg_program_export",
    "aqsg_program_free", "aqsg_batch_create", "aqsg_batch_update", "aqsg_batch_run",
    "aqsg_batch_info", "aqsg_batch_free",
    "aqsg_server_create", "aqsg_server_submit", "aqsg_server_start", "aqsg_server_poll",
    "aqsg_server_wait_idle", "aqsg_server_get_stats", "aqsg_server_destroy",
    "aqsg_expect_pauli", "aqsg_autotune", "aqsg_batch_tuning", "aqsg_selftest_bounded_wait",
    "aqsg_state_download_async", "aqsg_circuit_to_text", "aqsg_circuit_from_text",
    "aqsg_debug_tile_plan", "aqsg_debug_batch_image", "aqsg_debug_ctx_scratch", "aqsg_batch_traffic",
    "aqsg_noise_trajectory", "aqsg_noise_expect_z", "aqsg_program_plan",
]

_lib = None


class AqsgError(RuntimeError):
    """Error status from libaqsg; `.code` is the aqsg_status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code
        self.msg = msg


# status -> Python exception class (std::out_of_range ~ IndexError, ...)
class OutOfRange(AqsgError, IndexError):
    pass


class InvalidArgument(AqsgError, ValueError):
    pass


class DomainError(AqsgError, ValueError):
    pass


_EXC = {_abi.ERR_OUT_OF_RANGE: OutOfRange, _abi.ERR_INVALID_ARGUMENT: InvalidArgument,
        _abi.ERR_DOMAIN: DomainError}


def load_library(path: os.PathLike | str | None = None) -> C.CDLL:
    """Load libaqsg.so (built in-tree by __graft_entry__.build())."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"libaqsg.so not built at {p}; run __graft_entry__.build()")
    lib = C.CDLL(str(p))
    P, I, U64, D = C.c_void_p, C.c_int, C.c_uint64, C.c_double
    sig = {
        "aqsg_version": ([], I),
        "aqsg_last_error": ([C.c_char_p, C.c_size_t], C.c_size_t),
        "aqsg_init": ([I, C.POINTER(P)], I),
        "aqsg_shutdown": ([P], I),
        "aqsg_set_exec_mode": ([P, I], I),
        "aqsg_set_tensor_cores": ([P, I], I),
        "aqsg_set_whole_tile_max": ([P, I], I),
        "aqsg_synchronize": ([P], I),
        "aqsg_ctx_after": ([P, P], I),
        "aqsg_ctx_stream": ([P, C.POINTER(P)], I),
        "aqsg_launch_count": ([P, C.POINTER(U64)], I),
        "aqsg_state_alloc": ([P, I, I, C.POINTER(P)], I),
        "aqsg_state_free": ([P], I),
        "aqsg_state_info": ([P, C.POINTER(I), C.POINTER(I)], I),
        "aqsg_state_set_basis_index": ([P, U64], I),
        "aqsg_state_set_product": ([P, C.POINTER(C.c_float)], I),
        "aqsg_state_upload": ([P, P, I], I),
        "aqsg_state_download": ([P, P], I),
        "aqsg_state_download_async": ([P, P], I),
        "aqsg_state_download_range": ([P, U64, U64, P], I),
        "aqsg_state_copy": ([P, P], I),
        "aqsg_check_ops": ([I, C.POINTER(Op), I], I),
        "aqsg_apply_ops": ([P, C.POINTER(Op), I, I], I),
        "aqsg_qubit_prob": ([P, I, C.POINTER(D)], I),
        "aqsg_state_prob": ([P, U64, C.POINTER(D)], I),
        "aqsg_probs": ([P, P, I], I),
        "aqsg_norm2": ([P, C.POINTER(D)], I),
        "aqsg_sample": ([P, C.POINTER(D), U64, I, C.POINTER(U64)], I),
        "aqsg_sample_seeded": ([P, U64, U64, I, C.POINTER(U64)], I),
        "aqsg_collapse_qubit": ([P, I, D, C.POINTER(I), C.POINTER(D)], I),
        "aqsg_collapse_all": ([P, D, C.POINTER(U64)], I),
        "aqsg_expect_z": ([P, C.POINTER(D), C.POINTER(D)], I),
        "aqsg_expect_pauli": ([P, C.c_char_p, I, C.POINTER(D)], I),
        "aqsg_selftest_bounded_wait": ([P, C.c_uint32, C.POINTER(I)], I),
        "aqsg_sample_noalloc": ([P, C.POINTER(D), U64, I, C.POINTER(U64)], I),
        "aqsg_state_compare": ([P, P] + [C.POINTER(D)] * 5, I),
        "aqsg_circuit_to_text": ([I, C.POINTER(Op), I, C.c_char_p, C.c_size_t, C.POINTER(C.c_size_t)], I),
        "aqsg_circuit_from_text": ([C.c_char_p, C.POINTER(I), C.POINTER(Op), I, C.POINTER(I),
                                    C.POINTER(D), C.c_size_t, C.POINTER(C.c_size_t)], I),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    if path is None:
        _lib = lib
    return lib


def last_error() -> str:
    lib = load_library()
    buf = C.create_string_buffer(1024)
    lib.aqsg_last_error(buf, len(buf))
    return buf.value.decode()


def _check(rc: int) -> None:
    if rc != 0:
        raise _EXC.get(rc, AqsgError)(rc, last_error())


# ---- gate constructors (reference class names, include/quantum.h:857-1589) ----
# Each returns one aqsg_op.  Keyword `controls` / `control_values` add extra
# controls (the lowering of ControlGate / NControl_Gate).

def Barrier():
    return make_op(kinds.BARRIER)


def X(target, **kw):
    return make_op(kinds.X, (target,), **kw)


def Y(target, **kw):
    return make_op(kinds.Y, (target,), **kw)


def Z(target, **kw):
    return make_op(kinds.Z, (target,), **kw)


def H(target, **kw):
    return make_op(kinds.H, (target,), **kw)


def Phase(target, angle, **kw):
    return make_op(kinds.PHASE, (target,), angle=angle, **kw)


def RotX(target, angle, **kw):
    return make_op(kinds.RX, (target,), angle=angle, **kw)


def RotY(target, angle, **kw):
    return make_op(kinds.RY, (target,), angle=angle, **kw)


def RotZ(target, angle, **kw):
    return make_op(kinds.RZ, (target,), angle=angle, **kw)


def Swap(a, b, **kw):
    return make_op(kinds.SWAP, (a, b), **kw)


def CX(c, t, **kw):
    return make_op(kinds.CX, (c, t), **kw)


def CY(c, t, **kw):
    return make_op(kinds.CY, (c, t), **kw)


def CZ(c, t, **kw):
    return make_op(kinds.CZ, (c, t), **kw)


def CH(c, t, **kw):
    return make_op(kinds.CH, (c, t), **kw)


def CPhase(c, t, angle, **kw):
    return make_op(kinds.CPHASE, (c, t), angle=angle, **kw)


def CSwap(c, a, b, **kw):
    return make_op(kinds.CSWAP, (c, a, b), **kw)


def CRotX(c, t, angle, **kw):
    return make_op(kinds.CRX, (c, t), angle=angle, **kw)


def CRotY(c, t, angle, **kw):
    return make_op(kinds.CRY, (c, t), angle=angle, **kw)


def CRotZ(c, t, angle, **kw):
    return make_op(kinds.CRZ, (c, t), angle=angle, **kw)


def CCNot(a, b, t, **kw):
    return make_op(kinds.CCX, (a, b, t), **kw)


def Or(a, b, t, **kw):
    return make_op(kinds.OR, (a, b, t), **kw)


def Unitary(targets, matrix, **kw):
    return make_op(kinds.UNITARY, tuple(targets), matrix=matrix, **kw)


Not = X          # using Not = X        (quantum.h)
CNot = Xor = CX  # using CNot = CX; using Xor = CX
And = CCNot      # using And = CCNot


def fourier_transform(n: int, swaps: bool = False, angle_dtype=np.float32):
    """QFT gate list of aqs::fourier_transform (src/quantum_algo.cpp:103-114):
    for i = n-1..0: H(i), then CPhase(j, i, pi / 2^(i-j)) for j < i, the angle
    computed in float as the reference does (aqs::pi is a float).  swaps=True
    appends Swap(i, n-1-i) for i < n/2 (the textbook output order)."""
    pi = np.float32(3.14159265358979323846)
    ops = []
    for i in range(n - 1, -1, -1):
        ops.append(H(i))
        for j in range(i):
            ops.append(CPhase(j, i, float(pi / np.float32(1 << (i - j)))))
    if swaps:
        for i in range(n // 2):
            ops.append(Swap(i, n - 1 - i))
    return ops


# ---- engine objects ---------------------------------------------------------------

class Context:
    """An aqsg_ctx: one CUDA device + one stream."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = C.c_void_p()
        _check(self.lib.aqsg_init(device, C.byref(h)))
        self.h = h
        self.device = device

    def set_exec_mode(self, mode: int) -> None:
        _check(self.lib.aqsg_set_exec_mode(self.h, mode))

    def set_tensor_cores(self, enable: bool) -> None:
        _check(self.lib.aqsg_set_tensor_cores(self.h, 1 if enable else 0))

    def set_whole_tile_max(self, qubits: int) -> None:
        """aqsg_set_whole_tile_max: registers of at most `qubits` qubits run
        as one whole-register tile, larger ones in streaming tiles (0: the
        default, 14 qubits c64 / 13 c128)."""
        _check(self.lib.aqsg_set_whole_tile_max(self.h, qubits))

    def synchronize(self) -> None:
        _check(self.lib.aqsg_synchronize(self.h))

    def after(self, other: "Context") -> None:
        """aqsg_ctx_after: work queued here from now on waits for the work
        queued on `other` so far (no host blocking)."""
        _check(self.lib.aqsg_ctx_after(self.h, other.h))

    def stream_handle(self) -> int:
        """The context's cudaStream_t as an integer."""
        v = C.c_void_p()
        _check(self.lib.aqsg_ctx_stream(self.h, C.byref(v)))
        return v.value or 0

    def scratch_bytes(self) -> list:
        """aqsg_debug_ctx_scratch: bytes held in each of the context's
        grown-on-demand device scratch buffers (a testing aid)."""
        lib = load_library()
        f = lib.aqsg_debug_ctx_scratch
        f.argtypes = [C.c_void_p, C.POINTER(C.c_size_t), C.c_int, C.POINTER(C.c_int)]
        f.restype = C.c_int
        buf, cnt = (C.c_size_t * 8)(), C.c_int()
        _check(f(self.h, buf, 8, C.byref(cnt)))
        return list(buf[:cnt.value])

    def launch_count(self) -> int:
        v = C.c_uint64()
        _check(self.lib.aqsg_launch_count(self.h, C.byref(v)))
        return v.value

    def close(self) -> None:
        if self.h:
            _check(self.lib.aqsg_shutdown(self.h))
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class State:
    """An n-qubit register on the device (aqsg_state)."""

    def __init__(self, ctx: Context, n: int, dtype: int = C64):
        self.ctx, self.lib = ctx, ctx.lib
        self.n, self.dtype = n, dtype
        h = C.c_void_p()
        _check(self.lib.aqsg_state_alloc(ctx.h, n, dtype, C.byref(h)))
        self.h = h

    @property
    def np_dtype(self):
        return np.complex64 if self.dtype == C64 else np.complex128

    def free(self) -> None:
        if self.h:
            _check(self.lib.aqsg_state_free(self.h))
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.free()

    # preparation
    def set_basis(self, k: int) -> "State":
        _check(self.lib.aqsg_state_set_basis_index(self.h, k))
        return self

    def set_product(self, qubit_amps) -> "State":
        a = np.ascontiguousarray(np.asarray(qubit_amps, dtype=np.float32).reshape(-1))
        _check(self.lib.aqsg_state_set_product(self.h, a.ctypes.data_as(C.POINTER(C.c_float))))
        return self

    def upload(self, sv, normalize: bool = False) -> "State":
        a = np.ascontiguousarray(np.asarray(sv, dtype=self.np_dtype))
        assert a.size == 1 << self.n
        _check(self.lib.aqsg_state_upload(self.h, a.ctypes.data, 1 if normalize else 0))
        self.ctx.synchronize()
        return self

    def upload_ptr(self, ptr: int, normalize: bool = False) -> None:
        _check(self.lib.aqsg_state_upload(self.h, ptr, 1 if normalize else 0))

    def download(self, out=None) -> np.ndarray:
        if out is None:
            out = np.empty(1 << self.n, dtype=self.np_dtype)
        _check(self.lib.aqsg_state_download(self.h, out.ctypes.data))
        return out

    def download_ptr(self, ptr: int) -> None:
        _check(self.lib.aqsg_state_download(self.h, ptr))

    def download_async_ptr(self, ptr: int) -> None:
        """Enqueue the copy to host memory at ptr; complete after the
        context's next synchronize()."""
        _check(self.lib.aqsg_state_download_async(self.h, ptr))

    def compare(self, other: "State"):
        """(max |a - b|, <a|b>, |a|^2, |b|^2) in FP64, on the device."""
        v = [C.c_double() for _ in range(5)]
        _check(self.lib.aqsg_state_compare(self.h, other.h, *[C.byref(x) for x in v]))
        return v[0].value, complex(v[1].value, v[2].value), v[3].value, v[4].value

    def copy_from(self, other: "State") -> None:
        _check(self.lib.aqsg_state_copy(self.h, other.h))

    # simulation
    def apply(self, ops, mode: int = -1) -> None:
        arr = ops if isinstance(ops, C.Array) else op_array(list(ops))
        _check(self.lib.aqsg_apply_ops(self.h, arr, len(arr), mode))

    # measurement
    def qubit_prob(self, q: int) -> float:
        v = C.c_double()
        _check(self.lib.aqsg_qubit_prob(self.h, q, C.byref(v)))
        return v.value

    def state_prob(self, k: int) -> float:
        v = C.c_double()
        _check(self.lib.aqsg_state_prob(self.h, k, C.byref(v)))
        return v.value

    def probs(self, dtype=np.float64) -> np.ndarray:
        out = np.empty(1 << self.n, dtype=dtype)
        _check(self.lib.aqsg_probs(self.h, out.ctypes.data, 1 if dtype == np.float64 else 0))
        return out

    def norm2(self) -> float:
        v = C.c_double()
        _check(self.lib.aqsg_norm2(self.h, C.byref(v)))
        return v.value

    def sample(self, u, rule: int = SAMPLE_REFERENCE) -> np.ndarray:
        u = np.ascontiguousarray(np.asarray(u, dtype=np.float64).reshape(-1))
        out = np.empty(u.size, dtype=np.uint64)
        _check(self.lib.aqsg_sample(self.h, u.ctypes.data_as(C.POINTER(C.c_double)), u.size, rule,
                                    out.ctypes.data_as(C.POINTER(C.c_uint64))))
        return out

    def sample_noalloc(self, u, rule: int = SAMPLE_REFERENCE) -> np.ndarray:
        """aqsg_sample_noalloc: as sample(), with the library's static device
        scratch instead of allocated buffers (for callers that cannot allocate
        device memory while running)."""
        u = np.ascontiguousarray(np.asarray(u, dtype=np.float64).reshape(-1))
        out = np.empty(u.size, dtype=np.uint64)
        _check(self.lib.aqsg_sample_noalloc(self.h, u.ctypes.data_as(C.POINTER(C.c_double)), u.size,
                                            rule, out.ctypes.data_as(C.POINTER(C.c_uint64))))
        return out

    def sample_seeded(self, seed: int, count: int, rule: int = SAMPLE_REFERENCE) -> np.ndarray:
        out = np.empty(count, dtype=np.uint64)
        _check(self.lib.aqsg_sample_seeded(self.h, seed, count, rule,
                                           out.ctypes.data_as(C.POINTER(C.c_uint64))))
        return out

    def collapse_qubit(self, q: int, u: float):
        o, p = C.c_int(), C.c_double()
        _check(self.lib.aqsg_collapse_qubit(self.h, q, u, C.byref(o), C.byref(p)))
        return o.value, p.value

    def collapse_all(self, u: float) -> int:
        k = C.c_uint64()
        _check(self.lib.aqsg_collapse_all(self.h, u, C.byref(k)))
        return k.value

    def expect_z(self):
        z = np.empty(self.n, dtype=np.float64)
        zz = np.empty(max(self.n - 1, 1), dtype=np.float64)
        _check(self.lib.aqsg_expect_z(self.h, z.ctypes.data_as(C.POINTER(C.c_double)),
                                      zz.ctypes.data_as(C.POINTER(C.c_double))))
        return z, zz[: self.n - 1]

    def expect_pauli(self, strings) -> np.ndarray:
        """<psi|P|psi> (complex128) for each Pauli string (n letters from
        i/x/y/z, letter j on qubit j)."""
        strings = list(strings)
        for s in strings:
            if len(s) != self.n:
                raise InvalidArgument(-2, f"Pauli string {s!r} does not have {self.n} letters")
        out = np.empty(2 * max(len(strings), 1), dtype=np.float64)
        _check(self.lib.aqsg_expect_pauli(self.h, "".join(strings).encode(), len(strings),
                                          out.ctypes.data_as(C.POINTER(C.c_double))))
        return out[0::2][: len(strings)] + 1j * out[1::2][: len(strings)]


def circuit_to_text(n: int, ops) -> str:
    """aqsg_circuit_to_text: the circuit as text (the reference's gate
    representation with parameters, a "n;" header and "~q" zero-controls)."""
    lib = load_library()
    arr = op_array(list(ops)) if not isinstance(ops, C.Array) else ops
    need = C.c_size_t()
    _check(lib.aqsg_circuit_to_text(n, arr, len(arr), None, 0, C.byref(need)))
    buf = C.create_string_buffer(need.value)
    _check(lib.aqsg_circuit_to_text(n, arr, len(arr), buf, need.value, C.byref(need)))
    return buf.value.decode("utf-8")


def circuit_from_text(text: str):
    """aqsg_circuit_from_text: (n, ops) with the ops as an aqsg_op array
    (unitary matrices kept alive by the array)."""
    lib = load_library()
    raw = text.encode("utf-8")
    n, cnt, nd = C.c_int(), C.c_int(), C.c_size_t()
    _check(lib.aqsg_circuit_from_text(raw, C.byref(n), None, 0, C.byref(cnt), None, 0, C.byref(nd)))
    arr = (Op * max(cnt.value, 1))()
    mats = (C.c_double * max(nd.value, 1))()
    _check(lib.aqsg_circuit_from_text(raw, C.byref(n), arr, cnt.value, C.byref(cnt), mats, nd.value,
                                      C.byref(nd)))
    out = (Op * cnt.value).from_buffer(arr)
    out._keep = (arr, mats)
    return n.value, out


class TilePass(C.Structure):
    """struct aqsg_tile_pass (aqsg_debug.h)"""
    _fields_ = [("m", C.c_int32), ("L", C.c_int32), ("first", C.c_int32), ("count", C.c_int32),
                ("tbits", C.c_int32 * 16), ("tc", C.c_int32), ("matk", C.c_int32), ("tc_blob", C.c_uint32),
                ("tc_bytes", C.c_uint32)]


def debug_tile_plan(n: int, ops, dtype: int = C64, fuse_qubits: int = 0, whole_tile_max: int = 0,
                    tensor_cores: bool = False):
    """aqsg_debug_tile_plan: (passes, table bytes, pool bytes) of the tile
    plan the engine would run for ops (a testing aid); whole_tile_max and
    tensor_cores as set by Context.set_whole_tile_max / set_tensor_cores
    (defaults: the whole-tile default, the CUDA-core form; tensor_cores=2:
    the batched engine's form, fused permutations on the tensor cores too)."""
    lib = load_library()
    f = lib.aqsg_debug_tile_plan
    f.argtypes = [C.c_int, C.c_int, C.POINTER(Op), C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(TilePass), C.c_int,
                  C.POINTER(C.c_int), C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t), C.c_void_p, C.c_size_t,
                  C.POINTER(C.c_size_t)]
    f.restype = C.c_int
    arr = op_array(list(ops)) if not isinstance(ops, C.Array) else ops
    npass, tb, pb = C.c_int(), C.c_size_t(), C.c_size_t()
    tc = int(tensor_cores)  # False / True, or 2: the batched engine's form
    _check(f(n, dtype, arr, len(arr), fuse_qubits, whole_tile_max, tc, None, 0, C.byref(npass), None, 0,
             C.byref(tb), None, 0, C.byref(pb)))
    passes = (TilePass * max(npass.value, 1))()
    table = C.create_string_buffer(max(tb.value, 1))
    pool = C.create_string_buffer(max(pb.value, 1))
    _check(f(n, dtype, arr, len(arr), fuse_qubits, whole_tile_max, tc, passes, npass.value, C.byref(npass),
             table, tb.value, C.byref(tb), pool, pb.value, C.byref(pb)))
    return list(passes[:npass.value]), table.raw[:tb.value], pool.raw[:pb.value]


def debug_batch_image(circuits, fuse=None, tc=None, update=None) -> bytes:
    """aqsg_debug_batch_image: the plan image a batch of [(n, ops), ...]
    uploads, with the fusion width and tensor-core choice of each register
    of more than 14 qubits given (fuse, tc: one entry per such register), or
    the image after an update with the circuits `update` (a testing aid)."""
    lib = load_library()
    f = lib.aqsg_debug_batch_image
    f.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t,
                  C.POINTER(C.c_size_t)]
    f.restype = C.c_int
    arr, _ = Batch._encode(circuits)
    upd = Batch._encode(update)[0] if update is not None else None
    fz = (C.c_int * max(len(fuse), 1))(*fuse) if fuse is not None else None
    tz = (C.c_int * max(len(tc), 1))(*tc) if tc is not None else None
    size = C.c_size_t()
    _check(f(arr, len(arr), fz, tz, upd, None, 0, C.byref(size)))
    buf = C.create_string_buffer(max(size.value, 1))
    _check(f(arr, len(arr), fz, tz, upd, buf, size.value, C.byref(size)))
    return buf.raw[:size.value]


def check_ops(n: int, ops) -> None:
    lib = load_library()
    arr = op_array(list(ops))
    _check(lib.aqsg_check_ops(n, arr, len(arr)))


def qstate(zero, one):
    """Normalised single-qubit amplitudes as QState::force_normalize does
    (quantum.cpp:145-157, float arithmetic).  Returns 4 floats."""
    z, o = complex(zero), complex(one)
    q = np.array([z.real, z.imag, o.real, o.imag], dtype=np.float32)
    mag2 = np.float32(q[0] * q[0]) + np.float32(q[1] * q[1])
    mag2 = np.float32(mag2 + np.float32(q[2] * q[2]))
    mag2 = np.float32(mag2 + np.float32(q[3] * q[3]))
    if mag2 == 0:
        raise ValueError("Cannot normalize a null state")
    mag = np.float32(np.sqrt(mag2))
    return (q / mag).astype(np.float32)


# ---- compiled programs (gate fusion) ----------------------------------------------

def _bind_programs(lib):
    P, I = C.c_void_p, C.c_int
    lib.aqsg_compile.argtypes = [I, I, C.POINTER(Op), I, I, C.POINTER(P)]
    lib.aqsg_program_info.argtypes = [P, C.POINTER(I), C.POINTER(I)]
    lib.aqsg_run_program.argtypes = [P, P, I]
    lib.aqsg_program_export.argtypes = [P, C.POINTER(Op), I, C.POINTER(I)]
    lib.aqsg_program_free.argtypes = [P]
    lib.aqsg_program_plan.argtypes = [P, I, C.POINTER(I), C.POINTER(I), C.POINTER(C.c_uint64)]
    for f in ("aqsg_compile", "aqsg_program_info", "aqsg_run_program", "aqsg_program_export",
              "aqsg_program_free", "aqsg_program_plan"):
        getattr(lib, f).restype = I


class Program:
    """aqsg_compile: ops fused into dense unitaries on <= max_qubits qubits."""

    def __init__(self, n: int, ops, dtype: int = C64, max_qubits: int = 5):
        self.lib = load_library()
        _bind_programs(self.lib)
        arr = op_array(list(ops))
        h = C.c_void_p()
        _check(self.lib.aqsg_compile(n, dtype, arr, len(arr), max_qubits, C.byref(h)))
        self.h, self.n, self.dtype = h, n, dtype

    def info(self):
        f, s = C.c_int(), C.c_int()
        _check(self.lib.aqsg_program_info(self.h, C.byref(f), C.byref(s)))
        return f.value, s.value

    def plan(self, tensor_cores: bool = True):
        """aqsg_program_plan: {passes, tc_passes, hbm_bytes} of a tiled run."""
        p, t, b = C.c_int(), C.c_int(), C.c_uint64()
        _check(self.lib.aqsg_program_plan(self.h, 1 if tensor_cores else 0, C.byref(p), C.byref(t), C.byref(b)))
        return {"passes": p.value, "tc_passes": t.value, "hbm_bytes": b.value}

    def export(self):
        """The fused ops as aqsg_op structs (matrices point into the program)."""
        cnt = C.c_int()
        _check(self.lib.aqsg_program_export(self.h, None, 0, C.byref(cnt)))
        arr = (Op * cnt.value)()
        _check(self.lib.aqsg_program_export(self.h, arr, cnt.value, C.byref(cnt)))
        arr._prog = self  # keep the program (and its matrices) alive
        return arr

    def run(self, state: "State", mode: int = -1) -> None:
        _check(self.lib.aqsg_run_program(state.h, self.h, mode))

    def free(self) -> None:
        if self.h:
            _check(self.lib.aqsg_program_free(self.h))
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


# ---- batched engine ------------------------------------------------------------

class _Circuit(C.Structure):
    _fields_ = [("n", C.c_int32), ("count", C.c_int32), ("ops", C.POINTER(Op))]


def _bind_batch(lib):
    P, I, D = C.c_void_p, C.c_int, C.POINTER(C.c_double)
    lib.aqsg_batch_create.argtypes = [P, C.POINTER(_Circuit), I, C.POINTER(P)]
    lib.aqsg_batch_update.argtypes = [P, C.POINTER(_Circuit)]
    lib.aqsg_batch_run.argtypes = [P, D, D]
    lib.aqsg_batch_info.argtypes = [P, C.POINTER(I), C.POINTER(I), C.POINTER(I)]
    lib.aqsg_batch_free.argtypes = [P]
    lib.aqsg_batch_tuning.argtypes = [P, C.POINTER(I), C.POINTER(I)]
    lib.aqsg_batch_traffic.argtypes = [P, C.POINTER(C.c_uint64)]
    for f in ("aqsg_batch_create", "aqsg_batch_update", "aqsg_batch_run", "aqsg_batch_info",
              "aqsg_batch_free", "aqsg_batch_tuning", "aqsg_batch_traffic"):
        getattr(lib, f).restype = I


class Batch:
    """aqsg_batch: independent circuits [(n, ops), ...] run from |0...0> to
    <Z_q> and <Z_q Z_q+1>, captured once as a CUDA graph."""

    def __init__(self, ctx: Context, circuits):
        self.ctx, self.lib = ctx, ctx.lib
        _bind_batch(self.lib)
        arr, keep = self._encode(circuits)
        h = C.c_void_p()
        _check(self.lib.aqsg_batch_create(ctx.h, arr, len(arr), C.byref(h)))
        self.h = h
        self.ns = [n for n, _ in circuits]

    @staticmethod
    def _encode(circuits):
        arr = (_Circuit * len(circuits))()
        keep = []
        for i, (n, ops) in enumerate(circuits):
            if isinstance(ops, np.ndarray):  # structured array in aqsg_op layout
                a = np.ascontiguousarray(ops)
                ptr = C.cast(a.ctypes.data, C.POINTER(Op))
            else:
                a = ops if isinstance(ops, C.Array) else op_array(list(ops))
                ptr = C.cast(a, C.POINTER(Op))
            keep.append(a)
            arr[i].n, arr[i].count, arr[i].ops = n, len(a), ptr
        arr._keep = keep
        return arr, keep

    def update(self, circuits) -> None:
        arr, keep = self._encode(circuits)
        _check(self.lib.aqsg_batch_update(self.h, arr))

    def run(self):
        """Returns (z, zz): lists of per-circuit numpy arrays."""
        nz = sum(self.ns)
        z = np.empty(nz, dtype=np.float64)
        zz = np.empty(max(nz - len(self.ns), 1), dtype=np.float64)
        _check(self.lib.aqsg_batch_run(self.h, z.ctypes.data_as(C.POINTER(C.c_double)),
                                       zz.ctypes.data_as(C.POINTER(C.c_double))))
        zs, zzs, a, b = [], [], 0, 0
        for n in self.ns:
            zs.append(z[a:a + n])
            zzs.append(zz[b:b + n - 1])
            a, b = a + n, b + n - 1
        return zs, zzs

    def info(self):
        s, l, k = C.c_int(), C.c_int(), C.c_int()
        _check(self.lib.aqsg_batch_info(self.h, C.byref(s), C.byref(l), C.byref(k)))
        f, t = (C.c_int * max(l.value, 1))(), (C.c_int * max(l.value, 1))()
        _check(self.lib.aqsg_batch_tuning(self.h, f, t))
        hb = C.c_uint64()
        _check(self.lib.aqsg_batch_traffic(self.h, C.byref(hb)))
        return {"small": s.value, "large": l.value, "kernels": k.value,
                "fuse_qubits": list(f[:l.value]), "tensor_cores": list(t[:l.value]), "hbm_bytes": hb.value}

    def free(self) -> None:
        if self.h:
            _check(self.lib.aqsg_batch_free(self.h))
            self.h = None


# ---- serving runtime -----------------------------------------------------------

class Noise(C.Structure):
    """struct aqsg_noise: X, Y, Z probabilities per touched qubit after
    one-qubit gates (p1) and after gates on several qubits (p2)."""
    _fields_ = [("p1", C.c_float * 3), ("p2", C.c_float * 3)]

    @classmethod
    def pauli(cls, p1=(0.0, 0.0, 0.0), p2=(0.0, 0.0, 0.0)) -> "Noise":
        return cls((C.c_float * 3)(*p1), (C.c_float * 3)(*p2))

    @classmethod
    def depolarizing(cls, p1: float, p2: float) -> "Noise":
        """Depolarizing noise of strength p1 / p2 on each touched qubit."""
        return cls.pauli((p1 / 3,) * 3, (p2 / 3,) * 3)


def _bind_noise(lib):
    P, I, U64, D = C.c_void_p, C.c_int, C.c_uint64, C.POINTER(C.c_double)
    lib.aqsg_noise_trajectory.argtypes = [I, C.POINTER(Op), I, C.POINTER(Noise), U64, U64, C.POINTER(Op), I,
                                          C.POINTER(I)]
    lib.aqsg_noise_expect_z.argtypes = [P, I, C.POINTER(Op), I, C.POINTER(Noise), U64, I, D, D, D, D]
    lib.aqsg_noise_trajectory.restype = I
    lib.aqsg_noise_expect_z.restype = I


def noise_trajectory(n: int, ops, noise: Noise, seed: int, trajectory: int):
    """aqsg_noise_trajectory: the ops of one trajectory of the noisy circuit
    (the sampled Paulis inserted after the gates they follow)."""
    lib = load_library()
    _bind_noise(lib)
    arr = op_array(list(ops)) if not isinstance(ops, C.Array) else ops
    cnt = C.c_int()
    _check(lib.aqsg_noise_trajectory(n, arr, len(arr), C.byref(noise), seed, trajectory, None, 0, C.byref(cnt)))
    out = (Op * max(cnt.value, 1))()
    _check(lib.aqsg_noise_trajectory(n, arr, len(arr), C.byref(noise), seed, trajectory, out, cnt.value,
                                      C.byref(cnt)))
    res = (Op * cnt.value).from_buffer(out)
    res._keep = (arr, out)
    return res


def noisy_expect_z(ctx: "Context", n: int, ops, noise: Noise, seed: int, trajectories: int):
    """aqsg_noise_expect_z: (<Z_q>, <Z_q Z_q+1>, their standard errors) of
    the noisy circuit from |0...0>, estimated by `trajectories` trajectories
    run as one batch."""
    lib = load_library()
    _bind_noise(lib)
    arr = op_array(list(ops)) if not isinstance(ops, C.Array) else ops
    z, zz = np.zeros(n), np.zeros(n - 1)
    ze, zze = np.zeros(n), np.zeros(n - 1)
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    _check(lib.aqsg_noise_expect_z(ctx.h, n, arr, len(arr), C.byref(noise), seed, trajectories, dp(z), dp(zz),
                                   dp(ze), dp(zze)))
    return z, zz, ze, zze


class ServerDone(C.Structure):
    """struct aqsg_server_done."""
    _fields_ = [("ticket", C.c_uint64), ("status", C.c_int32), ("n", C.c_int32),
                ("lane", C.c_int32), ("fused_ops", C.c_int32), ("arrival_s", C.c_double),
                ("admit_s", C.c_double), ("done_s", C.c_double)]


class ServerStats(C.Structure):
    """struct aqsg_server_stats."""
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64),
                ("slab_bytes", C.c_uint64), ("peak_bytes", C.c_uint64),
                ("peak_running", C.c_int32), ("lanes", C.c_int32), ("launches", C.c_uint64),
                ("hbm_bytes", C.c_uint64)]


def _bind_server(lib):
    P, I, U64, U32, D = C.c_void_p, C.c_int, C.c_uint64, C.c_uint32, C.c_double
    lib.aqsg_server_create.argtypes = [I, I, U64, I, I, U32, C.POINTER(P)]
    lib.aqsg_server_submit.argtypes = [P, I, C.POINTER(Op), I, I, U32, U64, D,
                                       C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
    lib.aqsg_server_start.argtypes = [P]
    lib.aqsg_server_poll.argtypes = [P, C.POINTER(ServerDone), I, C.POINTER(I)]
    lib.aqsg_server_wait_idle.argtypes = [P, D]
    lib.aqsg_server_get_stats.argtypes = [P, C.POINTER(ServerStats)]
    lib.aqsg_server_destroy.argtypes = [P]
    for f in ("aqsg_server_create", "aqsg_server_submit", "aqsg_server_start", "aqsg_server_poll",
              "aqsg_server_wait_idle", "aqsg_server_get_stats", "aqsg_server_destroy"):
        getattr(lib, f).restype = I


class Server:
    """aqsg_server: a stream of independent requests (circuit from |0...0>,
    then `shots` seeded measure-all draws) admitted by arrival time and HBM
    onto concurrent lanes over one register slab."""

    def __init__(self, device: int = 0, dtype: int = C64, hbm_budget_bytes: int = 8 << 30,
                 lanes: int = 8, max_qubits: int = 28, max_shots: int = 1024):
        self.lib = load_library()
        _bind_server(self.lib)
        h = C.c_void_p()
        _check(self.lib.aqsg_server_create(device, dtype, hbm_budget_bytes, lanes, max_qubits,
                                           max_shots, C.byref(h)))
        self.h = h
        self._outs = {}  # ticket -> (outcome array, op array kept alive until submit returns)

    def submit(self, n: int, ops, shots: int = 1024, seed: int = 0, arrival_s: float = -1.0,
               fuse_qubits: int = 0) -> int:
        if isinstance(ops, np.ndarray):
            a = np.ascontiguousarray(ops)
            ptr, count = C.cast(a.ctypes.data, C.POINTER(Op)), len(a)
        else:
            a = ops if isinstance(ops, C.Array) else op_array(list(ops))
            ptr, count = C.cast(a, C.POINTER(Op)), len(a)
        out = np.zeros(max(shots, 1), dtype=np.uint64)
        t = C.c_uint64()
        _check(self.lib.aqsg_server_submit(self.h, n, ptr, count, fuse_qubits, shots, seed, arrival_s,
                                           out.ctypes.data_as(C.POINTER(C.c_uint64)), C.byref(t)))
        self._outs[t.value] = out[:shots]
        return t.value

    def submit_text(self, text: str, shots: int = 1024, seed: int = 0, arrival_s: float = -1.0,
                    fuse_qubits: int = 0) -> int:
        """Submit a request written as circuit text (aqsg_circuit_from_text)."""
        n, ops = circuit_from_text(text)
        return self.submit(n, ops, shots, seed, arrival_s, fuse_qubits)

    def start(self) -> None:
        _check(self.lib.aqsg_server_start(self.h))

    def poll(self, capacity: int = 4096):
        """Finished requests: list of dicts (ticket, status, n, lane, fused_ops,
        arrival_s, admit_s, done_s, outcomes)."""
        buf = (ServerDone * capacity)()
        k = C.c_int()
        _check(self.lib.aqsg_server_poll(self.h, buf, capacity, C.byref(k)))
        out = []
        for d in buf[:k.value]:
            rec = {f: getattr(d, f) for f, _ in ServerDone._fields_}
            rec["outcomes"] = self._outs.pop(d.ticket)
            out.append(rec)
        return out

    def wait_idle(self, timeout_s: float = 600.0) -> None:
        _check(self.lib.aqsg_server_wait_idle(self.h, timeout_s))

    def stats(self) -> dict:
        s = ServerStats()
        _check(self.lib.aqsg_server_get_stats(self.h, C.byref(s)))
        return {f: getattr(s, f) for f, _ in ServerStats._fields_}

    def close(self) -> None:
        if self.h:
            _check(self.lib.aqsg_server_destroy(self.h))
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- autotuner -----------------------------------------------------------------

class TuneEntry(C.Structure):
    """struct aqsg_tune_entry."""
    _fields_ = [("exec_mode", C.c_int32), ("fuse_qubits", C.c_int32), ("tensor_cores", C.c_int32),
                ("ops", C.c_int32), ("ms", C.c_double), ("tile_bits", C.c_int32), ("reserved", C.c_int32)]


def autotune(ctx: Context, n: int, ops, dtype: int = C64, reps: int = 2, all_timings: bool = True):
    """aqsg_autotune: returns (best, [every timing]) as dicts."""
    lib = ctx.lib
    lib.aqsg_autotune.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(Op), C.c_int, C.c_int,
                                  C.POINTER(TuneEntry), C.POINTER(TuneEntry), C.c_int, C.POINTER(C.c_int)]
    lib.aqsg_autotune.restype = C.c_int
    if isinstance(ops, np.ndarray):
        a = np.ascontiguousarray(ops)
        ptr, count = C.cast(a.ctypes.data, C.POINTER(Op)), len(a)
    else:
        a = ops if isinstance(ops, C.Array) else op_array(list(ops))
        ptr, count = C.cast(a, C.POINTER(Op)), len(a)
    best = TuneEntry()
    buf = (TuneEntry * 32)()
    k = C.c_int()
    _check(lib.aqsg_autotune(ctx.h, n, dtype, ptr, count, reps, C.byref(best), buf if all_timings else None,
                             32, C.byref(k)))
    conv = lambda e: {f: getattr(e, f) for f, _ in TuneEntry._fields_}
    return conv(best), [conv(e) for e in buf[:k.value]]
