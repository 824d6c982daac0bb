"""Helpers shared by the tests: golden-vector loading and op conversion."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

import afquantumsim_gb300 as aq
from afquantumsim_gb300 import _abi

GOLDEN = Path(__file__).resolve().parent / "golden" / "reference_kat.json"

_KIND = {"X": _abi.X, "Y": _abi.Y, "Z": _abi.Z, "H": _abi.H, "Phase": _abi.PHASE,
         "Swap": _abi.SWAP, "RotX": _abi.RX, "RotY": _abi.RY, "RotZ": _abi.RZ,
         "CX": _abi.CX, "CY": _abi.CY, "CZ": _abi.CZ, "CH": _abi.CH,
         "CPhase": _abi.CPHASE, "CSwap": _abi.CSWAP, "CRotX": _abi.CRX,
         "CRotY": _abi.CRY, "CRotZ": _abi.CRZ, "CCNot": _abi.CCX, "Or": _abi.OR}


def load_cases():
    return json.loads(GOLDEN.read_text())["cases"]


def to_ops(gates):
    return [_abi.make_op(_KIND[d["g"]], d["q"], angle=d.get("a", 0.0),
                         controls=d.get("c", ()), control_values=d.get("cv"))
            for d in gates]


def init_amps(init):
    """Per-qubit amplitudes after QState::force_normalize (float)."""
    from oracle import oracle
    return np.concatenate([oracle.ref32_qstate(complex(q[0], q[1]), complex(q[2], q[3]))
                           for q in init]).astype(np.float32)


def fequal(a: float, b: float, diff: float) -> bool:
    """tests.cpp:19-22: relative tolerance (an expected 0 must be exact)."""
    return abs(a - b) <= max(abs(a), abs(b)) * diff


def amp_ok(v: complex, re: float, im: float, cmp: str, tol: float) -> bool:
    if cmp == "exact":
        return v.real == re and v.imag == im
    return fequal(v.real, re, tol) and fequal(v.imag, im, tol)


def random_state(n: int, seed: int, dtype=np.complex128) -> np.ndarray:
    rng = np.random.default_rng(seed)
    v = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    v /= np.linalg.norm(v)
    return v.astype(dtype)


def random_circuit(n: int, depth: int, seed: int, kinds=None):
    """Seeded random circuit over every gate kind (with extra controls)."""
    rng = np.random.default_rng(seed)
    ops = []
    all_kinds = kinds or ["X", "Y", "Z", "H", "Phase", "RotX", "RotY", "RotZ", "Swap",
                          "CX", "CY", "CZ", "CH", "CPhase", "CSwap", "CRotX", "CRotY",
                          "CRotZ", "CCNot", "Or", "U2", "U3", "CU2"]
    for _ in range(depth):
        k = all_kinds[rng.integers(len(all_kinds))]
        if k.startswith("U") or k.startswith("CU"):
            kk = int(k[-1])
            if kk + (1 if k.startswith("C") else 0) > n:
                continue
            qs = rng.choice(n, size=kk + (1 if k.startswith("C") else 0), replace=False)
            m = np.linalg.qr(rng.standard_normal((1 << kk, 1 << kk))
                             + 1j * rng.standard_normal((1 << kk, 1 << kk)))[0]
            if k.startswith("C"):
                ops.append(aq.Unitary(qs[1:], m, controls=[qs[0]],
                                      control_values=int(rng.integers(2))))
            else:
                ops.append(aq.Unitary(qs, m))
            continue
        kind = _KIND[k]
        ar = _abi.ARITY[kind]
        if ar > n:
            continue
        qs = [int(x) for x in rng.choice(n, size=ar, replace=False)]
        angle = float(np.float32(rng.uniform(-np.pi, np.pi)))
        extra = []
        free = [q for q in range(n) if q not in qs]
        if free and rng.random() < 0.25:
            extra = [int(x) for x in rng.choice(free, size=min(len(free), int(rng.integers(1, 3))),
                                                replace=False)]
        cv = int(rng.integers(1 << len(extra))) if extra else None
        ops.append(_abi.make_op(kind, qs, angle=angle, controls=extra, control_values=cv))
    return ops
