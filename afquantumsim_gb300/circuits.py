"""Seeded synthetic workload circuits (lists of aqsg_op).

* `qft`            — aqs::fourier_transform(n) (src/quantum_algo.cpp:103-114),
                     optionally followed by Swap(i, n-1-i): the 24/28/30-qubit
                     plain-kernel workload.
* `plain_layers`   — H on every qubit, then layers of one seeded random
                     RotX/RotY/RotZ per qubit (angle uniform in [0, 2 pi)) and a
                     CX chain (i, i+1): the 12-qubit plain-method workload.
* `brickwork`      — depth-d brick-work: a Haar-random SU(2) on every qubit
                     (a normalised complex-Gaussian column (a, b) completed to
                     [[a, -conj b], [b, conj a]]), then CZ on (2i, 2i+1) in even
                     layers and (2i+1, 2i+2) in odd layers.  The SU(2) is given
                     either as its RotZ.RotY.RotZ Euler form (gates the
                     reference has) or as a 1-qubit unitary.
* `vqe_ansatz`     — hardware-efficient ansatz: per layer RotY and RotZ on every
                     qubit, then a CX ring (i, (i+1) mod n).

Angles are float32, as the reference's gate classes store them.
"""
from __future__ import annotations

import numpy as np

from . import CPhase, CX, CZ, H, RotX, RotY, RotZ, Swap, Unitary, fourier_transform


def qft(n: int, swaps: bool = True):
    return fourier_transform(n, swaps=swaps)


def plain_layers(n: int = 12, layers: int = 10, seed: int = 1):
    rng = np.random.default_rng(seed)
    ops = [H(q) for q in range(n)]
    rot = (RotX, RotY, RotZ)
    for _ in range(layers):
        for q in range(n):
            ops.append(rot[int(rng.integers(3))](q, float(np.float32(rng.uniform(0, 2 * np.pi)))))
        ops += [CX(i, i + 1) for i in range(n - 1)]
    return ops


def haar_su2(rng) -> np.ndarray:
    v = rng.standard_normal(2) + 1j * rng.standard_normal(2)
    a, b = v / np.linalg.norm(v)
    return np.array([[a, -np.conj(b)], [b, np.conj(a)]])


def euler_zyz(u: np.ndarray):
    """Angles (phi, theta, lam) with u = RotZ(phi) RotY(theta) RotZ(lam) for
    u = [[a, -conj b], [b, conj a]] in SU(2) (RotZ(x) = diag(e^-ix/2, e^ix/2),
    RotY(x) = [[c, -s], [s, c]] with c, s of x/2)."""
    a, b = u[0, 0], u[1, 0]
    theta = 2 * np.arctan2(abs(b), abs(a))
    phi = np.angle(b) - np.angle(a)
    lam = -np.angle(a) - np.angle(b)
    return phi, theta, lam


def brickwork(n: int, depth: int, seed: int = 4, form: str = "euler"):
    rng = np.random.default_rng(seed)
    ops = []
    for layer in range(depth):
        for q in range(n):
            u = haar_su2(rng)
            if form == "euler":
                phi, theta, lam = (float(np.float32(x)) for x in euler_zyz(u))
                # matrix product RotZ(phi) RotY(theta) RotZ(lam): apply lam first
                ops += [RotZ(q, lam), RotY(q, theta), RotZ(q, phi)]
            else:
                ops.append(Unitary([q], u))
        start = 0 if layer % 2 == 0 else 1
        ops += [CZ(i, i + 1) for i in range(start, n - 1, 2)]
    return ops


def vqe_ansatz(n: int, layers: int, params: np.ndarray):
    """params: (layers, n, 2) float32 angles (RotY, RotZ)."""
    ops = []
    for l in range(layers):
        for q in range(n):
            ops.append(RotY(q, float(params[l, q, 0])))
            ops.append(RotZ(q, float(params[l, q, 1])))
        if n > 1:
            ops += [CX(i, (i + 1) % n) for i in range(n)] if n > 2 else [CX(0, 1)]
    return ops


def gate_count(ops) -> int:
    return len(ops)


__all__ = ["qft", "plain_layers", "brickwork", "vqe_ansatz", "haar_su2", "euler_zyz", "CPhase", "Swap"]


def op_dtype():
    """numpy structured dtype with the exact layout of struct aqsg_op."""
    import ctypes as C

    from ._abi import Op
    names, formats, offsets = [], [], []
    fmt = {"kind": "<i4", "num_qubits": "<i4", "num_controls": "<i4", "control_values": "<u4",
           "angle": "<f4", "qubits": ("<i4", 5), "controls": ("<i4", 16), "matrix": "<u8"}
    for name, _ in Op._fields_:
        names.append(name)
        formats.append(fmt[name])
        offsets.append(getattr(Op, name).offset)
    return np.dtype({"names": names, "formats": formats, "offsets": offsets, "itemsize": C.sizeof(Op)})


def vqe_ops_array(n: int, layers: int, params: np.ndarray) -> np.ndarray:
    """vqe_ansatz(n, layers, params) as a structured array (fast for big
    sweeps): per layer RotY then RotZ on each qubit, then the CX ring."""
    from . import _abi
    ring = n if n > 2 else (1 if n == 2 else 0)
    per = 2 * n + ring
    a = np.zeros(layers * per, dtype=op_dtype())
    idx = np.arange(layers)[:, None] * per
    q = np.arange(n)
    ry = (idx + 2 * q).ravel()
    rz = (idx + 2 * q + 1).ravel()
    a["kind"][ry] = _abi.RY
    a["kind"][rz] = _abi.RZ
    a["num_qubits"][ry] = 1
    a["num_qubits"][rz] = 1
    a["qubits"][ry, 0] = np.tile(q, layers)
    a["qubits"][rz, 0] = np.tile(q, layers)
    a["angle"][ry] = params[:, :, 0].astype(np.float32).ravel()
    a["angle"][rz] = params[:, :, 1].astype(np.float32).ravel()
    if ring:
        cx = (idx + 2 * n + np.arange(ring)).ravel()
        a["kind"][cx] = _abi.CX
        a["num_qubits"][cx] = 2
        a["qubits"][cx, 0] = np.tile(np.arange(ring), layers)
        a["qubits"][cx, 1] = np.tile((np.arange(ring) + 1) % n, layers)
    return a


def vqe_sweep(count: int = 4096, seed: int = 5, n_range=(8, 20), layer_range=(4, 12)):
    """The batched VQE sweep: `count` hardware-efficient-ansatz circuits with
    qubits uniform in n_range, layers uniform in layer_range and angles
    uniform in [-pi, pi].  Returns [(n, structured op array), ...]."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.integers(n_range[0], n_range[1] + 1))
        L = int(rng.integers(layer_range[0], layer_range[1] + 1))
        params = rng.uniform(-np.pi, np.pi, size=(L, n, 2))
        out.append((n, vqe_ops_array(n, L, params)))
    return out
