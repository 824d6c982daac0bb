"""FP64 density-matrix oracle for circuits under a Pauli channel, and a
restatement of the engine's trajectory sampler.

TEST INFRASTRUCTURE ONLY: tests compare the engine's trajectory estimates
(aqsg_noise_expect_z) and trajectories (aqsg_noise_trajectory) with it.

The channel (the engine's definition; the reference declares an empty
QNoise class, include/quantum.h:475): after every gate, each qubit the gate
touches (targets and controls) independently becomes X rho X, Y rho Y or
Z rho Z with probabilities p[0], p[1], p[2], where p = p1 after one-qubit
gates and p2 after gates on several qubits.  Gates act as rho -> U rho U^+,
with U the gate's matrix as the per-gate FP64 oracle applies it.
"""
from __future__ import annotations

import numpy as np

from afquantumsim_gb300 import _abi

from . import oracle

MASK64 = (1 << 64) - 1


def touched(op) -> list[int]:
    """Targets, then controls, of an op."""
    k = op.num_qubits if op.kind == _abi.UNITARY else _abi.ARITY[op.kind]
    return [op.qubits[i] for i in range(k)] + [op.controls[i] for i in range(op.num_controls)]


def gate_unitary(n: int, op) -> np.ndarray:
    """The 2^n x 2^n matrix of one op, column by column from the FP64 oracle."""
    N = 1 << n
    cols = np.eye(N, dtype=np.complex128)
    out = np.empty((N, N), dtype=np.complex128)
    for k in range(N):
        out[:, k] = oracle.apply_f64(np.ascontiguousarray(cols[:, k]), [op])
    return out


def _pauli_on(n: int, q: int, which: int) -> np.ndarray:
    P = [np.array([[0, 1], [1, 0]], dtype=np.complex128),
         np.array([[0, -1j], [1j, 0]], dtype=np.complex128),
         np.array([[1, 0], [0, -1]], dtype=np.complex128)][which]
    m = np.ones((1, 1), dtype=np.complex128)
    for i in range(n):  # qubit 0 is the most significant index bit
        m = np.kron(m, P if i == q else np.eye(2))
    return m


def density_expect_z(n: int, ops, p1, p2):
    """<Z_q> and <Z_q Z_q+1> of the noisy circuit from |0...0>, exactly (FP64
    density matrix)."""
    N = 1 << n
    rho = np.zeros((N, N), dtype=np.complex128)
    rho[0, 0] = 1
    paulis = {(q, w): _pauli_on(n, q, w) for q in range(n) for w in range(3)}
    for op in ops:
        if op.kind == _abi.BARRIER:
            continue
        U = gate_unitary(n, op)
        rho = U @ rho @ U.conj().T
        t = touched(op)
        p = p1 if len(t) == 1 else p2
        for q in t:
            keep = 1.0 - float(np.float32(p[0])) - float(np.float32(p[1])) - float(np.float32(p[2]))
            acc = keep * rho
            for w in range(3):
                P = paulis[(q, w)]
                acc = acc + float(np.float32(p[w])) * (P @ rho @ P)
            rho = acc
    diag = np.real(np.diag(rho))
    idx = np.arange(N)
    bit = lambda q: (idx >> (n - 1 - q)) & 1  # noqa: E731
    z = np.array([np.sum(diag * (1 - 2 * bit(q))) for q in range(n)])
    zz = np.array([np.sum(diag * (1 - 2 * (bit(q) ^ bit(q + 1)))) for q in range(n - 1)])
    return z, zz


# ---- the sampler, restated -----------------------------------------------------------

def _mix64(z: int) -> int:
    # SplitMix64's finaliser (Steele, Lea, Flood, OOPSLA 2014)
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
    return z ^ (z >> 31)


def draw(seed: int, trajectory: int, gate: int, slot: int) -> float:
    h = _mix64(seed ^ 0x243F6A8885A308D3)
    h = _mix64(h ^ trajectory)
    h = _mix64(h ^ ((gate << 8 | slot) & MASK64))
    return (h >> 11) * (1.0 / 9007199254740992.0)


def trajectory_kinds(ops, p1, p2, seed: int, trajectory: int):
    """[(gate index, qubit, kind)] of the Paulis trajectory `trajectory`
    inserts, in order."""
    out = []
    for g, op in enumerate(ops):
        if op.kind == _abi.BARRIER:
            continue
        t = touched(op)
        p = [float(np.float32(x)) for x in (p1 if len(t) == 1 else p2)]
        for s, q in enumerate(t):
            u = draw(seed, trajectory, g, s)
            if u < p[0]:
                out.append((g, q, _abi.X))
            elif u < p[0] + p[1]:
                out.append((g, q, _abi.Y))
            elif u < p[0] + p[1] + p[2]:
                out.append((g, q, _abi.Z))
    return out
