"""FP64 reference for registers too large for the host oracle: the gates of
the quantum Fourier transform (H, controlled phase, Swap) applied one by one
to a complex128 PyTorch tensor on the GPU with PyTorch's own elementwise
operations -- no code of the engine runs.  Test infrastructure, like the C
oracle, which it is pinned against at 24 qubits
(tests/test_gpu_large_parity.py).

Conventions are the engine's and the reference's: qubit q is index bit
n - 1 - q (src/quantum.cpp:546); H has entries 1/sqrt(2); CPhase(c, t, a)
multiplies the amplitudes whose control and target bits are both 1 by
exp(i a), with a the gate's float angle taken in double; Swap exchanges the
two bits.  The circuit is fourier_transform(n) (src/quantum_algo.cpp:103-114)
plus the final Swaps.
"""
from __future__ import annotations

import math

import torch

from afquantumsim_gb300 import _abi

H = 0.70710678118654752440


def _bits(n, q):
    return n - 1 - q


def _view2(v: torch.Tensor, hi: int, lo: int) -> torch.Tensor:
    """v viewed as (rest, 2, mid, 2, low) with index bits hi > lo split out."""
    N = v.numel()
    return v.view(N >> (hi + 1), 2, 1 << (hi - lo - 1), 2, 1 << lo)


def apply_h(v: torch.Tensor, n: int, q: int) -> None:
    b = _bits(n, q)
    x = v.view(v.numel() >> (b + 1), 2, 1 << b)
    a, c = x[:, 0, :], x[:, 1, :]
    s = a + c
    c.sub_(a).mul_(-H)  # H (a - c)
    a.copy_(s).mul_(H)


def apply_cphase(v: torch.Tensor, n: int, c: int, t: int, angle: float) -> None:
    bc, bt = _bits(n, c), _bits(n, t)
    x = _view2(v, max(bc, bt), min(bc, bt))
    x[:, 1, :, 1, :].mul_(complex(math.cos(angle), math.sin(angle)))


def apply_swap(v: torch.Tensor, n: int, a: int, b: int) -> None:
    ba, bb = _bits(n, a), _bits(n, b)
    x = _view2(v, max(ba, bb), min(ba, bb))
    t = x[:, 0, :, 1, :].clone()
    x[:, 0, :, 1, :].copy_(x[:, 1, :, 0, :])
    x[:, 1, :, 0, :].copy_(t)


def apply_ops(v: torch.Tensor, n: int, ops) -> torch.Tensor:
    """Applies ops (H, CPhase and Swap without extra controls) in place to
    the complex128 tensor v of 2^n amplitudes."""
    assert v.dtype == torch.complex128 and v.is_contiguous() and v.numel() == 1 << n
    for o in ops:
        assert o.num_controls == 0, "extra controls are not restated here"
        if o.kind == _abi.H:
            apply_h(v, n, o.qubits[0])
        elif o.kind == _abi.CPHASE:
            apply_cphase(v, n, o.qubits[0], o.qubits[1], float(o.angle))
        elif o.kind == _abi.SWAP:
            apply_swap(v, n, o.qubits[0], o.qubits[1])
        elif o.kind == _abi.BARRIER:
            pass
        else:
            raise ValueError(f"gate kind {o.kind} is not restated here")
    return v


def errors(got: torch.Tensor, want: torch.Tensor) -> dict:
    """Max amplitude error, l2 norm of the difference and 1 - fidelity
    (|<want|got>|^2 / (|want|^2 |got|^2)) of got against the FP64 want,
    all in FP64 (both tensors on the same device)."""
    g = got.to(torch.complex128)
    d = g - want
    max_abs = float(d.abs().max())
    l2 = float(torch.linalg.vector_norm(d))
    ov = torch.vdot(want, g)
    fid = float(ov.abs() ** 2 / (torch.vdot(want, want).real * torch.vdot(g, g).real))
    return {"max_abs_err": max_abs, "l2_err": l2, "one_minus_fidelity": max(0.0, 1.0 - fid)}
