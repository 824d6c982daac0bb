"""Parity at the sizes that are timed: the QFT with swaps at 28 and 30 qubits
(complex64 and complex128, one gate per pass, plus tile passes at 28 qubits)
against an FP64 reference, and the fused brick-work circuit at 26 qubits,
depth 20, with the fused unitaries on the tensor cores, against the host
FP64 oracle.

The 28/30-qubit FP64 reference is tests/fp64_torch.py (the same gates as
PyTorch complex128 operations, no engine code), itself checked here against
the C oracle (oracle.apply_f64) at 10 qubits on the CPU and 24 qubits on the
GPU.  Tolerances (the benchmark spec's): complex64 within 1e-5 of FP64 per
amplitude, complex128 within 1e-12; because the amplitudes of a 30-qubit
state are ~3e-5, the complex64 checks also bound the l2 norm of the error
(the state has norm 1) and 1 - fidelity.
"""
import numpy as np
import pytest
import torch

import afquantumsim_gb300 as aq
from afquantumsim_gb300 import circuits
from oracle import oracle
from tests import _kat, fp64_torch

TOL64, L2_64, INFID64 = 1e-5, 1e-5, 1e-9
TOL128 = 1e-12


def test_fp64_torch_matches_oracle_cpu():
    n = 10
    v = _kat.random_state(n, 11)
    ops = aq.fourier_transform(n, swaps=True)
    want = oracle.apply_f64(v.copy(), ops)
    got = fp64_torch.apply_ops(torch.from_numpy(v.copy()), n, ops).numpy()
    assert np.max(np.abs(got - want)) < 1e-14


def seeded_state(n, seed, dtype):
    """i.i.d. standard-normal complex amplitudes, normalised in FP64, on cuda:0."""
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    x = torch.randn(1 << n, dtype=dtype, device="cuda", generator=g)
    x /= torch.linalg.vector_norm(x.to(torch.complex128)).to(x.real.dtype)
    return x


def engine_run(ctx, x, n, ops, mode):
    """Runs ops on a register holding x (through pinned host memory) and
    returns the result as a cuda tensor."""
    dt = aq.C64 if x.dtype == torch.complex64 else aq.C128
    host = torch.empty(x.numel(), dtype=x.dtype, pin_memory=True)
    host.copy_(x)
    with aq.State(ctx, n, dt) as st:
        st.upload_ptr(host.data_ptr())
        st.apply(ops, mode)
        st.download_ptr(host.data_ptr())
    return host.to("cuda")


@pytest.mark.gpu
def test_fp64_torch_matches_oracle_24q():
    n = 24
    v = _kat.random_state(n, 12)
    ops = aq.fourier_transform(n, swaps=True)
    want = oracle.apply_f64(v.copy(), ops)
    got = fp64_torch.apply_ops(torch.from_numpy(v.copy()).cuda(), n, ops).cpu().numpy()
    assert np.max(np.abs(got - want)) < 1e-14


@pytest.mark.gpu
@pytest.mark.parametrize("n,dtype,mode", [
    (28, torch.complex64, aq.EXEC_PER_GATE), (28, torch.complex64, aq.EXEC_TILED),
    (28, torch.complex128, aq.EXEC_PER_GATE), (28, torch.complex128, aq.EXEC_TILED),
    (30, torch.complex64, aq.EXEC_PER_GATE), (30, torch.complex128, aq.EXEC_PER_GATE),
], ids=["28-c64-per_gate", "28-c64-tiled", "28-c128-per_gate", "28-c128-tiled", "30-c64-per_gate",
        "30-c128-per_gate"])
def test_qft_vs_fp64(gpu_ctx, n, dtype, mode):
    ops = aq.fourier_transform(n, swaps=True)
    x = seeded_state(n, 3, dtype)
    got = engine_run(gpu_ctx, x, n, ops, mode)
    want = fp64_torch.apply_ops(x.to(torch.complex128), n, ops)
    del x
    e = fp64_torch.errors(got, want)
    print(n, dtype, mode, e)
    if dtype == torch.complex64:
        assert e["max_abs_err"] < TOL64 and e["l2_err"] < L2_64 and e["one_minus_fidelity"] < INFID64, e
    else:
        assert e["max_abs_err"] < TOL128 and e["l2_err"] < TOL128, e


@pytest.mark.gpu
def test_fused_brickwork_26_tensor_cores_vs_host_oracle(gpu_ctx):
    """Brick-work 26 qubits x 20 layers (Haar SU(2) as RotZ.RotY.RotZ + CZ,
    seed 4), compiled into <= 5-qubit unitaries applied on the tensor cores
    (split BF16, FP32 accumulation), from |0...0>, against the per-gate FP64
    oracle on the host."""
    n = 26
    ops = circuits.brickwork(n, 20, seed=4)
    prog = aq.Program(n, ops, aq.C64, max_qubits=5)
    gpu_ctx.set_tensor_cores(True)
    with aq.State(gpu_ctx, n, aq.C64) as st:
        st.set_basis(0)
        prog.run(st, aq.EXEC_TILED)
        got = st.download()
    prog.free()
    v = np.zeros(1 << n, dtype=np.complex128)
    v[0] = 1
    oracle.set_threads(0)
    want = oracle.apply_f64(v, ops)
    e = fp64_torch.errors(torch.from_numpy(got), torch.from_numpy(want))
    print("brickwork26x20 tensor cores", e)
    assert e["max_abs_err"] < TOL64 and e["one_minus_fidelity"] < 1e-6, e
