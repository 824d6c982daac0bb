"""Fused programs (aqsg_compile) on the GPU: tile passes with fused
unitaries on the tensor cores (tcgen05, split-BF16, FP32 accumulate) and on
the CUDA cores, against the FP64 oracle.  c64 tolerance 1e-5 absolute."""
import numpy as np
import pytest

import afquantumsim_gb300 as aq
from afquantumsim_gb300 import circuits
from oracle import oracle
from tests import _kat

pytestmark = pytest.mark.gpu


def run_prog(ctx, v, prog, dtype, mode):
    n = int(v.size).bit_length() - 1
    with aq.State(ctx, n, dtype) as st:
        st.upload(v)
        prog.run(st, mode)
        return st.download()


@pytest.mark.parametrize("tc", [True, False])
@pytest.mark.parametrize("n,k,seed", [(12, 5, 1), (12, 3, 2), (15, 5, 3), (16, 4, 4), (18, 5, 5),
                                      (20, 3, 6), (20, 5, 7)])
def test_fused_random_circuits(gpu_ctx, tc, n, k, seed):
    ops = _kat.random_circuit(n, 150, seed)
    v = _kat.random_state(n, seed)
    want = oracle.apply_f64(v.copy(), ops)
    prog = aq.Program(n, ops, aq.C64, max_qubits=k)
    gpu_ctx.set_tensor_cores(tc)
    try:
        got = run_prog(gpu_ctx, v.astype(np.complex64), prog, aq.C64, aq.EXEC_TILED)
    finally:
        gpu_ctx.set_tensor_cores(True)
    assert np.max(np.abs(got - want)) < 1e-5
    prog128 = aq.Program(n, ops, aq.C128, max_qubits=k)
    got128 = run_prog(gpu_ctx, v.copy(), prog128, aq.C128, aq.EXEC_TILED)
    assert np.max(np.abs(got128 - want)) < 1e-12


@pytest.mark.parametrize("n,depth", [(12, 8), (16, 20), (22, 10)])
def test_fused_brickwork(gpu_ctx, n, depth):
    ops = circuits.brickwork(n, depth, seed=4)
    v = _kat.random_state(n, 9)
    want = oracle.apply_f64(v.copy(), ops)
    prog = aq.Program(n, ops, aq.C64, max_qubits=5)
    for mode in (aq.EXEC_TILED, aq.EXEC_PER_GATE):
        got = run_prog(gpu_ctx, v.astype(np.complex64), prog, aq.C64, mode)
        err = np.max(np.abs(got - want))
        g = got.astype(np.complex128)
        fid = abs(np.vdot(want, g)) ** 2 / (np.vdot(want, want).real * np.vdot(g, g).real)
        assert err < 1e-5 and 1 - fid < 1e-7, (mode, err, fid)


def test_fused_permutation_unitary_bit_exact(gpu_ctx):
    """A 5-qubit permutation unitary in a tensor-core-capable tile pass: it
    runs on the CUDA cores (x * 1 + 0 * y), so it only moves amplitudes."""
    n = 15
    rng = np.random.default_rng(3)
    perm = rng.permutation(32)
    m = np.zeros((32, 32))
    m[perm, np.arange(32)] = 1
    ops = [aq.Unitary([1, 4, 7, 9, 12], m)]
    v = _kat.random_state(n, 2).astype(np.complex64)
    want = oracle.apply_f64(v.astype(np.complex128), ops)
    with aq.State(gpu_ctx, n, aq.C64) as st:
        st.upload(v)
        st.apply(ops, aq.EXEC_TILED)
        got = st.download()
    assert np.array_equal(got.astype(np.complex128), want)


@pytest.mark.parametrize("n,k", [(12, 5), (16, 5), (19, 4)])
def test_fused_permutation_circuit_bit_exact(gpu_ctx, n, k):
    """Permutation-only circuits (X, CX, CCNot, Swap, CSwap, Or) stay
    bit-exact when fused: the fused unitaries are permutation matrices."""
    ops = _kat.random_circuit(n, 200, 40 + n, kinds=["X", "CX", "CCNot", "Swap", "CSwap", "Or"])
    v = _kat.random_state(n, 5).astype(np.complex64)
    with aq.State(gpu_ctx, n, aq.C64) as st:
        st.upload(v)
        st.apply(ops, aq.EXEC_PER_GATE)
        want = st.download()
        prog = aq.Program(n, ops, aq.C64, max_qubits=k)
        st.upload(v)
        prog.run(st, aq.EXEC_TILED)
        got = st.download()
        prog.free()
    assert np.array_equal(got, want)


@pytest.mark.parametrize("tc", [True, False])
def test_runs_are_deterministic(gpu_ctx, tc):
    """Run-to-run determinism: the same program on the same input gives the
    same bits on a second run and on a second context (a fresh plan cache).
    Tile passes accumulate nothing with atomics, and the tensor-core run's
    renormalisation adds its per-CTA partials in a fixed order."""
    n = 20
    ops = circuits.brickwork(n, 12, seed=11)
    v = _kat.random_state(n, 4).astype(np.complex64)
    prog = aq.Program(n, ops, aq.C64, max_qubits=5)

    def three_runs(ctx):
        ctx.set_tensor_cores(tc)
        try:
            out = [run_prog(ctx, v, prog, aq.C64, aq.EXEC_TILED) for _ in range(2)]
            with aq.State(ctx, n, aq.C64) as st:  # the gates unfused, in tile passes
                st.upload(v)
                st.apply(ops, aq.EXEC_TILED)
                out.append(st.download())
        finally:
            ctx.set_tensor_cores(True)
        return out

    first = three_runs(gpu_ctx)
    with aq.Context(0) as other:
        second = three_runs(other)
    assert np.array_equal(first[0], first[1])
    assert np.array_equal(first[0], second[0]) and np.array_equal(first[1], second[1])
    assert np.array_equal(first[2], second[2])
    assert np.max(np.abs(first[0] - first[2])) < 1e-5
    prog.free()
