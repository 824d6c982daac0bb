"""The host tile encoder checked on the CPU: the plan the engine would run
(aqsg_debug_tile_plan: passes, op table with register phases, operand pool),
interpreted by a numpy restatement of the tile kernels' record semantics
(tests/tile_emulator.py), gives the FP64 oracle's state — for whole-register
and streaming passes, complex64 and complex128 encodings, fused and unfused
programs, every gate kind with extra controls.  The device code itself is
covered by the GPU parity tests."""
import numpy as np
import pytest

import afquantumsim_gb300 as aq
from afquantumsim_gb300 import circuits
from oracle import oracle
from tests import _kat
from tests.tile_emulator import run_plan


@pytest.mark.parametrize("dtype", [aq.C64, aq.C128])
@pytest.mark.parametrize("n,fuse,seed", [(6, 0, 1), (9, 0, 2), (10, 2, 3), (12, 0, 4), (12, 3, 5),
                                         (13, 4, 6), (15, 0, 7), (15, 2, 8), (16, 3, 9)])
def test_encoded_plan_equals_oracle(dtype, n, fuse, seed):
    ops = _kat.random_circuit(n, 120, seed)
    passes, table, pool = aq.debug_tile_plan(n, ops, dtype, fuse)
    v = _kat.random_state(n, seed)
    want = oracle.apply_f64(v.copy(), ops)
    got = run_plan(v, n, passes, table, pool, c64=(dtype == aq.C64))
    tol = 1e-5 if dtype == aq.C64 else 1e-12
    assert np.max(np.abs(got - want)) < tol


def test_vqe_plan_uses_register_phases():
    n = 16
    ops = circuits.vqe_ops_array(n, 3, np.random.default_rng(2).uniform(-np.pi, np.pi, size=(3, n, 2)))
    ops = list((aq.Op * len(ops)).from_buffer_copy(ops.tobytes()))
    passes, table, pool = aq.debug_tile_plan(n, ops, aq.C64, 0)
    recs = np.frombuffer(table, dtype=np.int32).reshape(-1, 40)
    assert (recs[:, 0] == 8).any()  # register-phase headers
    v = _kat.random_state(n, 3)
    got = run_plan(v, n, passes, table, pool, c64=True)
    assert np.max(np.abs(got - oracle.apply_f64(v.copy(), ops))) < 1e-5


@pytest.mark.parametrize("dtype,n,fuse,seed", [(aq.C64, 13, 0, 11), (aq.C64, 14, 2, 12), (aq.C64, 14, 5, 13),
                                               (aq.C128, 12, 0, 14), (aq.C128, 13, 3, 15)])
def test_streaming_tile_shape_for_small_registers(dtype, n, fuse, seed):
    # a register that fits one whole-register tile, encoded with the
    # whole-tile limit lowered to the streaming tile: streaming passes of
    # 2^12 (c64) / 2^11 (c128) amplitudes that still give the oracle's state
    stream = 12 if dtype == aq.C64 else 11
    ops = _kat.random_circuit(n, 150, seed)
    whole, _, _ = aq.debug_tile_plan(n, ops, dtype, fuse)
    assert [p.m for p in whole] == [n]
    passes, table, pool = aq.debug_tile_plan(n, ops, dtype, fuse, whole_tile_max=stream)
    assert passes and all(p.m == stream and p.L == (5 if dtype == aq.C64 else 4) for p in passes)
    # a limit above the dtype's maximum is clamped: the whole register again
    again, _, _ = aq.debug_tile_plan(n, ops, dtype, fuse, whole_tile_max=40)
    assert [p.m for p in again] == [n]
    v = _kat.random_state(n, seed)
    want = oracle.apply_f64(v.copy(), ops)
    got = run_plan(v, n, passes, table, pool, c64=(dtype == aq.C64))
    tol = 1e-5 if dtype == aq.C64 else 1e-12
    assert np.max(np.abs(got - want)) < tol


def test_whole_tile_limit_rejects_negative():
    with pytest.raises(aq.InvalidArgument):
        aq.debug_tile_plan(13, _kat.random_circuit(13, 10, 1), aq.C64, 0, whole_tile_max=-1)


@pytest.mark.parametrize("n,k,seed,gates,wmax", [(12, 5, 21, 40, 0), (13, 3, 22, 150, 12), (15, 5, 23, 150, 0),
                                                  (16, 4, 24, 150, 0), (17, 5, 25, 150, 0), (15, 3, 26, 150, 0)])
def test_tensor_core_plan_equals_oracle(n, k, seed, gates, wmax):
    # the tensor-core form of a fused program: split-BF16 B operands in the
    # K-major layout, the data-column and matrix-row tables, run as the
    # tensor cores compute it, gives the FP64 oracle's state (12 qubits: the
    # whole register as one tensor-core tile; 13 in streaming tiles)
    ops = _kat.random_circuit(n, gates, seed)
    passes, table, pool = aq.debug_tile_plan(n, ops, aq.C64, k, whole_tile_max=wmax, tensor_cores=True)
    assert any(p.tc for p in passes)
    v = _kat.random_state(n, seed)
    want = oracle.apply_f64(v.copy(), ops)
    got = run_plan(v, n, passes, table, pool, c64=True)
    assert np.max(np.abs(got - want)) < 1e-5
    # the same program's CUDA-core form agrees
    cc = run_plan(v, n, *aq.debug_tile_plan(n, ops, aq.C64, k, whole_tile_max=wmax), c64=True)
    assert np.max(np.abs(cc - want)) < 1e-5


def test_tensor_core_brickwork_plan_streaming_14():
    # a 14-qubit brick-work program in streaming tiles (the autotuner's
    # other tile shape) on the tensor cores
    n = 14
    ops = circuits.brickwork(n, 10, seed=3)
    passes, table, pool = aq.debug_tile_plan(n, ops, aq.C64, 5, whole_tile_max=12, tensor_cores=True)
    assert all(p.m == 12 for p in passes) and sum(p.tc for p in passes) >= 3
    v = _kat.random_state(n, 8)
    got = run_plan(v, n, passes, table, pool, c64=True)
    assert np.max(np.abs(got - oracle.apply_f64(v.copy(), ops))) < 1e-5
