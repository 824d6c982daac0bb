"""The autotuner (aqsg_autotune): every candidate is timed, the best is the
fastest of them, the choice is cached by circuit structure (a circuit with
new angles returns the cached choice), and running the circuit the chosen
way gives the oracle's state."""
import numpy as np
import pytest

import afquantumsim_gb300 as aq
from afquantumsim_gb300 import circuits
from oracle import oracle
from tests import _kat

pytestmark = pytest.mark.gpu


def test_autotune_candidates_and_cache(gpu_ctx):
    n = 16
    ops = circuits.brickwork(n, 6, seed=3)
    best, every = aq.autotune(gpu_ctx, n, ops, aq.C64, reps=1)
    assert len(every) == 3 + 4 * 2  # per gate, tiled, width 1, widths 2..5 x tensor cores on/off
    assert {(e["exec_mode"], e["fuse_qubits"], e["tensor_cores"]) for e in every} == \
        {(aq.EXEC_PER_GATE, 0, 0), (aq.EXEC_TILED, 0, 0), (aq.EXEC_TILED, 1, 0)} | \
        {(aq.EXEC_TILED, k, t) for k in range(2, 6) for t in (0, 1)}
    assert all(e["ms"] > 0 for e in every)
    assert best["ms"] == min(e["ms"] for e in every)
    # same structure, new angles: the cached choice comes back without timing
    ops2 = circuits.brickwork(n, 6, seed=4)
    again, none = aq.autotune(gpu_ctx, n, ops2, aq.C64, reps=1, all_timings=False)
    assert none == [] and again == best

    # run it the chosen way and compare with the oracle
    v = _kat.random_state(n, 1)
    want = oracle.apply_f64(v.copy(), ops)
    with aq.State(gpu_ctx, n, aq.C64) as st:
        st.upload(v.astype(np.complex64))
        gpu_ctx.set_tensor_cores(bool(best["tensor_cores"]))
        try:
            if best["fuse_qubits"]:
                p = aq.Program(n, ops, aq.C64, max_qubits=best["fuse_qubits"])
                p.run(st, best["exec_mode"])
                p.free()
            else:
                st.apply(ops, best["exec_mode"])
        finally:
            gpu_ctx.set_tensor_cores(True)
        got = st.download()
    assert np.max(np.abs(got - want)) < 1e-5


def test_autotune_c128_has_no_tensor_core_candidates(gpu_ctx):
    ops = circuits.plain_layers(10, 3, seed=2)
    best, every = aq.autotune(gpu_ctx, 10, ops, aq.C128, reps=1)
    assert len(every) == 3 + 4 and not any(e["tensor_cores"] for e in every)


def _run_way(ctx, n, ops, dtype, npdt, v, fuse, tc, mode=aq.EXEC_TILED):
    with aq.State(ctx, n, dtype) as st:
        st.upload(v.astype(npdt))
        ctx.set_tensor_cores(bool(tc))
        try:
            if fuse:
                p = aq.Program(n, ops, dtype, max_qubits=fuse)
                p.run(st, mode)
                p.free()
            else:
                st.apply(ops, mode)
        finally:
            ctx.set_tensor_cores(True)
        return st.download()


@pytest.mark.parametrize("dtype,npdt,n", [(aq.C64, np.complex64, 13), (aq.C64, np.complex64, 14),
                                          (aq.C128, np.complex128, 12), (aq.C128, np.complex128, 13)])
def test_streaming_tile_shape_matches_oracle(gpu_ctx, dtype, npdt, n):
    # registers that fit one whole-register tile, run in streaming tiles
    # instead (several CTAs, one launch per pass; c64 fused unitaries on the
    # tensor cores): the oracle's state, as in the whole-register shape
    stream = 12 if dtype == aq.C64 else 11
    ops = circuits.brickwork(n, 8, seed=n)
    v = _kat.random_state(n, 7)
    want = oracle.apply_f64(v.copy(), ops)
    tol = 1e-5 if dtype == aq.C64 else 1e-12
    ways = [(0, 0), (2, 0), (5, 0)] + ([(3, 1), (5, 1)] if dtype == aq.C64 else [])
    for shape in (stream, 0):
        gpu_ctx.set_whole_tile_max(shape)
        try:
            for fuse, tc in ways:
                got = _run_way(gpu_ctx, n, ops, dtype, npdt, v, fuse, tc)
                assert np.max(np.abs(got - want)) < tol, (shape, fuse, tc)
        finally:
            gpu_ctx.set_whole_tile_max(0)


def test_autotune_times_both_tile_shapes(gpu_ctx):
    n = 14
    ops = circuits.brickwork(n, 10, seed=5)
    best, every = aq.autotune(gpu_ctx, n, ops, aq.C64, reps=1)
    tiled = [(e["fuse_qubits"], e["tensor_cores"]) for e in every if e["exec_mode"] == aq.EXEC_TILED]
    assert len(every) == 1 + 2 * 10
    assert {e["tile_bits"] for e in every} == {0, 12, 14}
    for bits in (12, 14):
        assert sorted((e["fuse_qubits"], e["tensor_cores"]) for e in every if e["tile_bits"] == bits) == \
            sorted(set(tiled))
    assert all(e["tile_bits"] == 0 for e in every if e["exec_mode"] == aq.EXEC_PER_GATE)
    assert best["ms"] == min(e["ms"] for e in every)
    # run it the chosen way, tile shape included, and compare with the oracle
    v = _kat.random_state(n, 2)
    want = oracle.apply_f64(v.copy(), ops)
    gpu_ctx.set_whole_tile_max(best["tile_bits"] if 0 < best["tile_bits"] < n else 0)
    try:
        got = _run_way(gpu_ctx, n, ops, aq.C64, np.complex64, v, best["fuse_qubits"], best["tensor_cores"],
                       best["exec_mode"])
    finally:
        gpu_ctx.set_whole_tile_max(0)
    assert np.max(np.abs(got - want)) < 1e-5


def test_whole_tile_max_rejects_negative(gpu_ctx):
    with pytest.raises(aq.InvalidArgument):
        gpu_ctx.set_whole_tile_max(-1)
