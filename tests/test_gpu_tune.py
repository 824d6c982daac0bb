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
