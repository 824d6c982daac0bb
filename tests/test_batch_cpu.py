"""The vectorised VQE op builder equals the gate-by-gate builder (CPU)."""
import numpy as np

import afquantumsim_gb300 as aq
from afquantumsim_gb300 import circuits
from oracle import oracle


def test_vqe_ops_array_matches_builder():
    rng = np.random.default_rng(0)
    for n, L in ((1, 2), (2, 3), (5, 4), (9, 2)):
        params = rng.uniform(-np.pi, np.pi, size=(L, n, 2))
        arr = circuits.vqe_ops_array(n, L, params)
        ops = circuits.vqe_ansatz(n, L, params)
        assert len(arr) == len(ops)
        v = np.zeros(1 << n, dtype=np.complex128)
        v[0] = 1
        import ctypes as C
        a = (aq.Op * len(arr)).from_buffer_copy(arr.tobytes())
        got = oracle.apply_f64(v.copy(), list(a))
        want = oracle.apply_f64(v.copy(), ops)
        assert np.array_equal(got, want)
