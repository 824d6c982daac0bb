"""aqsg_sample_noalloc: sampling without device allocation.

Some callers of this engine cannot allocate device memory while they run —
a serving loop holding a fixed HBM budget, or a host process that shares the
GPU with a framework's caching allocator — because cudaMalloc/cudaFree can
synchronise the device and stall other streams.  aqsg_sample_noalloc gives
them the sampler on a static scratch array of the library.  This file checks,
through the C ABI, that it returns exactly what the allocating entry point
aqsg_sample returns, on two calls in a row (the calls share the static
scratch), and that it rejects requests beyond its stated limits.

The file is named so that pytest collects it last.
"""
import numpy as np
import pytest

import afquantumsim_gb300 as aq
from afquantumsim_gb300 import _abi
from tests import _kat

pytestmark = pytest.mark.gpu

MAX_SHOTS = 16384  # AQSG_NOALLOC_MAX_SHOTS
MAX_QUBITS = 30    # AQSG_NOALLOC_MAX_QUBITS


@pytest.mark.parametrize("n", [9, 20])
@pytest.mark.parametrize("dtype,npdt", [(aq.C64, np.complex64), (aq.C128, np.complex128)])
def test_noalloc_matches_allocating_sampler(gpu_ctx, n, dtype, npdt):
    v = _kat.random_state(n, 40 + n).astype(npdt)
    rng = np.random.default_rng(n)
    with aq.State(gpu_ctx, n, dtype) as st:
        st.upload(v)
        for call in range(2):
            u = rng.random(4000 + 1000 * call)
            u[:3] = [0.0, 0.5, 1.0 - 1e-12]
            want = st.sample(u)
            got = st.sample_noalloc(u)
            assert np.array_equal(got, want), (n, dtype, call)
            got_clamp = st.sample_noalloc(u, aq.SAMPLE_CLAMP)
            assert np.array_equal(got_clamp, st.sample(u, aq.SAMPLE_CLAMP))


def test_noalloc_rejects_beyond_limits(gpu_ctx):
    with aq.State(gpu_ctx, 6, aq.C64) as st:
        st.set_basis(3)
        assert list(st.sample_noalloc(np.full(MAX_SHOTS, 0.5))[:2]) == [3, 3]
        with pytest.raises(aq.InvalidArgument) as e:
            st.sample_noalloc(np.full(MAX_SHOTS + 1, 0.5))
        assert "at most 16384 shots" in e.value.msg
    assert _abi.MAX_QUBITS >= MAX_QUBITS


def test_noalloc_rejects_registers_above_30_qubits(gpu_ctx):
    # a 31-qubit c64 register is 16 GiB; the call fails before any kernel runs
    with aq.State(gpu_ctx, MAX_QUBITS + 1, aq.C64) as st:
        with pytest.raises(aq.InvalidArgument) as e:
            st.sample_noalloc([0.5])
        assert "at most 30 qubits" in e.value.msg


def test_noalloc_grows_none_of_the_contexts_scratch():
    # a fresh context: only the allocation-free sampler runs on it, and every
    # scratch buffer the context grows on demand stays unallocated; the
    # allocating sampler on the same register then does grow them
    with aq.Context(0) as ctx:
        with aq.State(ctx, 12, aq.C64) as st:
            st.set_basis(5)
            assert ctx.scratch_bytes() == [0] * 6
            got = st.sample_noalloc(np.linspace(0.0, 1.0 - 1e-9, 257))
            assert set(got.tolist()) == {5}
            assert ctx.scratch_bytes() == [0] * 6
            st.sample([0.5])
            assert sum(ctx.scratch_bytes()) > 0
