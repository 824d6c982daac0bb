"""Two registers on two contexts as an upload -> gates -> download pipeline
ordered with aqsg_ctx_after (the end-to-end pattern of the benchmark): every
step's result equals the same circuit run on its own."""
import numpy as np
import pytest
import torch

import afquantumsim_gb300 as aq
from tests import _kat

pytestmark = pytest.mark.gpu


def test_two_context_pipeline_ordered(gpu_ctx):
    n, steps = 18, 5
    ops = aq.fourier_transform(n, swaps=True)
    inputs = [_kat.random_state(n, 100 + s).astype(np.complex64) for s in range(steps)]
    want = []
    with aq.State(gpu_ctx, n) as st:
        for v in inputs:
            st.upload(v)
            st.apply(ops, aq.EXEC_PER_GATE)
            want.append(st.download())
    ctxs = [aq.Context(0), aq.Context(0)]
    sts = [aq.State(c, n) for c in ctxs]
    host_in = [torch.from_numpy(v).pin_memory() for v in inputs]
    host_out = [torch.empty(1 << n, dtype=torch.complex64).pin_memory() for _ in range(steps)]
    try:
        for s in range(steps):
            c, r = ctxs[s % 2], sts[s % 2]
            c.synchronize()
            r.upload_ptr(host_in[s].data_ptr())
            if s > 0:
                c.after(ctxs[(s - 1) % 2])
                r.apply(ops, aq.EXEC_PER_GATE)
                sts[(s - 1) % 2].download_async_ptr(host_out[s - 1].data_ptr())
            else:
                r.apply(ops, aq.EXEC_PER_GATE)
        sts[(steps - 1) % 2].download_async_ptr(host_out[steps - 1].data_ptr())
        for c in ctxs:
            c.synchronize()
        for s in range(steps):
            np.testing.assert_array_equal(host_out[s].numpy(), want[s])
        ctxs[0].after(ctxs[0])  # a context is ordered with itself: no-op
    finally:
        for r in sts:
            r.free()
        for c in ctxs:
            c.close()
