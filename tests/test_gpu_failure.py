"""Failure path without a GPU fault: a device wait that nothing releases
runs out after its limit, the call reports AQSG_ERR_TIMEOUT, and the context
keeps working."""
import ctypes as C

import pytest

import afquantumsim_gb300 as aq

pytestmark = pytest.mark.gpu


def test_bounded_wait_runs_out_and_context_stays_usable(gpu_ctx):
    lib = gpu_ctx.lib
    flag = C.c_int(-1)
    rc = lib.aqsg_selftest_bounded_wait(gpu_ctx.h, 2000, C.byref(flag))
    assert rc == -7 and flag.value == 1
    assert "ran out" in aq.last_error()
    with aq.State(gpu_ctx, 10) as st:
        st.set_basis(3)
        st.apply([aq.X(0), aq.H(5)], aq.EXEC_TILED)
        assert abs(st.norm2() - 1.0) < 1e-6
    assert lib.aqsg_selftest_bounded_wait(gpu_ctx.h, 0, C.byref(flag)) == -1
