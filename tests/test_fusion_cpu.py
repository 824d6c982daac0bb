"""Gate fusion (aqsg_compile) checked on the CPU: the exported fused program,
run by the FP64 oracle, equals the source circuit run by the oracle."""
import numpy as np
import pytest

import afquantumsim_gb300 as aq
from afquantumsim_gb300 import circuits
from oracle import oracle
from tests import _kat


@pytest.mark.parametrize("k", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("n,seed", [(4, 1), (7, 2), (9, 3)])
def test_fused_program_equals_source(k, n, seed):
    ops = _kat.random_circuit(n, 120, seed)
    v = _kat.random_state(n, seed)
    want = oracle.apply_f64(v.copy(), ops)
    prog = aq.Program(n, ops, aq.C128, max_qubits=k)
    fused, src = prog.info()
    assert src == len(ops) and fused <= len(ops)
    got = oracle.apply_f64(v.copy(), list(prog.export()))
    assert np.max(np.abs(got - want)) < 1e-12


def test_brickwork_fuses_and_matches():
    n = 10
    ops = circuits.brickwork(n, 6, seed=4)
    v = _kat.random_state(n, 4)
    want = oracle.apply_f64(v.copy(), ops)
    prog = aq.Program(n, ops, aq.C128, max_qubits=5)
    fused, src = prog.info()
    assert fused < src / 4
    assert np.max(np.abs(oracle.apply_f64(v.copy(), list(prog.export())) - want)) < 1e-12


def test_euler_form_is_the_haar_unitary():
    rng = np.random.default_rng(0)
    for _ in range(20):
        u = circuits.haar_su2(rng)
        phi, theta, lam = circuits.euler_zyz(u)
        rz = lambda x: np.diag([np.exp(-0.5j * x), np.exp(0.5j * x)])
        ry = lambda x: np.array([[np.cos(x / 2), -np.sin(x / 2)], [np.sin(x / 2), np.cos(x / 2)]])
        assert np.allclose(rz(phi) @ ry(theta) @ rz(lam), u)


def test_compile_validates_like_check():
    with pytest.raises(aq.OutOfRange):
        aq.Program(3, [aq.H(3)])
    with pytest.raises(aq.InvalidArgument):
        aq.Program(3, [aq.H(0)], max_qubits=6)


def test_program_plan_traffic():
    """aqsg_program_plan: one read + one write of the register per pass; a
    run with tensor-core passes adds the scale pass (its first and last
    passes carry the norm sums)."""
    n = 20
    prog = aq.Program(n, circuits.brickwork(n, 6, seed=4), aq.C64, max_qubits=5)
    reg = 8 << n
    off = prog.plan(tensor_cores=False)
    assert off["tc_passes"] == 0 and off["passes"] > 0
    assert off["hbm_bytes"] == 2 * reg * off["passes"]
    on = prog.plan(tensor_cores=True)
    assert 0 < on["tc_passes"] <= on["passes"]
    assert on["hbm_bytes"] in (2 * reg * on["passes"] + 2 * reg, 2 * reg * on["passes"] + 3 * reg,
                               2 * reg * on["passes"] + 4 * reg)
    prog.free()


def test_tensor_core_pass_op_limit():
    """A whole 12-qubit register with more ops than the tensor-core kernel
    holds in shared memory runs on the CUDA cores."""
    r = np.array([[0.6, 0.8], [-0.8, 0.6]])
    u3 = np.kron(np.kron(r, r.T), r).astype(np.complex64)  # dense, not a permutation
    # overlapping 3-qubit windows: no two neighbours fuse within 3 qubits
    ops = [aq.Unitary([w, w + 1, w + 2], u3) for w in [i % 10 for i in range(40)]]
    prog = aq.Program(12, ops, aq.C64, max_qubits=3)
    fused, _ = prog.info()
    assert fused > 24
    assert prog.plan(tensor_cores=True)["tc_passes"] == 0
    prog.free()
    few = aq.Program(12, ops[:10], aq.C64, max_qubits=3)
    assert few.plan(tensor_cores=True)["tc_passes"] == 1
    few.free()
