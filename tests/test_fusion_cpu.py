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
