"""Pin the CPU oracle to the reference's own known answers (test/tests.cpp).

Each golden case runs through all three oracle families: the FP64 per-gate
oracle, its FP32 twin, and the faithful FP32 restatement of the reference
algorithm (dense Kronecker / CSR operators).  CPU only.
"""
import numpy as np
import pytest

from oracle import oracle
from tests import _kat

CASES = _kat.load_cases()


def run_f64(n, amps, ops):
    sv = oracle.ref32_product_state(amps).astype(np.complex128)
    return oracle.apply_f64(sv, ops)


def run_f32(n, amps, ops):
    return oracle.apply_f32(oracle.ref32_product_state(amps), ops)


def run_ref32(n, amps, ops):
    return oracle.ref32_apply(oracle.ref32_product_state(amps), n, ops)


FAMILIES = {"f64": run_f64, "f32": run_f32, "ref32": run_ref32}


def matrix_of(n, ops, family):
    if family == "ref32":
        return oracle.ref32_compile(n, ops)
    cols = []
    for k in range(1 << n):
        e = np.zeros(1 << n, dtype=np.complex128 if family == "f64" else np.complex64)
        e[k] = 1
        cols.append(oracle.apply_f64(e, ops) if family == "f64" else oracle.apply_f32(e, ops))
    return np.stack(cols, axis=1)


@pytest.mark.parametrize("family", sorted(FAMILIES))
@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_golden(case, family):
    n = case["n"]
    t = case["type"]
    if t == "amplitudes":
        sv = FAMILIES[family](n, _kat.init_amps(case["init"]), _kat.to_ops(case["gates"]))
        cmp = case["cmp"]
        if family == "f64" and cmp == "exact":
            cmp = "fequal"  # FP64 math differs from the float literals in the last bits
        for idx, re, im in case["expect"]:
            v = complex(sv[idx])
            assert _kat.amp_ok(v, re, im, cmp, case["tol"] if cmp != "fequal" or case["cmp"] != "exact" else 1e-6), \
                (case["name"], idx, v, re, im)
    elif t in ("matrix_equal", "matrix_adjoint"):
        a = matrix_of(n, _kat.to_ops(case["a"]), family)
        b = matrix_of(n, _kat.to_ops(case["b"]), family)
        if t == "matrix_adjoint":
            a = a.conj().T
        if case["cmp"] == "exact" and family != "f64":
            assert np.array_equal(a, b), case["name"]
        else:
            assert np.max(np.abs(a - b)) < max(case["tol"], 1e-12 if family == "f64" else 1e-6)
    elif t == "peek_measure_all":
        sv = FAMILIES[family](n, _kat.init_amps(case["init"]), _kat.to_ops(case["gates"]))
        if family == "ref32":
            assert oracle.ref32_peek_measure_all(sv, 0.5) == case["expect"]
        p = oracle.probs(np.ascontiguousarray(sv))
        assert oracle.first_index(p, 0.5) == case["expect"]
    elif t == "marginals":
        sv = oracle.ref32_product_state(_kat.init_amps(case["init"]))
        for q, e in enumerate(case["expect"]):
            if family == "ref32":
                got = oracle.ref32_qubit_probability_true(sv, q)
            else:
                got = oracle.qubit_prob_f64(sv.astype(np.complex128), q)
            if case["cmp"] == "exact":
                assert abs(got - e) <= (0 if family == "ref32" else 1e-7), (q, got, e)
            else:
                assert _kat.fequal(got, e, case["tol"]), (q, got, e)
    elif t == "statevector_equal":
        a = oracle.ref32_product_state(_kat.init_amps(case["init_a"]))
        b = FAMILIES[family](n, _kat.init_amps(case["init_b"]), _kat.to_ops(case["gates"]))
        tol = max(case["tol"], 1e-7 if family == "f64" else 0.0)
        assert np.max(np.abs(a - b)) <= tol, (a, b)
    elif t == "collapse":
        sv = oracle.ref32_product_state(_kat.init_amps(case["init"])).astype(np.complex128)
        q = case["qubit"]
        p1 = oracle.qubit_prob_f64(sv, q)
        m = 1 << (n - 1 - q)
        idx = np.arange(1 << n)
        for outcome, expect in case["branches"].items():
            keep = ((idx & m) != 0) == (outcome == "1")
            p = p1 if outcome == "1" else 1 - p1
            out = np.where(keep, sv / np.sqrt(p), 0)
            for k, re, im in expect:
                assert _kat.amp_ok(complex(out[k]), re, im, "fequal", case["tol"])
    else:
        raise AssertionError(t)


def test_qstate_normalisation():
    """QState constructor / normalisation known answers, tests.cpp:42-110."""
    q = oracle.ref32_qstate(0.6, 0.8j)
    assert q[0] == np.float32(0.6) and q[3] == np.float32(0.8)
    q = oracle.ref32_qstate(3, 4)
    assert q[0] == np.float32(0.6) and q[2] == np.float32(0.8)
    q = oracle.ref32_qstate(1 + 2j, 3 + 4j)
    v = np.array([1, 2, 3, 4], dtype=np.float32)
    mag = np.float32(np.sqrt(np.float32(np.float32(np.float32(v[0] * v[0]) + v[1] * v[1]) + v[2] * v[2]) + v[3] * v[3]))
    assert np.array_equal(q, v / mag)
    with pytest.raises(ValueError):
        oracle.ref32_qstate(0, 0)
