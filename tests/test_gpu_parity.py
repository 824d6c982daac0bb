"""GPU parity: the CUDA engine (through the C ABI) against the CPU oracle and
the reference's known answers.

Tolerances: permutation gates bit-exact; c64 within 1e-5 absolute of the
FP64 oracle (1e-6 of the FP32 oracle); c128 within 1e-12 of the FP64 oracle.
"""
import numpy as np
import pytest

import afquantumsim_gb300 as aq
from oracle import oracle
from tests import _kat

pytestmark = pytest.mark.gpu

MODES = [aq.EXEC_PER_GATE, aq.EXEC_TILED]
DTYPES = [(aq.C64, np.complex64), (aq.C128, np.complex128)]
TOL64 = 1e-5
TOL128 = 1e-12


def run(ctx, sv, ops, dtype, mode):
    n = int(sv.size).bit_length() - 1
    with aq.State(ctx, n, dtype) as st:
        st.upload(sv)
        st.apply(ops, mode)
        return st.download()


# ---- known answers of test/tests.cpp ------------------------------------------------

CASES = _kat.load_cases()
AMP = [c for c in CASES if c["type"] == "amplitudes"]


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("case", AMP, ids=[c["name"] for c in AMP])
def test_golden_amplitudes(gpu_ctx, case, mode):
    n = case["n"]
    amps = _kat.init_amps(case["init"])
    for dtype, _ in DTYPES:
        with aq.State(gpu_ctx, n, dtype) as st:
            st.set_product(amps)
            st.apply(_kat.to_ops(case["gates"]), mode)
            sv = st.download()
        cmp = case["cmp"] if dtype == aq.C64 else ("fequal" if case["cmp"] == "exact" else case["cmp"])
        tol = case["tol"] if cmp == case["cmp"] else 1e-6
        for idx, re, im in case["expect"]:
            assert _kat.amp_ok(complex(sv[idx]), re, im, cmp, tol), (case["name"], dtype, idx, sv[idx])


def gpu_matrix(ctx, n, ops, dtype, mode):
    cols = []
    for k in range(1 << n):
        with aq.State(ctx, n, dtype) as st:
            st.set_basis(k)
            st.apply(ops, mode)
            cols.append(st.download())
    return np.stack(cols, axis=1)


MAT = [c for c in CASES if c["type"] in ("matrix_equal", "matrix_adjoint")]


@pytest.mark.parametrize("case", MAT, ids=[c["name"] for c in MAT])
def test_golden_matrices(gpu_ctx, case):
    n = case["n"]
    for mode in MODES:
        a = gpu_matrix(gpu_ctx, n, _kat.to_ops(case["a"]), aq.C64, mode)
        b = gpu_matrix(gpu_ctx, n, _kat.to_ops(case["b"]), aq.C64, mode)
        if case["type"] == "matrix_adjoint":
            a = a.conj().T
        if case["cmp"] == "exact":
            assert np.array_equal(a, b)
        else:
            assert np.max(np.abs(a - b)) < case["tol"]
        # and the circuit matrix equals the faithful restatement's compile()
        ref = oracle.ref32_compile(n, _kat.to_ops(case["b"]))
        assert np.max(np.abs(b - ref)) < 1e-6


@pytest.mark.parametrize("case", [c for c in CASES if c["type"] == "peek_measure_all"],
                         ids=lambda c: c["name"])
def test_golden_peek(gpu_ctx, case):
    with aq.State(gpu_ctx, case["n"], aq.C64) as st:
        st.set_product(_kat.init_amps(case["init"]))
        st.apply(_kat.to_ops(case["gates"]))
        assert int(st.sample([0.5])[0]) == case["expect"]


@pytest.mark.parametrize("case", [c for c in CASES if c["type"] == "marginals"],
                         ids=lambda c: c["name"])
def test_golden_marginals(gpu_ctx, case):
    with aq.State(gpu_ctx, case["n"], aq.C64) as st:
        st.set_product(_kat.init_amps(case["init"]))
        for q, e in enumerate(case["expect"]):
            got = st.qubit_prob(q)
            if case["cmp"] == "exact":
                assert abs(got - e) < 1e-7
            else:
                assert _kat.fequal(got, e, case["tol"])


def test_golden_collapse(gpu_ctx):
    case = [c for c in CASES if c["type"] == "collapse"][0]
    for u, branch in ((0.0, "1"), (0.999, "0")):
        with aq.State(gpu_ctx, case["n"], aq.C64) as st:
            st.set_product(_kat.init_amps(case["init"]))
            outcome, p = st.collapse_qubit(case["qubit"], u)
            assert str(outcome) == branch
            sv = st.download()
        for k, re, im in case["branches"][branch]:
            assert _kat.amp_ok(complex(sv[k]), re, im, "fequal", case["tol"])


def test_product_state_bit_exact(gpu_ctx):
    """set_product reproduces the reference's Kronecker chain in float."""
    rng = np.random.default_rng(5)
    n = 11
    amps = np.concatenate([oracle.ref32_qstate(complex(*rng.standard_normal(2)),
                                               complex(*rng.standard_normal(2)))
                           for _ in range(n)])
    with aq.State(gpu_ctx, n, aq.C64) as st:
        st.set_product(amps)
        got = st.download()
    assert np.array_equal(got, oracle.ref32_product_state(amps))


# ---- every gate kind at every placement ---------------------------------------------

PERM = {"X", "Swap", "CX", "CSwap", "CCNot", "Or"}


def placements(kind, n):
    import itertools
    ar = aq._abi.ARITY[_kat._KIND[kind]]
    return [p for p in itertools.permutations(range(n), ar)]


@pytest.mark.parametrize("kind", sorted(_kat._KIND))
def test_every_gate_every_placement(gpu_ctx, kind):
    n = 5
    v = _kat.random_state(n, 17)
    for qs in placements(kind, n):
        for extra in ([], [q for q in range(n) if q not in qs][:1]):
            op = aq.make_op(_kat._KIND[kind], qs, angle=0.7312, controls=extra)
            want64 = oracle.apply_f64(v.copy(), [op])
            want32 = oracle.apply_f32(v.astype(np.complex64), [op])
            for mode in MODES:
                g64 = run(gpu_ctx, v.astype(np.complex64), [op], aq.C64, mode)
                g128 = run(gpu_ctx, v.copy(), [op], aq.C128, mode)
                if kind in PERM:
                    assert np.array_equal(g64, want32), (kind, qs, extra)
                    assert np.array_equal(g128, want64), (kind, qs, extra)
                else:
                    assert np.max(np.abs(g64 - want32)) < 1e-6, (kind, qs, extra)
                    assert np.max(np.abs(g64 - want64)) < TOL64
                    assert np.max(np.abs(g128 - want64)) < TOL128, (kind, qs, extra)


@pytest.mark.parametrize("k", [1, 2, 3, 4, 5])
def test_unitary_gates(gpu_ctx, k):
    n = 8
    rng = np.random.default_rng(k)
    v = _kat.random_state(n, 23)
    for trial in range(4):
        qs = [int(x) for x in rng.choice(n, size=k, replace=False)]
        m = np.linalg.qr(rng.standard_normal((1 << k, 1 << k)) + 1j * rng.standard_normal((1 << k, 1 << k)))[0]
        free = [q for q in range(n) if q not in qs]
        ctl = [int(x) for x in rng.choice(free, size=min(2, len(free)), replace=False)] if trial % 2 else []
        op = aq.Unitary(qs, m, controls=ctl, control_values=int(rng.integers(1 << len(ctl))) if ctl else None)
        want = oracle.apply_f64(v.copy(), [op])
        for mode in MODES:
            assert np.max(np.abs(run(gpu_ctx, v.astype(np.complex64), [op], aq.C64, mode) - want)) < TOL64
            assert np.max(np.abs(run(gpu_ctx, v.copy(), [op], aq.C128, mode) - want)) < TOL128


@pytest.mark.parametrize("n,depth,seed", [(6, 200, 1), (10, 300, 2), (13, 300, 3), (14, 300, 5), (16, 200, 4), (20, 120, 6)])
def test_random_circuits(gpu_ctx, n, depth, seed):
    ops = _kat.random_circuit(n, depth, seed)
    v = _kat.random_state(n, seed)
    want = oracle.apply_f64(v.copy(), ops)
    for mode in MODES:
        assert np.max(np.abs(run(gpu_ctx, v.astype(np.complex64), ops, aq.C64, mode) - want)) < TOL64
        assert np.max(np.abs(run(gpu_ctx, v.copy(), ops, aq.C128, mode) - want)) < TOL128


def test_permutation_circuit_bit_exact(gpu_ctx):
    """X, CX, CCX, Swap, CSwap, Or move amplitudes without arithmetic."""
    n = 14
    ops = _kat.random_circuit(n, 400, 9, kinds=sorted(PERM))
    v = _kat.random_state(n, 9)
    for mode in MODES:
        assert np.array_equal(run(gpu_ctx, v.astype(np.complex64), ops, aq.C64, mode),
                              oracle.apply_f32(v.astype(np.complex64), ops))
        assert np.array_equal(run(gpu_ctx, v.copy(), ops, aq.C128, mode),
                              oracle.apply_f64(v.copy(), ops))


def test_reference_algorithm_parity_12q(gpu_ctx):
    """The reference's own algorithm (faithful FP32 restatement) and the
    engine agree on the 12-qubit plain-method workload: H layer, then 10
    layers of seeded random RX/RY/RZ + CX chain."""
    n = 12
    rng = np.random.default_rng(1)
    ops = [aq.H(q) for q in range(n)]
    for _ in range(10):
        for q in range(n):
            kind = [aq.RotX, aq.RotY, aq.RotZ][int(rng.integers(3))]
            ops.append(kind(q, float(np.float32(rng.uniform(0, 2 * np.pi)))))
        ops += [aq.CX(i, i + 1) for i in range(n - 1)]
    v = np.zeros(1 << n, dtype=np.complex64)
    v[0] = 1
    ref = oracle.ref32_apply(v.copy(), n, ops)
    for mode in MODES:
        with aq.State(gpu_ctx, n, aq.C64) as st:
            st.set_basis(0)
            st.apply(ops, mode)
            got = st.download()
        assert np.max(np.abs(got - ref)) < 1e-5


# ---- large registers: size-independent properties --------------------------------------

def _bitrev(x, n):
    idx = np.arange(1 << n)
    r = np.zeros_like(idx)
    for b in range(n):
        r |= ((idx >> b) & 1) << (n - 1 - b)
    return x[r]


@pytest.mark.parametrize("dtype,npdt,tol", [(aq.C64, np.complex64, 1e-6), (aq.C128, np.complex128, 1e-8)])
def test_qft_24_matches_fft(gpu_ctx, dtype, npdt, tol):
    """24-qubit QFT with swaps equals sqrt(N) * bitrev(ifft(bitrev(v))) (the
    float angles pi/2^k cost ~1e-7 against the exact DFT)."""
    n = 24
    v = _kat.random_state(n, 3)
    want = _bitrev(np.fft.ifft(_bitrev(v, n)) * np.sqrt(1 << n), n)
    for mode in MODES:
        got = run(gpu_ctx, v.astype(npdt), aq.fourier_transform(n, swaps=True), dtype, mode)
        assert np.max(np.abs(got - want)) < tol


def test_qft_24_c128_vs_oracle(gpu_ctx):
    n = 24
    v = _kat.random_state(n, 4)
    ops = aq.fourier_transform(n, swaps=True)
    want = oracle.apply_f64(v.copy(), ops)
    got = run(gpu_ctx, v.copy(), ops, aq.C128, aq.EXEC_PER_GATE)
    assert np.max(np.abs(got - want)) < TOL128


def test_qft_roundtrip_28(gpu_ctx):
    """QFT followed by its inverse returns the input (28 qubits, c64)."""
    n = 28
    rng = np.random.default_rng(8)
    v = (rng.standard_normal(1 << n, dtype=np.float32)
         + 1j * rng.standard_normal(1 << n, dtype=np.float32)).astype(np.complex64)
    v /= np.float32(np.sqrt(np.sum(np.abs(v.astype(np.complex128)) ** 2)))  # FP64 norm
    fwd = aq.fourier_transform(n, swaps=True)
    inv = []
    for o in reversed(fwd):
        if o.kind == aq.kinds.CPHASE:
            inv.append(aq.CPhase(o.qubits[0], o.qubits[1], -o.angle))
        else:
            inv.append(o)
    with aq.State(gpu_ctx, n, aq.C64) as st:
        st.upload(v)
        st.apply(fwd, aq.EXEC_PER_GATE)
        assert abs(st.norm2() - 1.0) < 1e-5
        st.apply(inv, aq.EXEC_PER_GATE)
        got = st.download()
    assert np.max(np.abs(got - v)) < 1e-5


# ---- measurement ----------------------------------------------------------------------

@pytest.mark.parametrize("n", [3, 12, 17])
def test_probabilities_and_marginals(gpu_ctx, n):
    v = _kat.random_state(n, n)
    p = oracle.probs(v)
    for dtype, npdt in DTYPES:
        with aq.State(gpu_ctx, n, dtype) as st:
            st.upload(v.astype(npdt))
            tol = 1e-6 if dtype == aq.C64 else 1e-12
            assert np.max(np.abs(st.probs() - oracle.probs(v.astype(npdt)))) < 1e-12
            assert abs(st.norm2() - 1) < tol
            for q in range(n):
                assert abs(st.qubit_prob(q) - oracle.qubit_prob_f64(v.astype(npdt), q)) < 1e-12
            k = (1 << n) - 3
            assert abs(st.state_prob(k) - p[k]) < tol
            pf = st.probs(np.float32)
            assert np.max(np.abs(pf - p)) < 1e-6


@pytest.mark.parametrize("n", [1, 5, 12, 13, 18])
def test_sampling_matches_oracle_cdf(gpu_ctx, n):
    v = _kat.random_state(n, 100 + n)
    rng = np.random.default_rng(n)
    u = rng.random(3000)
    for dtype, npdt in DTYPES:
        sv = v.astype(npdt)
        p = oracle.probs(sv)
        cdf = np.cumsum(p)
        with aq.State(gpu_ctx, n, dtype) as st:
            st.upload(sv)
            got = st.sample(u)
        want = np.searchsorted(cdf, u, side="right")
        close = np.abs(cdf[np.minimum(want, len(cdf) - 1)] - u) < 1e-12
        assert np.all((got == want) | close)


def test_sampling_rules_and_seeded(gpu_ctx):
    from tests.test_oracle_cross import philox_uniform
    n = 9
    v = np.zeros(1 << n, dtype=np.complex64)
    v[5] = 0.6
    v[300] = 0.8j
    with aq.State(gpu_ctx, n, aq.C64) as st:
        st.upload(v)
        tot = st.norm2()
        # cdf: 0.6f^2 = 0.36000001 at index 5, then the total at index 300
        assert list(st.sample([0.0, 0.35, 0.37, 0.99])) == [5, 5, 300, 300]
        # above the total probability: the reference returns 0 (quantum.cpp:356)
        assert int(st.sample([tot + 1e-9], aq.SAMPLE_REFERENCE)[0]) == 0
        assert int(st.sample([tot + 1e-9], aq.SAMPLE_CLAMP)[0]) == 300
        seeded = st.sample_seeded(1234, 500)
        us = [philox_uniform(1234, i) for i in range(500)]
        assert np.array_equal(seeded, st.sample(us))


def test_sampling_statistics(gpu_ctx):
    """99.9% confidence band per outcome, as tests.cpp:343-406 checks."""
    n = 5
    amps = np.concatenate([oracle.ref32_qstate(1, 1), oracle.ref32_qstate(-2, 3),
                           oracle.ref32_qstate(0, 1), oracle.ref32_qstate(1, 0),
                           oracle.ref32_qstate(0.6j, 0.8)])
    reps = 10000
    with aq.State(gpu_ctx, n, aq.C64) as st:
        st.set_product(amps)
        counts = np.bincount(st.sample_seeded(42, reps).astype(np.int64), minlength=1 << n)
        p = st.probs()
    for k in range(1 << n):
        sd = np.sqrt(p[k] * (1 - p[k]))
        exp = reps * p[k]
        d = np.sqrt(reps) * 3.291 * sd
        assert exp - d - 1 <= counts[k] <= exp + d + 1


def test_collapse_all(gpu_ctx):
    n = 8
    v = _kat.random_state(n, 77, np.complex64)
    with aq.State(gpu_ctx, n, aq.C64) as st:
        st.upload(v)
        k = st.collapse_all(0.42)
        sv = st.download()
    want = int(np.searchsorted(np.cumsum(oracle.probs(v)), 0.42, side="right"))
    assert k == want and sv[k] == 1 and np.count_nonzero(sv) == 1


@pytest.mark.parametrize("n", [1, 2, 6, 12, 21, 23])
def test_expect_z(gpu_ctx, n):
    v = _kat.random_state(n, 300 + n)
    idx = np.arange(1 << n)
    for dtype, npdt in DTYPES:
        sv = v.astype(npdt)
        p = oracle.probs(sv)
        bits = [((idx >> (n - 1 - q)) & 1) for q in range(n)]
        wz = np.array([np.sum(p * (1 - 2 * b)) for b in bits])
        wzz = np.array([np.sum(p * (1 - 2 * (bits[q] ^ bits[q + 1]))) for q in range(n - 1)])
        with aq.State(gpu_ctx, n, dtype) as st:
            st.upload(sv)
            z, zz = st.expect_z()
        assert np.max(np.abs(z - wz)) < 1e-10
        if n > 1:
            assert np.max(np.abs(zz - wzz)) < 1e-10


def test_upload_normalises_and_rejects_null(gpu_ctx):
    with aq.State(gpu_ctx, 4, aq.C64) as st:
        st.upload(np.full(16, 2 + 0j, dtype=np.complex64), normalize=True)
        assert np.allclose(st.download(), 0.25)
        with pytest.raises(aq.InvalidArgument):
            st.upload(np.zeros(16, dtype=np.complex64), normalize=True)


def test_errors_on_device_calls(gpu_ctx):
    with aq.State(gpu_ctx, 3, aq.C64) as st:
        st.set_basis(0)
        with pytest.raises(aq.DomainError):
            aq.check_ops(2, [aq.CSwap(0, 1, 2)])
        with pytest.raises(aq.OutOfRange):
            st.qubit_prob(3)
        with pytest.raises(aq.OutOfRange):
            st.apply([aq.H(3)])
        with pytest.raises(aq.InvalidArgument):
            st.apply([aq.CX(1, 1)])
