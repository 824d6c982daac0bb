"""Pauli-string expectation values (aqsg_expect_pauli) against dense
Kronecker products (small n) and the mask formula in numpy FP64 (n = 20);
a Hamiltonian's energy from its Pauli decomposition equals <psi|H|psi>."""
import itertools

import numpy as np
import pytest

import afquantumsim_gb300 as aq
from tests import _kat

pytestmark = pytest.mark.gpu

PAULI = {"i": np.eye(2), "x": np.array([[0, 1], [1, 0]]), "y": np.array([[0, -1j], [1j, 0]]),
         "z": np.diag([1, -1])}


def dense(s):
    m = np.ones((1, 1))
    for ch in s:  # letter j = qubit j = index bit n-1-j: the first Kronecker factor
        m = np.kron(m, PAULI[ch.lower()])
    return m


def masks_expect(v, s):
    n = len(s)
    x = z = ny = 0
    for j, ch in enumerate(s.lower()):
        b = 1 << (n - 1 - j)
        if ch in "xy":
            x |= b
        if ch in "yz":
            z |= b
        ny += ch == "y"
    k = np.arange(v.size, dtype=np.int64)
    par = np.zeros(v.size, dtype=np.int64)
    zz = k & z
    while np.any(zz):
        par ^= zz & 1
        zz >>= 1
    sign = 1 - 2 * par
    return (1j ** ny) * np.sum(sign * np.conj(v[k ^ x]) * v)


def random_strings(n, count, rng):
    return ["".join(rng.choice(list("ixyz"), size=n)) for _ in range(count)]


@pytest.mark.parametrize("n", [1, 3, 6, 10])
@pytest.mark.parametrize("dtype", [aq.C64, aq.C128])
def test_pauli_against_dense(gpu_ctx, n, dtype):
    rng = np.random.default_rng(n)
    v = _kat.random_state(n, n + 1)
    strings = random_strings(n, 21, rng) + ["i" * n, "Y" * n, "x" * n]
    npdt = np.complex64 if dtype == aq.C64 else np.complex128
    vd = v.astype(npdt).astype(np.complex128)
    want = np.array([np.vdot(vd, dense(s) @ vd) for s in strings])
    with aq.State(gpu_ctx, n, dtype) as st:
        st.upload(v.astype(npdt))
        got = st.expect_pauli(strings)
    tol = 1e-6 if dtype == aq.C64 else 1e-12
    assert np.max(np.abs(got - want)) < tol
    assert abs(got[len(strings) - 3] - np.vdot(vd, vd)) < tol


def test_pauli_twenty_qubits_mask_formula(gpu_ctx):
    n = 20
    rng = np.random.default_rng(7)
    v = _kat.random_state(n, 3)
    strings = random_strings(n, 11, rng)
    strings += ["z" * n, "i" * (n - 1) + "x", "x" + "i" * (n - 1), strings[0].replace("x", "y")]
    with aq.State(gpu_ctx, n, aq.C128) as st:
        st.upload(v)
        got = st.expect_pauli(strings)
    want = np.array([masks_expect(v, s) for s in strings])
    assert np.max(np.abs(got - want)) < 1e-12


def test_hamiltonian_energy_from_decomposition(gpu_ctx):
    n = 4
    rng = np.random.default_rng(1)
    a = rng.standard_normal((16, 16)) + 1j * rng.standard_normal((16, 16))
    H = (a + a.conj().T) / 2
    strings, coeffs = [], []
    for t in itertools.product("ixyz", repeat=n):
        s = "".join(t)
        c = np.trace(dense(s).conj().T @ H) / 16
        if abs(c) ** 2 > 1e-12:
            strings.append(s)
            coeffs.append(c)
    v = _kat.random_state(n, 9)
    with aq.State(gpu_ctx, n, aq.C128) as st:
        st.upload(v)
        vals = st.expect_pauli(strings)
    assert abs(np.dot(coeffs, vals) - np.vdot(v, H @ v)) < 1e-11


def test_pauli_rejects_bad_letters(gpu_ctx):
    with aq.State(gpu_ctx, 3, aq.C64) as st:
        st.set_basis(0)
        with pytest.raises(aq.InvalidArgument):
            st.expect_pauli(["xqz"])
        with pytest.raises(aq.InvalidArgument):
            st.expect_pauli(["xz"])
        assert st.expect_pauli(["zzz"])[0] == 1.0
