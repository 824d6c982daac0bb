"""The oracle's restatement of QSimulator::set_basis (src/quantum.cpp:416-465):
the float form of the reference's algorithm (dense Kronecker operator)
agrees with the FP64 form for every change of basis, the matrices are the
reference's (z_to_x, z_to_y read row-major, x_to_z their inverse), and the
missing break at :443 makes leaving Y use the X-to-Z matrix.  CPU only; the
GPU side is tests/cpp/test_set_basis.cpp."""
import numpy as np
import pytest

from oracle import oracle

Z, Y, X = oracle.BASIS_Z, oracle.BASIS_Y, oracle.BASIS_X
h = 0.70710678118
Z_TO_X = np.array([[h, h], [h, -h]])
Z_TO_Y = np.array([[h, h], [-1j * h, 1j * h]])
X_TO_Z = np.linalg.inv(Z_TO_X)


def product_state(n, seed):
    rng = np.random.default_rng(seed)
    v = np.ones(1, dtype=np.complex128)
    for _ in range(n):
        q = rng.standard_normal(2) + 1j * rng.standard_normal(2)
        v = np.kron(v, q / np.linalg.norm(q))
    return v


@pytest.mark.parametrize("frm,to,want", [
    (Z, X, Z_TO_X), (Z, Y, Z_TO_Y), (X, Z, X_TO_Z),
    (Y, Z, X_TO_Z),                       # the fall-through: not inv(Z_TO_Y)
    (X, Y, Z_TO_Y @ X_TO_Z), (Y, X, Z_TO_X @ X_TO_Z),
])
def test_basis_matrices(frm, to, want):
    assert np.allclose(oracle.ref32_basis_matrix(frm, to), want, atol=1e-6)


def test_leaving_y_is_not_the_inverse_of_entering_it():
    m = oracle.ref32_basis_matrix(Y, Z) @ oracle.ref32_basis_matrix(Z, Y)
    assert not np.allclose(m, np.eye(2), atol=1e-2)
    assert np.allclose(oracle.ref32_basis_matrix(X, Z) @ oracle.ref32_basis_matrix(Z, X), np.eye(2), atol=1e-6)


@pytest.mark.parametrize("frm", [Z, Y, X])
@pytest.mark.parametrize("to", [Z, Y, X])
def test_float_algorithm_matches_fp64(frm, to):
    n = 5
    v = product_state(n, 10 * frm + to)
    a = oracle.ref32_set_basis(v.astype(np.complex64), frm, to)
    b = oracle.set_basis_f64(v.copy(), frm, to)
    m = np.eye(2) if frm == to else oracle.ref32_basis_matrix(frm, to).astype(np.complex128)
    full = np.ones((1, 1))
    for _ in range(n):
        full = np.kron(full, m)
    assert np.max(np.abs(a - b)) < 1e-6
    assert np.max(np.abs(b - full @ v)) < 1e-6


def test_z_to_x_on_zero_state_is_uniform():
    n = 4
    v = np.zeros(1 << n, dtype=np.complex64)
    v[0] = 1
    oracle.ref32_set_basis(v, Z, X)
    assert np.allclose(v, 0.25, atol=1e-6)
