"""Noise by trajectories on the GPU: aqsg_noise_expect_z runs the
trajectories as one batch; each trajectory's expectations equal the FP64
oracle of that trajectory's circuit, and their mean matches the FP64
density-matrix expectations of the noisy circuit within 5 standard errors
(the errors the call itself reports)."""
import numpy as np
import pytest

import afquantumsim_gb300 as aq
from oracle import noise as onoise
from oracle import oracle
from tests.test_noise_cpu import small_circuit

pytestmark = pytest.mark.gpu


def test_noisy_expectations_match_density_matrix(gpu_ctx):
    n, T, seed = 5, 8192, 31
    ops = small_circuit(n, 6)
    p1, p2 = (0.02, 0.01, 0.03), (0.04, 0.02, 0.04)
    nz = aq.Noise.pauli(p1, p2)
    z, zz, ze, zze = aq.noisy_expect_z(gpu_ctx, n, ops, nz, seed, T)
    z_exact, zz_exact = onoise.density_expect_z(n, ops, p1, p2)
    assert np.all(ze > 0) and np.all(ze < 2 / np.sqrt(T))
    assert np.all(np.abs(z - z_exact) < 5 * ze + 1e-4), (z, z_exact, ze)
    assert np.all(np.abs(zz - zz_exact) < 5 * zze + 1e-4), (zz, zz_exact, zze)
    z_clean, _ = onoise.density_expect_z(n, ops, (0, 0, 0), (0, 0, 0))
    assert np.max(np.abs(z_clean - z_exact)) > 10 * np.max(ze)


def test_each_trajectory_is_exact(gpu_ctx):
    """A batch of explicit trajectories: every register's <Z> equals the FP64
    oracle of its circuit, and the batch mean equals aqsg_noise_expect_z."""
    n, T, seed = 6, 64, 5
    ops = small_circuit(n, 7)
    nz = aq.Noise.depolarizing(0.05, 0.08)
    trajs = [(n, aq.noise_trajectory(n, ops, nz, seed, t)) for t in range(T)]
    b = aq.Batch(gpu_ctx, trajs)
    z, zz = b.run()
    b.free()
    idx = np.arange(1 << n)
    for t in range(0, T, 9):
        v = np.zeros(1 << n, dtype=np.complex128)
        v[0] = 1
        v = oracle.apply_f64(v, list(trajs[t][1]))
        p = np.abs(v) ** 2
        want = np.array([np.sum(p * (1 - 2 * ((idx >> (n - 1 - q)) & 1))) for q in range(n)])
        assert np.max(np.abs(np.asarray(z[t]) - want)) < 1e-5
    zm, _, _, _ = aq.noisy_expect_z(gpu_ctx, n, ops, nz, seed, T)
    assert np.max(np.abs(np.mean(np.array(z), axis=0) - zm)) < 1e-12
