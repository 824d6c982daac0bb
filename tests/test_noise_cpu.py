"""Noise by trajectories, on the CPU: the engine's sampler
(aqsg_noise_trajectory) draws exactly what its restatement draws, inserts
Paulis at the requested rates, validates its inputs, and its trajectories,
run one by one by the FP64 oracle, average to the density-matrix oracle's
expectations."""
import numpy as np
import pytest

import afquantumsim_gb300 as aq
from oracle import noise as onoise
from oracle import oracle


def small_circuit(n, seed):
    rng = np.random.default_rng(seed)
    ops = []
    for _ in range(3):
        for q in range(n):
            ops.append(aq.RotY(q, float(np.float32(rng.uniform(-np.pi, np.pi)))))
            ops.append(aq.RotZ(q, float(np.float32(rng.uniform(-np.pi, np.pi)))))
        ops += [aq.CX(i, i + 1) for i in range(n - 1)]
    ops.append(aq.CCNot(0, 1, 2))
    ops.append(aq.H(1, controls=[2]))
    return ops


@pytest.mark.parametrize("seed,traj", [(1, 0), (1, 7), (99, 123456), (2**63 + 5, 3)])
def test_sampler_matches_restatement(seed, traj):
    n = 4
    ops = small_circuit(n, 3)
    p1, p2 = (0.05, 0.02, 0.08), (0.1, 0.05, 0.03)
    got = aq.noise_trajectory(n, ops, aq.Noise.pauli(p1, p2), seed, traj)
    draws = onoise.trajectory_kinds(ops, p1, p2, seed, traj)
    want = []  # (kind, first qubit) of each op: every source gate, then the Paulis drawn after it
    for g, op in enumerate(ops):
        want.append((op.kind, op.qubits[0]))
        want += [(kind, q) for gg, q, kind in draws if gg == g]
    assert [(o.kind, o.qubits[0]) for o in got] == want
    assert len(draws) > 0


def test_insertion_rates():
    n = 3
    ops = [aq.H(0), aq.CX(0, 1), aq.CCNot(0, 1, 2)]
    p1, p2 = (0.1, 0.05, 0.2), (0.02, 0.3, 0.1)
    counts = np.zeros((2, 3))
    T = 20000
    for t in range(T):
        for g, q, kind in onoise.trajectory_kinds(ops, p1, p2, 11, t):
            counts[0 if g == 0 else 1, [aq.kinds.X, aq.kinds.Y, aq.kinds.Z].index(kind)] += 1
    # gate 0 touches 1 qubit, gates 1 and 2 touch 2 + 3 qubits
    rate1, rate2 = counts[0] / T, counts[1] / (5 * T)
    assert np.all(np.abs(rate1 - p1) < 5 * np.sqrt(np.array(p1) / T) + 1e-3)
    assert np.all(np.abs(rate2 - p2) < 5 * np.sqrt(np.array(p2) / (5 * T)) + 1e-3)
    # the C sampler agrees on a few of them
    nz = aq.Noise.pauli(p1, p2)
    for t in range(5):
        got = aq.noise_trajectory(n, ops, nz, 11, t)
        assert len(got) == len(ops) + len(onoise.trajectory_kinds(ops, p1, p2, 11, t))


def test_noise_arguments_are_checked():
    ops = [aq.H(0)]
    with pytest.raises(aq.InvalidArgument):
        aq.noise_trajectory(2, ops, aq.Noise.pauli((-0.1, 0, 0)), 1, 0)
    with pytest.raises(aq.InvalidArgument):
        aq.noise_trajectory(2, ops, aq.Noise.pauli((0.5, 0.4, 0.2)), 1, 0)
    with pytest.raises(aq.OutOfRange):
        aq.noise_trajectory(2, [aq.H(3)], aq.Noise.depolarizing(0.1, 0.1), 1, 0)
    assert len(aq.noise_trajectory(2, ops, aq.Noise.depolarizing(0.0, 0.0), 5, 9)) == 1


def test_trajectory_mean_matches_density_matrix():
    """The unravelling itself: T trajectories run by the FP64 per-gate
    oracle average to the density-matrix expectations within 5 standard
    errors."""
    n, T = 3, 3000
    ops = small_circuit(n, 4)
    p1, p2 = (0.03, 0.02, 0.04), (0.05, 0.05, 0.05)
    z_exact, zz_exact = onoise.density_expect_z(n, ops, p1, p2)
    nz = aq.Noise.pauli(p1, p2)
    zs = np.zeros((T, n))
    idx = np.arange(1 << n)
    for t in range(T):
        v = np.zeros(1 << n, dtype=np.complex128)
        v[0] = 1
        v = oracle.apply_f64(v, list(aq.noise_trajectory(n, ops, nz, 21, t)))
        p = np.abs(v) ** 2
        zs[t] = [np.sum(p * (1 - 2 * ((idx >> (n - 1 - q)) & 1))) for q in range(n)]
    mean, err = zs.mean(0), zs.std(0, ddof=1) / np.sqrt(T)
    assert np.all(np.abs(mean - z_exact) < 5 * err + 1e-3), (mean, z_exact, err)
    # and the channel matters here: the noiseless values are far away
    z_clean, _ = onoise.density_expect_z(n, ops, (0, 0, 0), (0, 0, 0))
    assert np.max(np.abs(z_clean - z_exact)) > 10 * np.max(err)
