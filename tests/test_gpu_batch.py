"""The batched engine (aqsg_batch_*): <Z_q> and <Z_q Z_q+1> of many
independent circuits of uneven size, against the FP64 oracle; parameter
updates; each result is the same alone and in the batch."""
import numpy as np
import pytest

import afquantumsim_gb300 as aq
from afquantumsim_gb300 import circuits
from oracle import oracle
from tests import _kat

pytestmark = pytest.mark.gpu


def oracle_z(n, ops):
    v = np.zeros(1 << n, dtype=np.complex128)
    v[0] = 1
    if len(ops):
        import ctypes as C
        if isinstance(ops, np.ndarray):
            ops = list((aq.Op * len(ops)).from_buffer_copy(ops.tobytes()))
        v = oracle.apply_f64(v, ops)
    p = np.abs(v) ** 2
    idx = np.arange(1 << n)
    bits = [((idx >> (n - 1 - q)) & 1) for q in range(n)]
    z = np.array([np.sum(p * (1 - 2 * b)) for b in bits])
    zz = np.array([np.sum(p * (1 - 2 * (bits[q] ^ bits[q + 1]))) for q in range(n - 1)])
    return z, zz


def test_batch_mixed_sizes_against_oracle(gpu_ctx):
    rng = np.random.default_rng(11)
    items = []
    for n in [3, 8, 10, 11, 12, 13, 14, 15, 16, 17, 20, 9, 14, 1, 2]:
        if rng.random() < 0.5 and n >= 2:
            ops = _kat.random_circuit(n, 60, int(rng.integers(1 << 30)),
                                      kinds=["X", "Y", "Z", "H", "RotX", "RotY", "RotZ", "CX", "CZ", "CPhase",
                                             "Swap", "CCNot", "U2"] if n >= 3 else ["H", "RotY", "X"])
        else:
            L = int(rng.integers(1, 5))
            ops = circuits.vqe_ops_array(n, L, rng.uniform(-np.pi, np.pi, size=(L, n, 2)))
        items.append((n, ops))
    b = aq.Batch(gpu_ctx, items)
    info = b.info()
    assert info["small"] + info["large"] == len(items) and info["large"] == 4
    z, zz = b.run()
    for (n, ops), zi, zzi in zip(items, z, zz):
        wz, wzz = oracle_z(n, ops)
        assert np.max(np.abs(zi - wz)) < 1e-5, n
        if n > 1:
            assert np.max(np.abs(zzi - wzz)) < 1e-5, n
    # second replay gives the same numbers
    z2, zz2 = b.run()
    assert all(np.array_equal(a, c) for a, c in zip(z, z2))
    b.free()


def test_batch_update_and_alone_vs_mix(gpu_ctx):
    rng = np.random.default_rng(3)
    shapes = [(9, 3), (12, 2), (14, 2), (16, 3), (18, 2)]
    def make():
        return [(n, circuits.vqe_ops_array(n, L, rng.uniform(-np.pi, np.pi, size=(L, n, 2))))
                for n, L in shapes]
    items = make()
    b = aq.Batch(gpu_ctx, items)
    b.run()
    new = make()
    b.update(new)
    z, zz = b.run()
    for (n, ops), zi in zip(new, z):
        assert np.max(np.abs(zi - oracle_z(n, ops)[0])) < 1e-5
    # alone: the same circuit as a one-item batch
    for k, (n, ops) in enumerate(new):
        alone = aq.Batch(gpu_ctx, [(n, ops)])
        za, zza = alone.run()
        assert np.max(np.abs(za[0] - z[k])) < 1e-12
        alone.free()
    with pytest.raises(aq.InvalidArgument):
        b.update(new[:-1] + [(new[-1][0], new[-1][1][:-1])])
    b.free()


def test_batch_groups_of_equal_structure(gpu_ctx):
    """Large registers with the same structure run as one group (one launch
    per tile pass for all of them): each matches the oracle and equals the
    same circuit run alone."""
    rng = np.random.default_rng(21)
    shapes = [(15, 3)] * 5 + [(16, 2)] * 3 + [(11, 2), (9, 3)]
    items = [(n, circuits.vqe_ops_array(n, L, rng.uniform(-np.pi, np.pi, size=(L, n, 2)))) for n, L in shapes]
    b = aq.Batch(gpu_ctx, items)
    z, zz = b.run()
    for (n, ops), zi, zzi in zip(items, z, zz):
        wz, wzz = oracle_z(n, ops)
        assert np.max(np.abs(zi - wz)) < 1e-5
        assert np.max(np.abs(zzi - wzz)) < 1e-5
    for k in (0, 4, 6):
        n, ops = items[k]
        alone = aq.Batch(gpu_ctx, [(n, ops)])
        za, _ = alone.run()
        assert np.max(np.abs(za[0] - z[k])) < 1e-12
        alone.free()
    b.free()


def test_batch_groups_on_tensor_cores(gpu_ctx):
    """VQE registers of 17 qubits tune to fused unitaries on the tensor
    cores; a group of them runs one persistent tensor-core launch per pass
    whose CTAs cross from one register's tiles into the next (reloading the
    operands): every register matches the oracle and equals the same circuit
    run alone."""
    rng = np.random.default_rng(7)
    shapes = [(17, 4)] * 6
    items = [(n, circuits.vqe_ops_array(n, L, rng.uniform(-np.pi, np.pi, size=(L, n, 2)))) for n, L in shapes]
    b = aq.Batch(gpu_ctx, items)
    info = b.info()
    assert info["large"] == 6 and all(info["tensor_cores"]), info
    z, zz = b.run()
    for (n, ops), zi, zzi in zip(items, z, zz):
        wz, wzz = oracle_z(n, ops)
        assert np.max(np.abs(zi - wz)) < 1e-5
        assert np.max(np.abs(zzi - wzz)) < 1e-5
    n, ops = items[3]
    alone = aq.Batch(gpu_ctx, [(n, ops)])
    za, zza = alone.run()
    np.testing.assert_array_equal(za[0], z[3])
    np.testing.assert_array_equal(zza[0], zz[3])
    alone.free()
    b.free()
