"""The batch plan image checked on the CPU (aqsg_debug_batch_image): what
aqsg_batch_update writes in place, on all host threads, equals what
aqsg_batch_create builds for the same circuits; each small circuit's ops sit
in its size class's table with their pool offsets moved to the class pool,
and the tile-record restatement runs them there to the FP64 oracle's state;
an update with another structure is refused.  The device runs of the same
batches are covered by the GPU batch tests."""
import numpy as np
import pytest

import afquantumsim_gb300 as aq
from afquantumsim_gb300 import circuits
from oracle import oracle
from tests import _kat
from tests.tile_emulator import run_plan

NS = [6, 9, 11, 12, 14, 15, 16, 16, 17]
LAYERS = 3


def sweep(seed, ns=NS, layers=LAYERS):
    rng = np.random.default_rng(seed)
    return [(n, circuits.vqe_ops_array(n, layers, rng.uniform(-np.pi, np.pi, size=(layers, n, 2)))) for n in ns]


def as_ops(a):
    return list((aq.Op * len(a)).from_buffer_copy(np.ascontiguousarray(a).tobytes()))


@pytest.mark.parametrize("fuse,tc", [([0, 0, 0, 0], [0, 0, 0, 0]), ([0, 2, 4, 5], [0, 0, 1, 1]),
                                     ([3, 3, 3, 3], [1, 1, 1, 1]), ([2, 5, 5, 2], [0, 1, 1, 0])])
def test_update_writes_the_created_image(fuse, tc):
    a, b = sweep(1), sweep(2)
    img_a = aq.debug_batch_image(a, fuse, tc)
    img_b = aq.debug_batch_image(b, fuse, tc)
    assert len(img_a) == len(img_b) and img_a != img_b
    assert aq.debug_batch_image(a, fuse, tc, update=b) == img_b
    assert aq.debug_batch_image(a, fuse, tc, update=a) == img_a


def test_update_with_many_circuits_on_all_threads():
    """More circuits than one host thread's chunk: the parallel writes land
    in their own slots."""
    ns = [int(n) for n in np.random.default_rng(3).integers(5, 18, size=96)]
    large = sum(n > 14 for n in ns)
    fuse, tc = [2 + k % 4 for k in range(large)], [k % 2 for k in range(large)]
    a, b = sweep(4, ns, 2), sweep(5, ns, 2)
    assert aq.debug_batch_image(a, fuse, tc, update=b) == aq.debug_batch_image(b, fuse, tc)


def test_class_table_runs_to_the_oracle_state():
    """Small circuits of one size class share a table and a pool: each one's
    ops, run from its place there, give the oracle's state."""
    rng = np.random.default_rng(11)

    def dense(qs):
        d = 1 << len(qs)
        return aq.Unitary(qs, np.linalg.qr(rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d)))[0])

    cs = [(12, _kat.random_circuit(12, 60, s) + [dense([1, 5]), dense([0, 3, 7])]) for s in range(3)]
    cs.append((11, _kat.random_circuit(11, 40, 9) + [dense([2, 4, 9])]))
    image = aq.debug_batch_image(cs)
    plans = [aq.debug_tile_plan(n, ops, aq.C64, 0) for n, ops in cs]
    ttotal = sum(len(t) for _, t, _ in plans)
    poff = (ttotal + 255) & ~255
    first, pbase = 0, 0
    for (n, ops), (passes, table, pool) in zip(cs, plans):
        assert len(passes) == 1 and passes[0].m == n  # one whole-register pass
        passes[0].first = first // 160
        v = _kat.random_state(n, 7)
        got = run_plan(v, n, passes, image[:ttotal], image[poff:], c64=True)
        assert np.max(np.abs(got - oracle.apply_f64(v.copy(), ops))) < 1e-5
        # the circuit's own pool at its base; its own records where the base is 0
        assert len(pool) > 0 and image[poff + pbase:poff + pbase + len(pool)] == pool
        if pbase == 0:
            assert image[first:first + len(table)] == table
        first += len(table)
        pbase = (pbase + len(pool) + 255) & ~255


def test_large_plan_image_is_the_encoded_plan():
    """A lone register of more than 14 qubits: its image is its tile plan,
    table then pool at the next 256-byte boundary."""
    n = 16
    ops = as_ops(sweep(6, [n])[0][1])
    for fuse in (0, 2, 3):
        passes, table, pool = aq.debug_tile_plan(n, ops, aq.C64, fuse)
        image = aq.debug_batch_image([(n, ops)], [fuse], [0])
        poff = (len(table) + 255) & ~255
        assert image[:len(table)] == table
        assert image[poff:poff + len(pool)] == pool
        v = _kat.random_state(n, 2)
        got = run_plan(v, n, passes, image[:len(table)], image[poff:], c64=True)
        assert np.max(np.abs(got - oracle.apply_f64(v.copy(), ops))) < 1e-5


@pytest.mark.parametrize("fuse", [3, 4, 5])
def test_tensor_core_plan_after_update_runs_to_the_oracle(fuse):
    """A register of more than 14 qubits on the tensor cores: after an update
    with new angles its image is the new circuit's tensor-core plan in the
    batched engine's form, and the tile-record restatement (split-BF16
    operands decoded from the image) runs it to the oracle's state."""
    n = 16
    a, b = sweep(6, [n]), sweep(7, [n])
    image = aq.debug_batch_image(a, [fuse], [1], update=b)
    ops = as_ops(b[0][1])
    passes, table, pool = aq.debug_tile_plan(n, ops, aq.C64, fuse, tensor_cores=2)
    assert all(p.tc for p in passes)
    poff = (len(table) + 255) & ~255
    assert image[:len(table)] == table and image[poff:poff + len(pool)] == pool
    v = _kat.random_state(n, 2)
    got = run_plan(v, n, passes, image[:len(table)], image[poff:], c64=True)
    assert np.max(np.abs(got - oracle.apply_f64(v.copy(), ops))) < 1e-5


def test_update_refuses_another_structure():
    a = sweep(1)
    fuse, tc = [2, 2, 3, 4], [0, 0, 1, 1]
    deeper = sweep(2, NS, LAYERS + 1)
    with pytest.raises(aq.InvalidArgument, match="structure changed"):
        aq.debug_batch_image(a, fuse, tc, update=deeper)
    other_n = sweep(2, NS[:-1] + [18])
    with pytest.raises(aq.InvalidArgument, match="qubit count"):
        aq.debug_batch_image(a, fuse, tc, update=other_n)
    # a dense two-qubit unitary in place of a CX of a small register
    b = sweep(2)
    ops = as_ops(b[3][1])
    k = next(i for i, o in enumerate(ops) if o.kind == aq._abi.CX)
    u = np.linalg.qr(np.random.default_rng(1).normal(size=(4, 4)) + 1j * np.random.default_rng(2).normal(size=(4, 4)))[0]
    ops[k] = aq.Unitary([ops[k].qubits[0], ops[k].qubits[1]], u)
    b[3] = (b[3][0], ops)
    with pytest.raises(aq.InvalidArgument, match="structure changed"):
        aq.debug_batch_image(a, fuse, tc, update=b)
