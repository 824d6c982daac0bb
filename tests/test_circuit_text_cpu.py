"""Circuit text (aqsg_circuit_to_text / aqsg_circuit_from_text): the
reference's gate representation extended into a replayable format.  Checked
on the CPU: random circuits over every kind (extra controls, zero-controls,
unitaries) survive a round trip with the same FP64 oracle result and the
same canonical text; the reference's own strings (parameter-free gates, S/T
names, barriers) read as their gates; malformed text fails with the
reference's exception classes."""
import numpy as np
import pytest

import afquantumsim_gb300 as aq
from oracle import oracle
from tests import _kat


@pytest.mark.parametrize("n,seed", [(3, 1), (6, 2), (9, 3), (12, 4)])
def test_round_trip_random_circuits(n, seed):
    ops = _kat.random_circuit(n, 150, seed)
    text = aq.circuit_to_text(n, ops)
    n2, back = aq.circuit_from_text(text)
    assert n2 == n
    assert aq.circuit_to_text(n2, back) == text  # canonical
    v = _kat.random_state(n, seed)
    want = oracle.apply_f64(v.copy(), ops)
    got = oracle.apply_f64(v.copy(), list(back))
    np.testing.assert_array_equal(got, want)


def test_reference_strings_read_as_their_gates():
    n, ops = aq.circuit_from_text("4;X,0,1:3;X,1,1:0,2;X,2,1:0,1,3;Swap,0,2:1,3;H,1,1:0,1;"
                                  "Z,1,1:2,3;S,0,1:2;S†,0,1:1;T,0,1:0;T†,0,1:3;B;P;")
    assert n == 4
    want = [aq.X(3), aq.CX(0, 2), aq.CCNot(0, 1, 3), aq.Swap(1, 3), aq.CH(0, 1), aq.CZ(2, 3),
            aq.Phase(2, np.float32(np.pi) / 2), aq.Phase(1, -np.float32(np.pi) / 2),
            aq.Phase(0, np.float32(np.pi) / 4), aq.Phase(3, -np.float32(np.pi) / 4),
            aq.Barrier(), aq.Barrier()]
    assert aq.circuit_to_text(n, ops) == aq.circuit_to_text(4, want)
    v = _kat.random_state(4, 7)
    np.testing.assert_array_equal(oracle.apply_f64(v.copy(), list(ops)), oracle.apply_f64(v.copy(), want))


def test_zero_controls_and_whitespace():
    ops = [aq.X(2, controls=[0, 1], control_values=0b10), aq.RotY(1, 0.5, controls=[3], control_values=0)]
    text = aq.circuit_to_text(4, ops)
    assert text == "4;X,2,1:~0,1,2;RotY(0.5),1,1:~3,1;"
    n, back = aq.circuit_from_text(" 4 ;\n X,2,1:~0, 1,2 ;\tRotY(0.5),1,1:~3,1;\n")
    assert aq.circuit_to_text(n, back) == text


@pytest.mark.parametrize("text,exc,msg", [
    ("3;RotX,0,1:0;", aq.InvalidArgument, "needs its angle"),
    ("3;Foo,0,1:0;", aq.InvalidArgument, "unknown gate"),
    ("3;X,0,1:3;", aq.OutOfRange, "Cannot add gate at the given qubit position"),
    ("3;X,1,1:0;", aq.InvalidArgument, "does not match the counts"),
    ("3;X,0,1:0", aq.InvalidArgument, "must end with"),
    ("X,0,1:0;", aq.InvalidArgument, "qubit count"),
    ("3;U(1,0,0,0),0,2:0,1;", aq.InvalidArgument, "2 x 4^k"),
    ("3;H(0.5),0,1:0;", aq.InvalidArgument, "takes no parameter"),
    ("3;X,1,1:1,1;", aq.InvalidArgument, None),
])
def test_malformed_text(text, exc, msg):
    with pytest.raises(exc) as e:
        aq.circuit_from_text(text)
    if msg:
        assert msg in str(e.value)


def test_mutated_text_parses_or_fails_cleanly():
    """Random edits of valid texts (deleted, inserted, repeated or cut
    characters) either read as a circuit whose canonical text reads back to
    itself and whose ops pass the gate checks, or fail with an engine
    error; the parser never reads past its input."""
    rng = np.random.default_rng(17)
    bases = [aq.circuit_to_text(n, _kat.random_circuit(n, 12, s)) for n, s in [(3, 1), (5, 2), (7, 3)]]
    bases.append("4;X,0,1:3;X,1,1:0,2;Swap,0,2:1,3;S†,0,1:2;B;P;U(1,0,0,0,0,0,1,0),0,1:2;")
    alphabet = list("0123456789;:,.()~-+eE ") + ["RotX", "U(", "†", "\t", "\n", "1e308", "nan", "-0"]
    errors = aq.AqsgError
    parsed = failed = 0
    for trial in range(3000):
        t = bases[trial % len(bases)]
        for _ in range(int(rng.integers(1, 4))):
            i = int(rng.integers(0, len(t) + 1))
            op = int(rng.integers(0, 4))
            if op == 0 and t:
                t = t[:i] + t[i + 1:]
            elif op == 1:
                t = t[:i] + alphabet[int(rng.integers(len(alphabet)))] + t[i:]
            elif op == 2:
                j = min(len(t), i + int(rng.integers(1, 8)))
                t = t[:j] + t[i:j] + t[j:]
            else:
                t = t[:i]
        try:
            n, ops = aq.circuit_from_text(t)
        except errors:
            failed += 1
            continue
        parsed += 1
        aq.check_ops(n, list(ops))
        canon = aq.circuit_to_text(n, ops)
        n2, back = aq.circuit_from_text(canon)
        assert n2 == n and aq.circuit_to_text(n2, back) == canon
    assert parsed > 100 and failed > 100


def test_size_query_validates_like_the_parse():
    """The size query (ops NULL) refuses what the parse proper refuses."""
    import ctypes as C
    lib = aq.load_library()
    n, cnt, nd = C.c_int(), C.c_int(), C.c_size_t()
    for text in ["4;X,1,1:0,22;", "3;Swap,0,2:1,1;", "2;U(1,0,0,0,0,0,1,0),0,1:2;"]:
        rc = lib.aqsg_circuit_from_text(text.encode(), C.byref(n), None, 0, C.byref(cnt), None, 0, C.byref(nd))
        assert rc != 0
        with pytest.raises(aq.AqsgError):
            aq.circuit_from_text(text)
