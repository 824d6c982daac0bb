"""The C-ABI library: loads, exports every declared symbol, struct layout
matches the header, and op validation reproduces the reference's check()
exceptions and messages.  No GPU needed (no compute calls)."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

import afquantumsim_gb300 as aq
from afquantumsim_gb300 import _abi

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    text = "".join(h.read_text() for h in sorted((ROOT / "include").glob("*.h")))
    return sorted(set(re.findall(r"^\s*(?:int|size_t)\s+(aqsg_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol():
    lib = aq.load_library()
    names = declared_symbols()
    assert len(names) >= 25
    for name in names:
        assert hasattr(lib, name), name
    assert set(aq.EXPORTS) == set(names)


def test_struct_layout_matches_header(tmp_path):
    src = tmp_path / "layout.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "aqsg.h"\n'
                   'int main(void){printf("%zu %zu %zu %zu %zu\\n", sizeof(aqsg_op),'
                   ' offsetof(aqsg_op, angle), offsetof(aqsg_op, qubits),'
                   ' offsetof(aqsg_op, controls), offsetof(aqsg_op, matrix)); return 0;}\n')
    exe = tmp_path / "layout"
    subprocess.run(["gcc", f"-I{ROOT / 'include'}", str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    O = _abi.Op
    assert got == [C.sizeof(O), O.angle.offset, O.qubits.offset, O.controls.offset,
                   O.matrix.offset]


def test_version():
    assert aq.load_library().aqsg_version() == 1


# (gate, n, expected exception, message) — the check() of each gate class,
# src/quantum.cpp:533-1886
CHECKS = [
    (aq.X(4), 4, aq.OutOfRange, "Cannot add gate at the given qubit position"),
    (aq.RotY(7, 0.3), 4, aq.OutOfRange, "Cannot add gate at the given qubit position"),
    (aq.Swap(0, 1), 1, aq.DomainError, "Gate not supported for given simulation"),
    (aq.Swap(1, 1), 3, aq.InvalidArgument, "Cannot use the swap gate on the same target qubits"),
    (aq.CX(2, 2), 3, aq.InvalidArgument, "Control qubit cannot be the same as the target qubit"),
    (aq.CZ(0, 5), 3, aq.OutOfRange, "Cannot add gate at the given qubit position"),
    (aq.CRotX(1, 1, 0.5), 3, aq.InvalidArgument, "Control qubit cannot be the same as the target qubit"),
    (aq.CSwap(0, 1, 2), 2, aq.DomainError, "Gate not supported for given circuit"),
    (aq.CSwap(1, 1, 2), 3, aq.InvalidArgument, "Control qubit cannot be the same as the target qubit"),
    (aq.CSwap(0, 2, 2), 3, aq.InvalidArgument, "Cannot use the swap gate on the same target qubits"),
    (aq.CCNot(0, 1, 1), 3, aq.InvalidArgument, "Control qubit cannot be the same as the target qubit"),
    (aq.Or(0, 1, 2), 2, aq.DomainError, "Gate not supported for given simulation"),
    (aq.X(1, controls=[1]), 3, aq.OutOfRange,
     "Control qubit cannot be one of the target qubits of the gate"),
    (aq.X(1, controls=[5]), 3, aq.OutOfRange, "Control qubit must be inside the circuit qubit range"),
]


@pytest.mark.parametrize("op,n,exc,msg", CHECKS)
def test_check_messages(op, n, exc, msg):
    with pytest.raises(exc) as e:
        aq.check_ops(n, [op])
    assert e.value.msg == msg


def test_valid_ops_pass_check():
    aq.check_ops(5, aq.fourier_transform(5, swaps=True))
    aq.check_ops(3, [aq.CCNot(0, 0, 2), aq.Or(1, 1, 0), aq.Barrier()])  # as the reference allows
