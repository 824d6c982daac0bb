"""The aqs:: C++ layer (the reference-facing API) through compiled C++ test
programs: host-side logic on the CPU (lowering checked by the oracle), and
the restated assertions of the reference's test/tests.cpp on the GPU."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
BUILD = ROOT / "afquantumsim_gb300" / "_build"
ORACLE_BUILD = ROOT / "oracle" / "_build"


def compile_program(name: str, tmp_path: Path, with_oracle: bool) -> Path:
    from afquantumsim_gb300 import build as b
    b.build_all()
    exe = tmp_path / name
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", f"-I{ROOT / 'afquantumsim_gb300' / 'cpp'}",
           f"-I{ROOT / 'include'}", f"-I{ROOT / 'oracle'}", f"-I{ROOT / 'tests' / 'cpp'}",
           str(ROOT / "tests" / "cpp" / f"{name}.cpp"), f"-L{BUILD}", "-laqs", "-laqsg",
           f"-Wl,-rpath,{BUILD}", "-o", str(exe)]
    if with_oracle:
        cmd[-2:-2] = [f"-L{ORACLE_BUILD}", "-laqs_oracle", f"-Wl,-rpath,{ORACLE_BUILD}"]
    subprocess.run(cmd, check=True)
    return exe


def run_program(exe: Path) -> None:
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=900)
    print(res.stdout)
    assert res.returncode == 0, res.stderr + res.stdout


def test_host_api(tmp_path):
    run_program(compile_program("test_host_api", tmp_path, with_oracle=True))


@pytest.mark.gpu
def test_reference_suite_on_gpu(tmp_path):
    run_program(compile_program("test_reference_suite", tmp_path, with_oracle=False))


@pytest.mark.gpu
def test_set_basis_on_gpu(tmp_path):
    # QSimulator::set_basis for Z->X, Z->Y, X->Z, Y->Z, X->Y, Y->X against the
    # oracle's restatement (including the fall-through of the reference's
    # missing break), full state vector
    run_program(compile_program("test_set_basis", tmp_path, with_oracle=True))
