"""The integer-pipe binary64 add and multiply (csrc/softfp64.cuh) give the
same bits as IEEE 754 round-to-nearest-even hardware arithmetic: the header
compiled for the host against the host's FP unit on ~14 million operand
pairs of every class (tests/cpp/softfp64_check.cpp)."""
from __future__ import annotations

import pathlib
import shutil
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
CSRC = ROOT / "high-order-accurate-cfd-solver-code-for-heterogenous-hardware-cpu-and-gpgpu-_gb300" / "csrc"


def test_soft_add_mul_bit_exact_on_host(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "softfp64_check"
    subprocess.run([cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-I", str(CSRC),
                    str(ROOT / "tests" / "cpp" / "softfp64_check.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe), "2000000", "7"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " 0 mismatches" in r.stdout
