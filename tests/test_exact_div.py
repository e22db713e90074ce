"""Shared-reciprocal division and power-of-two scaling (csrc/exact_div.cuh)
give the bits of IEEE division x / b and of the product x * 2^K: on the host
against the host's arithmetic (CPU), and on the GB300 against the GPU's own
(GPU), on ~9 million operand pairs per run including quotients within
~2^-53 ulp of a rounding midpoint and operands of every class, subnormal,
Inf and NaN included (tests/cpp/div_cases.h)."""
from __future__ import annotations

import pathlib
import shutil
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
CSRC = ROOT / "high-order-accurate-cfd-solver-code-for-heterogenous-hardware-cpu-and-gpgpu-_gb300" / "csrc"
CPP = ROOT / "tests" / "cpp"


@pytest.mark.parametrize("qprod", [0, 1])
def test_exact_division_on_host(tmp_path, qprod):
    """Both ways of forming the first quotient (CFD_XDIV_QPROD)."""
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "exact_div_check"
    subprocess.run([cxx, "-std=c++17", "-O2", "-ffp-contract=off", f"-DCFD_XDIV_QPROD={qprod}", "-I", str(CSRC),
                    "-I", str(CPP), str(CPP / "exact_div_check.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe), "1000000", "11"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " 0 mismatches" in r.stdout and " 0 scale2 mismatches" in r.stdout and " 0 pow2_over mismatches" in r.stdout
    assert " 0 rcp mismatches" in r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("qprod", [0, 1])
def test_exact_division_on_gpu(tmp_path, qprod):
    from cfd_gb300 import build
    exe = tmp_path / "exact_div_gpu"
    subprocess.run([build.nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "--fmad=false",
                    f"-DCFD_XDIV_QPROD={qprod}", "-I", str(CSRC), "-I", str(CPP), str(CPP / "exact_div_gpu.cu"),
                    "-o", str(exe)], check=True)
    r = subprocess.run([str(exe), "1000000", "12"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " 0 mismatches" in r.stdout and " 0 scale2 mismatches" in r.stdout and " 0 pow2_over mismatches" in r.stdout
    assert " 0 rcp mismatches" in r.stdout
