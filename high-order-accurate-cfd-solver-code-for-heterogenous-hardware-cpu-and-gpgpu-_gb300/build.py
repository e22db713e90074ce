"""Builds libcfd_gb300.so (CUDA, sm_103a) in-tree with nvcc.

Each .cu under csrc/ is compiled to an object in parallel, then linked into
one shared library next to this file.  Only the sm_103a target is generated.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess
import sys

PKG = pathlib.Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
LIB = PKG / "libcfd_gb300.so"
OBJ_DIR = PKG / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I" + str(INCLUDE), "-I" + str(CSRC)]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcfd_gb300.so")


# Translation units whose FP64 arithmetic must follow the reference's
# evaluation order: no contraction of a*b+c into FMA.
EXACT_FP64 = {"dropin.cu", "structured.cu", "batch_fp64.cu", "boundary.cu", "face_fp64_mb2.cu", "face_fp64_mb3.cu",
              "face_fp64_mb4.cu"}
# Translation units of the mixed and split precision forms: approximate FP32
# division and square root (single-precision only; FP64 arithmetic is
# unaffected) and FMA contraction.
FAST_FP32 = {"mixed.cu", "batch_mixed.cu", "split.cu", "batch_split.cu"}


# Translation units whose host code follows the reference's evaluation order
# (the geometry producer): no FMA contraction of host arithmetic either.
EXACT_HOST = {"geometry.cu"}


def sources() -> list[pathlib.Path]:
    return sorted(CSRC.glob("*.cu"))


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*")) + list(INCLUDE.glob("*.h")) + [pathlib.Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> pathlib.Path:
    """Compile every csrc/*.cu for sm_103a and link libcfd_gb300.so.  Extra
    nvcc flags may be passed in the CFD_NVCC_EXTRA environment variable."""
    if not force and not _stale():
        return LIB
    cc = nvcc()
    OBJ_DIR.mkdir(exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []

    def compile_one(src: pathlib.Path):
        obj = OBJ_DIR / (src.stem + ".o")
        fmad = ["--fmad=false"] if src.name in EXACT_FP64 else []
        if src.name in FAST_FP32:
            fmad += ["--prec-div=false", "--prec-sqrt=false"]
        if src.name in EXACT_HOST:
            fmad += ["-Xcompiler", "-ffp-contract=off"]
        user = os.environ.get("CFD_NVCC_EXTRA", "").split()
        cmd = [cc, *ARCH, *NVCC_FLAGS, *fmad, *extra, *user, "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        return src, obj, r

    objs = []
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        for src, obj, r in ex.map(compile_one, sources()):
            if verbose or ptxas_info or r.returncode != 0:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {src.name}")
            objs.append(str(obj))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, *ARCH, "-shared", "-o", str(tmp), *objs, "-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("nvcc link failed")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
