"""Build ``libneb_gb300.so`` in-tree with nvcc for sm_103a (GB300).

Each translation unit under ``csrc/`` is compiled in parallel, then linked
with cuSOLVER / cuBLAS (FP64 eigensolve and small FP64 GEMMs).  The library
is written next to this file; ``neb_gb300._native`` loads it from there.

    python -m neb_gb300.build          # or neb_gb300.build.build()
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = PKG / "libneb_gb300.so"
SOURCES = ["abi.cu", "spectral.cu", "spectral_mixed.cu", "tc_path.cu", "modes.cu", "peel.cu",
           "rollout.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found (set $NVCC)")


def cuda_lib_dir(exe: str) -> str:
    base = Path(exe).resolve().parent.parent
    for sub in ("lib64", "lib", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib"):
        if (base / sub / "libcusolver.so").exists() or (base / sub).exists():
            return str(base / sub)
    return str(base / "lib64")


def flags(extra=()) -> list[str]:
    return [*ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
            f"-I{INCLUDE}", f"-I{CSRC}", "--expt-relaxed-constexpr", *extra]


def build(verbose: bool = False, ptxas_info: bool = False) -> Path:
    exe = nvcc()
    BUILD.mkdir(exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []

    def compile_one(src: str) -> tuple[str, str]:
        obj = BUILD / (Path(src).stem + ".o")
        cmd = [exe, *flags(extra), "-c", str(CSRC / src), "-o", str(obj)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{res.stderr}")
        return str(obj), res.stderr

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as pool:
        results = list(pool.map(compile_one, SOURCES))
    for _, log in results:
        if log and (verbose or ptxas_info):
            sys.stderr.write(log)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [exe, *ARCH, "-shared", "-o", str(tmp), *[o for o, _ in results],
           f"-L{cuda_lib_dir(exe)}", "-lcusolver", "-lcublas", "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv))
