"""Build the in-tree shared libraries.

    python -m mara3p_gb300.build          # libmara_gb300.so (+ the oracle if asked)

libmara_gb300.so holds every CUDA kernel and the C ABI declared in
include/mara_gb300.h. Each .cu translation unit is compiled for sm_103a only
(one -gencode), in parallel, then linked with nvcc -shared. Outputs land next
to this file and are git-ignored.
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
OBJ = PKG / "_build"
LIB = PKG / "libmara_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17",
    "-Xcompiler", "-fPIC,-ffp-contract=off",
    f"-I{ROOT / 'include'}",
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build mara_gb300")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)


def build_library(verbose: bool = False) -> Path:
    sources = sorted(CSRC.glob("*.cu"))
    headers = sorted(CSRC.glob("*.cuh")) + sorted((ROOT / "include").glob("*.h"))
    OBJ.mkdir(exist_ok=True)
    newest_header = max((h.stat().st_mtime for h in headers), default=0.0)
    cc = nvcc()

    def compile_one(src: Path) -> Path:
        obj = OBJ / (src.stem + ".o")
        if obj.exists() and obj.stat().st_mtime >= max(src.stat().st_mtime, newest_header):
            return obj
        _run([cc, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)])
        if verbose:
            print(f"[build] {src.name}", flush=True)
        return obj

    with ThreadPoolExecutor(max_workers=min(len(sources), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, sources))
    if not LIB.exists() or LIB.stat().st_mtime < max(o.stat().st_mtime for o in objs):
        _run([cc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"])
        if verbose:
            print(f"[build] {LIB.name}", flush=True)
    return LIB


DRIVER_SRC = Path(__file__).resolve().parent / "driver" / "mara_minidisk.cpp"
DRIVER = Path(__file__).resolve().parent / "mara_minidisk"


def build_driver(verbose: bool = False) -> Path:
    """The C++17 minidisk driver (problems/minidisk.cpp's main loop) on the C
    ABI, linked against libmara_gb300.so next to it."""
    if DRIVER.exists() and DRIVER.stat().st_mtime >= max(DRIVER_SRC.stat().st_mtime, LIB.stat().st_mtime,
                                                         (ROOT / "include" / "mara_gb300.h").stat().st_mtime):
        return DRIVER
    _run([nvcc(), "-std=c++17", "-O2", "-I", str(ROOT / "include"), str(DRIVER_SRC), "-L", str(LIB.parent),
          "-lmara_gb300", "-lcudart", "-Xlinker", "-rpath,$ORIGIN", "-o", str(DRIVER)])
    if verbose:
        print(f"[build] {DRIVER.name}", flush=True)
    return DRIVER


def build_oracle(reference: bool = False) -> None:
    """Compile oracle/ (test infrastructure) with make; reference=True also
    builds oracle/_ref from the reference checkout when one is present (the
    Makefile's REF variable names where; the MARA_REF environment variable
    overrides it)."""
    _run(["make", "-s", "-C", str(ROOT / "oracle")])
    if reference:
        ref = os.environ.get("MARA_REF")
        _run(["make", "-s", "-C", str(ROOT / "oracle"), "ref-if-present", *([f"REF={ref}"] if ref else [])])


if __name__ == "__main__":
    build_library(verbose=True)
    build_driver(verbose=True)
    if "--oracle" in sys.argv:
        build_oracle(reference=True)
