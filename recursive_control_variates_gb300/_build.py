"""Builds librcv.so (the sm_103a CUDA library behind the C ABI in include/rcv.h).

The library is compiled in-tree into ``recursive_control_variates_gb300/_build``
with nvcc, one translation unit per process, then linked with the static CUDA
runtime.  ``-fmad=false`` keeps every float operation separately rounded, which
the tracers rely on for agreement with the CPU oracle.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
CSRC = PKG_DIR / "csrc"
BUILD_DIR = PKG_DIR / "_build"
INCLUDE = PKG_DIR.parent / "include"
LIB_NAME = "librcv.so"

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "-fmad=false",
    "--expt-relaxed-constexpr",
    "-Xcompiler",
    "-fPIC,-O3,-ffp-contract=off",
    f"-I{INCLUDE}",
]


def nvcc_path() -> str:
    cand = shutil.which("nvcc")
    if cand:
        return cand
    default = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(default):
        return default
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build librcv")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _digest() -> str:
    h = hashlib.sha256()
    for p in sorted(list(CSRC.glob("*")) + [INCLUDE / "rcv.h"]):
        if p.is_file():
            h.update(p.name.encode())
            h.update(p.read_bytes())
    h.update(" ".join(ARCH_FLAGS + NVCC_FLAGS).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def source_digest() -> str:
    """Digest of the CUDA sources and the C header only (the same on every
    machine): profile summaries record it, so that a figure captured from
    other sources is recognised as stale."""
    h = hashlib.sha256()
    for p in sorted(list(CSRC.glob("*")) + [INCLUDE / "rcv.h"]):
        if p.is_file():
            h.update(p.name.encode())
            h.update(p.read_bytes())
    return h.hexdigest()[:16]


def lib_path() -> Path:
    return BUILD_DIR / LIB_NAME


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile librcv.so if the sources changed; returns the library path."""
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    stamp = BUILD_DIR / "stamp.txt"
    digest = _digest()
    out = lib_path()
    if not force and out.exists() and stamp.exists() and stamp.read_text() == digest:
        return out
    nvcc = nvcc_path()
    objs = []

    def compile_one(src: Path) -> Path:
        obj = BUILD_DIR / (src.stem + ".o")
        cmd = [nvcc, *ARCH_FLAGS, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")
        if verbose and res.stderr:
            print(res.stderr)
        return obj

    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 1))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = out.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH_FLAGS, "-shared", "-o", str(tmp), *map(str, objs), "-Xcompiler", "-fPIC"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, out)
    stamp.write_text(digest)
    return out


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
