"""Build recipe for the CPU oracle (test infrastructure, not product code).

Compiles ``oracle/rcv_oracle.cpp`` into ``oracle/_build/liboracle.so`` with
``-ffp-contract=off`` so that float operations are rounded one at a time, the
same way the GPU library (built with ``-fmad=false``) rounds them.

The reference itself (rgl-epfl/recursive_control_variates) is pure Python on
top of Mitsuba 3 / Dr.Jit, which are not vendored and not installed, so there
is no reference source to compile here: this recipe builds only the
restatement.
"""
from __future__ import annotations

import hashlib
import os
import subprocess
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
BUILD_DIR = ORACLE_DIR / "_build"
SRCS = [ORACLE_DIR / "rcv_oracle.cpp", ORACLE_DIR / "rcv_oracle_surface.cpp"]
LIB = BUILD_DIR / "liboracle.so"
# Tuned for the host it is built on (-mcpu=native on Arm, -march=native on
# x86): the build runs on every machine that uses it.  -ffp-contract=off and
# -fno-fast-math keep one rounding per float operation, so the native tuning
# changes speed only, never a result.
NATIVE = ["-mcpu=native"] if os.uname().machine in ("aarch64", "arm64") else ["-march=native"]
FLAGS = ["-O3", *NATIVE, "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread"]


def flags_text() -> str:
    """Compiler and flags of the build, as the CPU baseline reports them."""
    return f"{os.environ.get('CXX', 'g++')} " + " ".join(f for f in FLAGS if f not in ("-fPIC", "-shared"))


def build(force: bool = False) -> Path:
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    h = hashlib.sha256(b"".join(s.read_bytes() for s in SRCS) + " ".join(FLAGS).encode() + os.uname().machine.encode())
    stamp = BUILD_DIR / "stamp.txt"
    if not force and LIB.exists() and stamp.exists() and stamp.read_text() == h.hexdigest():
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [os.environ.get("CXX", "g++"), *FLAGS, *map(str, SRCS), "-o", str(tmp)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    stamp.write_text(h.hexdigest())
    return LIB


if __name__ == "__main__":
    print(build(force=True))
