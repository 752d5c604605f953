"""Build recipe for the oracle's C restatement (test infrastructure only).

Compiles ``oracle/swe_oracle.c`` into ``oracle/_ref/liborc.so`` with
``-ffp-contract=off`` (no fused multiply-add: the reference's float64 arithmetic
rounds after every operation) and OpenMP for the CPU-baseline timing.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "swe_oracle.c"
OUT_DIR = HERE / "_ref"
LIB = OUT_DIR / "liborc.so"


def build(force: bool = False) -> Path:
    OUT_DIR.mkdir(exist_ok=True)
    if LIB.exists() and not force and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    tmp = OUT_DIR / f".liborc.{os.getpid()}.so"
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
           "-std=c11", str(SRC), "-o", str(tmp), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
