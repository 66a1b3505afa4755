"""Builds the CPU oracle (liboracle.so) with gcc.  TEST INFRASTRUCTURE.

``-ffp-contract=off`` is essential: without it gcc on aarch64 fuses
multiply-adds, and the oracle's FP32 ray arithmetic would stop matching the
device bit for bit.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
BUILD_DIR = ORACLE_DIR / "_build"
LIB = BUILD_DIR / "liboracle.so"
SOURCES = [ORACLE_DIR / "rt_oracle.c"]
DEPS = SOURCES + [ORACLE_DIR / "rt_oracle.h", ORACLE_DIR / "rt_oracle_shade.inc",
                  ORACLE_DIR.parent / "include" / "rtcore.h", Path(__file__)]
CFLAGS = ["-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
          "-fno-strict-aliasing", "-pthread", "-Wall"]


def build(force: bool = False) -> Path:
    if not force and LIB.exists() and all(d.stat().st_mtime <= LIB.stat().st_mtime for d in DEPS):
        return LIB
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["gcc", *CFLAGS, "-o", str(tmp), *map(str, SOURCES), "-lm"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
