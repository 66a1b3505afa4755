"""Builds librtcore.so (the C-ABI ray-tracing core) for sm_103a with nvcc.

The library is compiled in-tree into ``_build/`` next to this file.  Each
``.cu`` translation unit is compiled in parallel, then linked with the static
CUDA runtime, exporting only the ``rt_*`` symbols of ``include/rtcore.h``.
Every unit is compiled with ``-fmad=false``: the ray-generation, transform and
triangle-test arithmetic must round after every operation, in the order the
source gives, to match the CPU oracle bit for bit.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
CSRC = PKG_DIR / "csrc"
BUILD_DIR = PKG_DIR / "_build"
INCLUDE_DIR = PKG_DIR.parent / "include"
LIB_NAME = "librtcore.so"
SOURCES = ["rt_api.cu", "rt_build.cu", "rt_trace.cu", "rt_serve.cu", "rt_assets.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "-fmad=false",
    "-prec-div=true",
    "-prec-sqrt=true",
    "-ftz=false",
    "-Xcompiler",
    "-fPIC,-fvisibility=hidden,-O2",
    "-I" + str(INCLUDE_DIR),
]


def nvcc_path() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build librtcore")


def library_path() -> Path:
    return BUILD_DIR / LIB_NAME


def _inputs() -> list[Path]:
    files = [CSRC / s for s in SOURCES]
    files += sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h"))
    files += sorted(INCLUDE_DIR.glob("*.h")) + [Path(__file__)]
    return files


def _up_to_date(out: Path) -> bool:
    if not out.exists():
        return False
    t = out.stat().st_mtime
    return all(f.stat().st_mtime <= t for f in _inputs())


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> Path:
    """Compiles and links librtcore.so; returns its path."""
    out = library_path()
    if not force and not extra_flags and _up_to_date(out):
        return out
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    nvcc = nvcc_path()
    flags = NVCC_FLAGS + (extra_flags or [])
    procs = []
    objs = []
    for src in SOURCES:
        obj = BUILD_DIR / (Path(src).stem + ".o")
        objs.append(obj)
        cmd = [nvcc, *ARCH, *flags, "-c", str(CSRC / src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd))
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    errors = []
    for src, p in procs:
        log, _ = p.communicate()
        if verbose and log:
            print(log)
        if p.returncode != 0:
            errors.append(f"{src}:\n{log}")
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    tmp = out.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", str(tmp), *map(str, objs)]
    if verbose:
        print(" ".join(cmd))
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc link failed:\n" + r.stdout)
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
