"""Build libcvb.so (the C-ABI library) in-tree with nvcc for sm_103a.

Each translation unit compiles in parallel into curvib_old_gb300/_build/, then
links into curvib_old_gb300/_build/libcvb.so.  Rebuilds only what changed.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
SRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libcvb.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-I", str(SRC), "-I", str(INCLUDE)] + ARCH


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (cand == "nvcc" or Path(cand).exists()):
            return cand
    raise FileNotFoundError("nvcc not found")


def _sources():
    return sorted(list(SRC.glob("*.cu")) + list(SRC.glob("*.cpp")))


def _headers_mtime():
    hs = list(SRC.glob("*.h")) + list(SRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    return max((h.stat().st_mtime for h in hs), default=0.0)


# Files whose arithmetic must round operation by operation as the reference's
# C does: no multiply-add contraction.
PER_FILE_FLAGS = {"kernels_momentum.cu": ["--fmad=false"]}


def _compile(src: Path, extra) -> Path:
    obj = OUT / (src.stem + ".o")
    if obj.exists() and obj.stat().st_mtime > max(src.stat().st_mtime, _headers_mtime()):
        return obj
    extra = list(extra) + PER_FILE_FLAGS.get(src.name, [])
    cmd = [nvcc()] + NVCC_FLAGS + list(extra) + ["-c", str(src), "-o", str(obj)]
    if src.suffix == ".cpp":
        cmd = [nvcc(), "-x", "cu"] + NVCC_FLAGS + list(extra) + ["-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError(f"nvcc failed on {src.name}")
    return obj


def build(verbose: bool = False, extra=()) -> Path:
    OUT.mkdir(exist_ok=True)
    srcs = _sources()
    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    newest = max(o.stat().st_mtime for o in objs)
    if not LIB.exists() or LIB.stat().st_mtime < newest:
        cmd = [nvcc()] + ARCH + ["-shared", "-o", str(LIB)] + [str(o) for o in objs] + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link of libcvb.so failed")
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
