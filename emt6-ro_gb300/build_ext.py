"""Build the sm_103a CUDA library libemt6ro_gb300.so in-tree.

    python emt6-ro_gb300/build_ext.py

Four translation units (step kernels, host engine + C ABI, the
allocation-free entry point, the surrogate MLP) compiled in parallel by nvcc
for sm_103a only, then linked into emt6ro/_lib/libemt6ro_gb300.so next
to the Python package that loads it.  --fmad=false and -ffp-contract=off make
every floating-point expression round exactly as written.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
INCLUDE = HERE.parent / "include"
OUT_DIR = HERE / "emt6ro" / "_lib"
LIB = OUT_DIR / "libemt6ro_gb300.so"
OBJ_DIR = HERE / "_build"
SOURCES = ["emt6_kernels.cu", "emt6_host.cu", "emt6_noalloc.cu", "surrogate.cu"]
HEADERS = ["emt6_device.cuh", "emt6_kernels.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
         "-I", str(INCLUDE)]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = [CSRC / s for s in SOURCES + HEADERS] + [INCLUDE / "emt6ro_gb300.h",
                                                     INCLUDE / "emt6ro_surrogate.h", Path(__file__)]
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    if not (force or stale()):
        return LIB
    OUT_DIR.mkdir(parents=True, exist_ok=True)
    OBJ_DIR.mkdir(exist_ok=True)
    cc = nvcc()
    procs = []
    objs = []
    for s in SOURCES:
        o = OBJ_DIR / (Path(s).stem + ".o")
        objs.append(o)
        cmd = [cc, *ARCH, *FLAGS, "-c", str(CSRC / s), "-o", str(o)]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if verbose or p.returncode:
            sys.stderr.write(out.decode(errors="replace"))
        if p.returncode:
            raise RuntimeError("nvcc failed: " + " ".join(cmd))
    tmp = LIB.with_suffix(".so.tmp")
    subprocess.run([cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
