"""Build recipes for the oracle (test infrastructure only).

build_oracle()  compiles oracle/emt6_oracle.c -> oracle/_build/liborc.so.
build_ref()     compiles the reference's own host-side sources where they lie
                (only when the reference checkout is present) together with
                oracle/ref_shim.cc -> oracle/_ref/libemt6_ref.so.  It never
                copies reference sources; outputs go to oracle/_ref/ only.

Both are plain gcc/g++ invocations (no cmake, no reference build system).
Every float expression is compiled with -ffp-contract=off so the oracle
evaluates exactly what its source says on x86-64 and aarch64 alike.
"""
from __future__ import annotations

import os
import platform
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
REFERENCE_ROOT = Path(os.environ.get("EMT6_REFERENCE_ROOT", "/root/reference"))
CUDA_INC = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "include"

ORACLE_LIB = BUILD / "liborc.so"
REF_LIB = REF_OUT / "libemt6_ref.so"


def _arch_flags() -> list[str]:
    # fmaf() must be a hardware instruction for speed; both ISAs round it
    # identically (IEEE fused multiply-add), so results do not depend on it.
    return ["-mfma"] if platform.machine() in ("x86_64", "AMD64") else []


def _run(cmd: list[str]) -> None:
    subprocess.run(cmd, check=True)


def _stale(out: Path, srcs: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(s.stat().st_mtime > t for s in srcs)


def build_oracle(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    srcs = [HERE / "emt6_oracle.c", HERE / "emt6_oracle.h"]
    if force or _stale(ORACLE_LIB, srcs):
        tmp = ORACLE_LIB.with_suffix(".so.tmp")
        _run(["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", *_arch_flags(), "-fPIC",
              "-shared", "-o", str(tmp), str(HERE / "emt6_oracle.c"), "-lm", "-lpthread"])
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def reference_available() -> bool:
    return (REFERENCE_ROOT / "src" / "emt6ro" / "cell" / "cell.cu").exists()


def build_ref(force: bool = False) -> Path | None:
    """Reference host code + shim; returns None when the reference is absent."""
    if not reference_available():
        return None
    REF_OUT.mkdir(exist_ok=True)
    src = REFERENCE_ROOT / "src"
    ref_srcs = [src / "emt6ro/cell/cell.cu", src / "emt6ro/parameters/parameters.cc",
                src / "emt6ro/state/state.cc", src / "emt6ro/common/random-engine.cc"]
    mine = [HERE / "ref_shim.cc", HERE / "emt6_oracle.c", HERE / "emt6_oracle.h"]
    if not (force or _stale(REF_LIB, ref_srcs + mine)):
        return REF_LIB
    inc = ["-I", str(src), "-I", str(REFERENCE_ROOT / "third-party" / "json"),
           "-I", str(CUDA_INC), "-I", str(HERE)]
    common = ["-O2", "-DNDEBUG", "-ffp-contract=off", "-fPIC"]
    objs = []
    for s in ref_srcs:
        o = REF_OUT / (s.stem + ".o")
        lang = ["-x", "c++"] if s.suffix == ".cu" else []
        _run(["g++", "-std=c++14", *common, *inc, *lang, "-c", str(s), "-o", str(o)])
        objs.append(o)
    o = REF_OUT / "ref_shim.o"
    _run(["g++", "-std=c++14", *common, *inc, "-c", str(HERE / "ref_shim.cc"), "-o", str(o)])
    objs.append(o)
    o = REF_OUT / "orc_refmode.o"
    _run(["gcc", "-std=gnu11", *common, "-DORC_REF_CELL", "-I", str(HERE), "-c",
          str(HERE / "emt6_oracle.c"), "-o", str(o)])
    objs.append(o)
    tmp = REF_LIB.with_suffix(".so.tmp")
    _run(["g++", "-shared", "-o", str(tmp), *map(str, objs), "-lm", "-lpthread"])
    os.replace(tmp, REF_LIB)
    return REF_LIB


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref(force=True))
