"""Build recipes for the oracle (test infrastructure only).

build_oracle()  compiles oracle/emt6_oracle.c -> oracle/_build/liborc.so.
build_oracle_fast()  compiles the same file for timing only (bench.py's CPU
                baseline) -> oracle/_build/liborc_fast.so: -O3 with FP
                contraction allowed.  Its results may differ from the
                checker's in the last bits; nothing checks against it.
build_ref()     compiles the reference's own host-side sources where they lie
                (only when the reference checkout is present) together with
                oracle/ref_shim.cc -> oracle/_ref/libemt6_ref.so.  It never
                copies reference sources; outputs go to oracle/_ref/ only.
build_ref_cubin()  compiles the reference's CUDA sources where they lie
                (src/emt6ro/{simulation,diffusion,statistics,cell,common}/*.cu,
                nvcc -dc, the reference's own CMake flags: C++14, relocatable
                device code) and device-links them into one sm_103a cubin,
                oracle/_ref/emt6ro_ref_sm103a.cubin (reference checkout only;
                the cubin holds device code alone, so it is the same file for
                any host architecture).
build_ref_cell_cubin()  compiles oracle/ref_cell_kernels.cu (kernels driving the
                reference's templated cell functions with injected draws)
                against the reference's headers, with its cell/cell.cu,
                nvcc defaults (FMA contraction, CUDA expf), device-linked
                into oracle/_ref/emt6ro_ref_cell_sm103a.cubin (reference
                checkout only; device code alone, like the cubin above).
build_ref_gpu_driver()  compiles oracle/ref_gpu_driver.cu, the host loop that
                launches those cubins' kernels -> oracle/_build/libref_gpu.so.

All are plain gcc/g++/nvcc invocations (no cmake, no reference build system).
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
# the reference checkout: $EMT6_REFERENCE_ROOT, else a sibling directory of
# this repository named "reference"
REFERENCE_ROOT = Path(os.environ.get("EMT6_REFERENCE_ROOT") or HERE.parent.parent / "reference")
CUDA_INC = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "include"

ORACLE_LIB = BUILD / "liborc.so"
ORACLE_FAST_LIB = BUILD / "liborc_fast.so"
REF_LIB = REF_OUT / "libemt6_ref.so"
REF_CUBIN = REF_OUT / "emt6ro_ref_sm103a.cubin"
REF_CELL_CUBIN = REF_OUT / "emt6ro_ref_cell_sm103a.cubin"
REF_GPU_LIB = BUILD / "libref_gpu.so"
NVCC = str(Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc")
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]


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
        _run(["gcc", "-O3", "-std=gnu11", "-ffp-contract=off", *_arch_flags(), "-fPIC",
              "-shared", "-o", str(tmp), str(HERE / "emt6_oracle.c"), "-lm", "-lpthread"])
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def fast_flags() -> list[str]:
    """The timing-only build: -O3 with FP contraction for the compiler's
    generic target of the host architecture (NEON on aarch64).  A
    -mcpu=neoverse-v2 build raised SIGILL on the GB300 machine's host, so no CPU
    tuning is applied."""
    return ["-O3", "-ffp-contract=fast", *_arch_flags()]


def build_oracle_fast(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    srcs = [HERE / "emt6_oracle.c", HERE / "emt6_oracle.h"]
    if force or _stale(ORACLE_FAST_LIB, srcs):
        tmp = ORACLE_FAST_LIB.with_suffix(".so.tmp")
        _run(["gcc", *fast_flags(), "-std=gnu11", "-fPIC", "-shared", "-o", str(tmp),
              str(HERE / "emt6_oracle.c"), "-lm", "-lpthread"])
        os.replace(tmp, ORACLE_FAST_LIB)
    return ORACLE_FAST_LIB


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
    common = ["-O3", "-DNDEBUG", "-ffp-contract=off", "-fPIC", *_arch_flags()]
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


def build_ref_cubin(force: bool = False) -> Path | None:
    """Reference device code -> one linked sm_103a cubin; None when absent."""
    if not reference_available():
        return REF_CUBIN if REF_CUBIN.exists() else None
    src = REFERENCE_ROOT / "src"
    cu = [src / "emt6ro" / f for f in ("simulation/simulation.cu", "diffusion/diffusion.cu",
                                      "statistics/statistics.cu", "common/random-engine.cu",
                                      "cell/cell.cu", "common/instr.cu")]
    if not (force or _stale(REF_CUBIN, cu)):
        return REF_CUBIN
    objdir = REF_OUT / "cu"
    objdir.mkdir(parents=True, exist_ok=True)
    inc = ["-I", str(src), "-I", str(REFERENCE_ROOT / "third-party" / "json")]
    from concurrent.futures import ThreadPoolExecutor
    objs = [objdir / (s.stem + ".o") for s in cu]
    with ThreadPoolExecutor(len(cu)) as ex:
        list(ex.map(lambda so: _run([NVCC, *GENCODE, "-dc", "-O3", "-DNDEBUG", "-std=c++14",
                                     *inc, "-Xcompiler", "-fPIC", "-w", str(so[0]), "-o",
                                     str(so[1])]), zip(cu, objs)))
    tmp = REF_OUT / "emt6ro_ref_sm103a.tmp.cubin"
    _run([NVCC, *GENCODE, "-dlink", "--cubin", "-o", str(tmp), *map(str, objs)])
    os.replace(tmp, REF_CUBIN)
    return REF_CUBIN


def build_ref_cell_cubin(force: bool = False) -> Path | None:
    """The reference's cell model driven by injected draws, device code ->
    one linked sm_103a cubin; None when the reference is absent."""
    if not reference_available():
        return REF_CELL_CUBIN if REF_CELL_CUBIN.exists() else None
    src = REFERENCE_ROOT / "src"
    cu = [HERE / "ref_cell_kernels.cu", src / "emt6ro" / "cell" / "cell.cu"]
    if not (force or _stale(REF_CELL_CUBIN, cu)):
        return REF_CELL_CUBIN
    objdir = REF_OUT / "cellcu"
    objdir.mkdir(parents=True, exist_ok=True)
    inc = ["-I", str(src), "-I", str(REFERENCE_ROOT / "third-party" / "json")]
    objs = [objdir / (s.stem + ".o") for s in cu]
    for so, o in zip(cu, objs):
        _run([NVCC, *GENCODE, "-dc", "-O3", "-DNDEBUG", "-std=c++14", *inc, "-Xcompiler",
              "-fPIC", "-w", str(so), "-o", str(o)])
    tmp = REF_OUT / "emt6ro_ref_cell_sm103a.tmp.cubin"
    _run([NVCC, *GENCODE, "-dlink", "--cubin", "-o", str(tmp), *map(str, objs)])
    os.replace(tmp, REF_CELL_CUBIN)
    return REF_CELL_CUBIN


def build_ref_gpu_driver(force: bool = False) -> Path:
    """Host loop for the reference's kernels (driver API) -> oracle/_build/libref_gpu.so."""
    BUILD.mkdir(exist_ok=True)
    srcs = [HERE / "ref_gpu_driver.cu", HERE / "emt6_oracle.h"]
    if force or _stale(REF_GPU_LIB, srcs):
        cuda = Path(NVCC).parent.parent
        stubs = [d for d in (cuda / "lib64" / "stubs", cuda / "targets" / "sbsa-linux" / "lib" / "stubs",
                             cuda / "lib" / "stubs") if d.exists()]
        tmp = REF_GPU_LIB.with_suffix(".so.tmp")
        _run([NVCC, *GENCODE, "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC",
              "-I", str(HERE), str(HERE / "ref_gpu_driver.cu"), "-o", str(tmp),
              *[f"-L{d}" for d in stubs], "-lcuda"])
        os.replace(tmp, REF_GPU_LIB)
    return REF_GPU_LIB


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_oracle_fast(force=True))
    print(build_ref(force=True))
    print(build_ref_cubin(force=True))
    print(build_ref_cell_cubin(force=True))
    print(build_ref_gpu_driver(force=True))
