"""Build of the native library (libplsqr_gpu.so) and the plsqr3_gpu program.

Every CUDA translation unit is compiled for sm_103a only; the host sources
(file formats, synthetic problems, text reports) are compiled by the host
compiler through nvcc with OpenMP and without FMA contraction (the synthetic
generator relies on that to give the same bits on x86_64 and aarch64).  The
translation units are compiled in parallel, outputs stay in lib/ next to this
file (in-tree, git-ignored).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIB = PKG / "lib"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["plsqr_gpu.cu", "mixed.cu", "slab.cu", "noalloc.cu", "batched.cu", "multi.cu", "unet.cu"]
CPP_SOURCES = ["formats.cpp", "synth.cpp", "report.cpp", "files_ctx.cpp"]
LIBNAME = "libplsqr_gpu.so"


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _common() -> list[str]:
    return ["-O3", "-std=c++17", "-I", str(INCLUDE), "-I", str(CSRC),
            "-Xcompiler", "-fPIC,-fopenmp,-ffp-contract=off,-Wall,-Wno-unknown-pragmas"]


def _compile(src: Path, obj: Path, defines: tuple[str, ...] = ()) -> None:
    cmd = [nvcc(), *ARCH, "-lineinfo", *_common(), *defines, "-c", str(src), "-o", str(obj)]
    if src.suffix == ".cu":
        cmd += ["-Xptxas", "-v"] if os.environ.get("PLSQR_PTXAS_VERBOSE") else []
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip() and os.environ.get("PLSQR_PTXAS_VERBOSE"):
        sys.stderr.write(r.stderr)


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, check: bool = False) -> Path:
    """Compile libplsqr_gpu.so and plsqr3_gpu; returns the library path.
    check: the bounds-checked library instead (-DPLSQR_CHECK, objects in
    lib/check/, lib/libplsqr_gpu_check.so; no program), for tests."""
    LIB.mkdir(exist_ok=True)
    odir = LIB / "check" if check else LIB
    odir.mkdir(exist_ok=True)
    defines = ("-DPLSQR_CHECK",) if check else ()
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [INCLUDE / "plsqr_gpu.h"]
    srcs = [CSRC / s for s in CU_SOURCES + CPP_SOURCES]
    objs = [odir / (s.name + ".o") for s in srcs]
    jobs = [(s, o) for s, o in zip(srcs, objs) if force or _stale(o, [s, *headers])]
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for f in [ex.submit(_compile, s, o, defines) for s, o in jobs]:
                f.result()
    so = LIB / ("libplsqr_gpu_check.so" if check else LIBNAME)
    if force or jobs or _stale(so, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(so), *map(str, objs),
               "-Xcompiler", "-fopenmp", "-lgomp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if check:
        return so
    exe = LIB / "plsqr3_gpu"
    main_c = CSRC / "plsqr3_main.c"
    if force or _stale(exe, [main_c, so, INCLUDE / "plsqr_gpu.h"]):
        cmd = ["gcc", "-O2", "-std=c11", "-Wall", "-I", str(INCLUDE), str(main_c), "-o", str(exe),
               "-L", str(LIB), "-lplsqr_gpu", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"build of plsqr3_gpu failed: {' '.join(cmd)}\n{r.stderr}")
    return so


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
