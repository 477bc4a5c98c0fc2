"""Build of libhcc_gb300.so: nvcc for sm_103a, one object per translation unit, compiled in parallel.

The FP64 translation units (neighbour search, MLS geometry, FP64 stage kernels) are compiled with -fmad=false so
that no multiply-add is contracted: their results follow the reference's rounding step for step. The FP32 bulk
kernels keep the default contraction. The learned predictor's unit is compiled with -fmad=false too: its FP32
stencil features follow the oracle's operation sequence bit for bit.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libhcc_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-lineinfo", "--expt-relaxed-constexpr", "-Xptxas", "-O3"]

UNITS = {
    "hcc_api.cu": [],
    "hcc_util.cu": [],
    "hcc_search.cu": ["-fmad=false"],
    "hcc_mls.cu": ["-fmad=false"],
    "hcc_stage_f64_r1.cu": ["-fmad=false"],
    "hcc_stage_f64_r2.cu": ["-fmad=false"],
    "hcc_stage_f32_r1.cu": ["-ftz=true"],
    "hcc_stage_f32_r2.cu": ["-ftz=true"],
    "hcc_noalloc.cu": ["-fmad=false"],
    "hcc_tiles.cu": [],
    "hcc_learn.cu": ["-fmad=false"],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _stale(obj: Path, deps) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build(verbose: bool = False, jobs: int | None = None, extra_flags=None, lib_path=None, build_dir=None) -> Path:
    """Compile every CUDA translation unit and link the shared library; returns its path. `extra_flags`,
    `lib_path` and `build_dir` build a variant (e.g. other launch shapes) next to the default library."""
    global BUILD, LIB
    BUILD = Path(build_dir) if build_dir else PKG / "_build"
    LIB = Path(lib_path) if lib_path else PKG / "libhcc_gb300.so"
    BUILD.mkdir(parents=True, exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "hcc.h"]
    extra = list(extra_flags or [])
    cmds = []
    objs = []
    for unit, flags in UNITS.items():
        src = CSRC / unit
        obj = BUILD / (unit + ".o")
        objs.append(obj)
        if _stale(obj, [src, *headers]) or extra:
            cmds.append([nvcc(), *ARCH, *COMMON, *flags, *extra, "-c", str(src), "-o", str(obj)])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed ({cmd[-3]}):\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, flush=True)
        return r

    with ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        list(ex.map(run, cmds))
    if cmds or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        link = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs)]
        run(link)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
