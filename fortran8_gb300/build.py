"""Build the in-tree CUDA library ``fortran8_gb300/libf8.so`` for sm_103a.

Each translation unit is compiled by nvcc in parallel and linked into one
shared object that exports the C ABI of include/f8.h.  The FP64 kernels are
compiled with ``--fmad=false`` so that their arithmetic keeps the reference's
operation order (no fused multiply-add contraction).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
LIB = HERE / "libf8.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-fast-math",
          "-diag-suppress", "177"]
# translation unit -> extra flags
UNITS = {
    "f8_step_fp64.cu": ["--fmad=false"],
    "f8_api.cu": ["--fmad=false"],
    "f8_step_mixed.cu": [],
    "f8_fftsolve.cu": ["--fmad=false"],
    "f8_diag.cu": ["--fmad=false"],
    "f8_adjoint.cu": ["--fmad=false"],
    "f8_adjoint_mixed.cu": [],
}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA library cannot be built")


def _sources_newer(target: Path) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    deps = list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h"))
    deps.append(HERE.parent / "include" / "f8.h")
    deps.append(Path(__file__))
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and not _sources_newer(LIB):
        return LIB
    nvcc = _nvcc()
    objdir = HERE / "_build"
    objdir.mkdir(exist_ok=True)

    def compile_unit(item):
        src, extra = item
        obj = objdir / (Path(src).stem + ".o")
        cmd = [nvcc, *ARCH, *COMMON, *extra, "-c", str(CSRC / src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS.items()))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
