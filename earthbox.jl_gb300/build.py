"""Build libebgpu.so (the C-ABI CUDA library) in-tree for sm_103a.

The translation units are compiled in parallel with nvcc and linked into
``earthbox.jl_gb300/_build/libebgpu.so``.  A rebuild happens only when a source
or header is newer than the library.
"""
from __future__ import annotations

import os
import pathlib
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = pathlib.Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libebgpu.so"
SOURCES = ["eb_ctx.cu", "eb_locate.cu", "eb_scatter.cu", "eb_gather.cu", "eb_advect.cu", "eb_rheology.cu",
           "eb_noalloc.cu", "eb_stokes_build.cu", "eb_stokes_solve.cu", "eb_heat.cu",
           "eb_pipeline.cu", "eb_step_boundary.cu", "eb_recycle.cu", "eb_nn.cu", "eb_nn_net.cu"]
# The Stokes assembly reproduces the reference's FP64 coefficients operation by
# operation, so no multiply-add contraction there.
EXTRA_FLAGS = {"eb_stokes_build.cu": ["-fmad=false"], "eb_heat.cu": ["-fmad=false"],
               "eb_step_boundary.cu": ["-fmad=false"], "eb_recycle.cu": ["-fmad=false"]}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _deps() -> list[pathlib.Path]:
    return [CSRC / s for s in SOURCES] + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [ROOT / "include" / "ebgpu.h"]


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _deps())


def build(force: bool = False, verbose: bool = False) -> pathlib.Path:
    """Compile every .cu under csrc/ for sm_103a and link libebgpu.so."""
    if not force and up_to_date():
        return LIB
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()

    def compile_one(src: str) -> pathlib.Path:
        obj = BUILD / (pathlib.Path(src).stem + ".o")
        cmd = [nvcc, *ARCH, *FLAGS, *EXTRA_FLAGS.get(src, []), "-c", str(CSRC / src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = BUILD / "libebgpu.so.tmp"
    cmd = [nvcc, *ARCH, "-shared", *map(str, objs), "-o", str(tmp), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
