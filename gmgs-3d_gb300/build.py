"""Build libgmgs.so (sm_103a) in-tree with nvcc; no CMake, no torch.

    python gmgs-3d_gb300/build.py [--debug] [--jobs N]

Each .cu translation unit compiles in parallel into _build/, then one shared
library is linked into gmgs-3d_gb300/gmgs/libgmgs.so.  --debug builds the
checked library gmgs-3d_gb300/gmgs/libgmgs_checked.so instead (GMGS_CHECKED:
every instrumented gather, scatter and shared-memory access tests its index
and the C ABI reports an out-of-range one; host code at -O0 -g); load it by
setting GMGS_LIB to its path.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = ROOT / "_build" / "gmgs"
LIB = PKG / "gmgs" / "libgmgs.so"
LIB_CHECKED = PKG / "gmgs" / "libgmgs_checked.so"
SOURCES = ["api.cu", "setup.cu", "operators.cu", "solver.cu", "post.cu", "fine.cu", "tc.cu", "noalloc.cu", "voxelize.cu",
           "coarse.cu"]
# the voxeliser decides inside/outside by exact FP64 comparisons: no FMA contraction
FILE_FLAGS = {"voxelize.cu": ["-fmad=false", "-Xcompiler", "-ffp-contract=off"]}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def flags(debug: bool) -> list[str]:
    f = ["-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", str(ROOT / "include"), "-I", str(CSRC),
         "-I", str(BUILD),
         "--expt-relaxed-constexpr", "-Xptxas", "-v" if os.environ.get("GMGS_PTXAS_V") else "-O3"]
    f += ["-O0", "-g", "-DGMGS_CHECKED"] if debug else ["-O3"]
    return ARCH + f


def obj_dir(debug: bool) -> Path:
    """Object files of each build mode live apart, so a debug build never
    leaves objects that a later release build would take as up to date."""
    return BUILD / ("debug" if debug else "release")


# the default-material coefficient table the streaming kernels include
# (generated from the library's host element code by gen_default_stencil.cu)
DEFAULT_STENCIL = BUILD / "gmgs_default_stencil.h"


def generate_default_stencil() -> Path:
    gen_src = CSRC / "gen_default_stencil.cu"
    deps = [gen_src, CSRC / "element_host.h", CSRC / "gmgs_internal.cuh"]
    exe = BUILD / "gen_default_stencil"
    # regenerated on every machine that builds (the generator's executable is
    # not carried between machines): the host arithmetic may differ by platform
    if (DEFAULT_STENCIL.exists() and exe.exists()
            and all(DEFAULT_STENCIL.stat().st_mtime >= d.stat().st_mtime for d in deps)):
        return DEFAULT_STENCIL
    BUILD.mkdir(parents=True, exist_ok=True)
    cmd = [nvcc(), "-std=c++17", "-O3", "-I", str(ROOT / "include"), "-I", str(CSRC), str(gen_src), "-o", str(exe)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for gen_default_stencil.cu:\n{res.stdout}\n{res.stderr}")
    tmp = DEFAULT_STENCIL.with_suffix(".tmp")
    res = subprocess.run([str(exe), str(tmp)], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"gen_default_stencil failed:\n{res.stdout}\n{res.stderr}")
    tmp.replace(DEFAULT_STENCIL)
    return DEFAULT_STENCIL


def compile_one(src: str, debug: bool) -> Path:
    out = obj_dir(debug) / (Path(src).stem + ".o")
    srcp = CSRC / src
    deps = [srcp] + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [ROOT / "include" / "gmgs.h", DEFAULT_STENCIL]
    if out.exists() and all(out.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return out
    cmd = [nvcc(), *flags(debug), *FILE_FLAGS.get(src, []), "-c", str(srcp), "-o", str(out)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    if os.environ.get("GMGS_PTXAS_V"):
        sys.stderr.write(res.stderr)
    return out


def build(debug: bool = False, jobs: int | None = None) -> Path:
    obj_dir(debug).mkdir(parents=True, exist_ok=True)
    generate_default_stencil()
    srcs = [s for s in SOURCES if (CSRC / s).exists()]
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: compile_one(s, debug), srcs))
    newest = max(o.stat().st_mtime for o in objs)
    lib = LIB_CHECKED if debug else LIB
    if lib.exists() and lib.stat().st_mtime >= newest:
        return lib
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    return lib


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--debug", action="store_true")
    ap.add_argument("--jobs", type=int, default=None)
    a = ap.parse_args()
    print(build(a.debug, a.jobs))
