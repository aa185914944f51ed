"""Build libwkgpu.so in-tree: C++ host runtime (g++) + sm_103a kernels (nvcc).

Run as ``python -m wukonggpu_gb300.build`` or through ``__graft_entry__.build()``.
Objects go to ``wukonggpu_gb300/_build/``; the library is
``wukonggpu_gb300/libwkgpu.so``.  Translation units compile in parallel and
are rebuilt only when a source or header is newer than the object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libwkgpu.so"
# the seeded graph generator alone (host code, no CUDA): the CPU baseline loads
# it to make its graph without mapping the GPU library
GEN_LIB = PKG / "libwkgen.so"
GEN_SRCS = ("wk_gen.cpp", "wk_error.cpp")
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _newest_header() -> float:
    hs = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    return max((h.stat().st_mtime for h in hs), default=0.0)


def _compile(src: Path, cuda: Path, hdr_mtime: float) -> Path:
    obj = BUILD / (src.name + ".o")
    if obj.exists() and obj.stat().st_mtime >= max(src.stat().st_mtime, hdr_mtime):
        return obj
    if src.suffix == ".cu":
        cmd = [str(cuda / "bin" / "nvcc"), "-O3", "-std=c++17", *ARCH, "-lineinfo",
               "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
               "-I", str(CSRC), "-c", str(src), "-o", str(obj)]
    else:
        cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
               "-I", str(cuda / "include"), "-I", str(CSRC), "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> Path:
    cuda = _cuda_home()
    BUILD.mkdir(exist_ok=True)
    srcs = sorted(CSRC.glob("*.cpp")) + sorted(CSRC.glob("*.cu"))
    hdr = _newest_header()
    with cf.ThreadPoolExecutor(max_workers=max(2, min(16, os.cpu_count() or 2))) as ex:
        objs = list(ex.map(lambda s: _compile(s, cuda, hdr), srcs))
    newest = max(o.stat().st_mtime for o in objs)
    if not LIB.exists() or LIB.stat().st_mtime < newest:
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [str(cuda / "bin" / "nvcc"), "-shared", *ARCH, "-o", str(tmp), *map(str, objs),
               "-cudart", "static", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    gen_objs = [BUILD / (n + ".o") for n in GEN_SRCS]
    if not GEN_LIB.exists() or GEN_LIB.stat().st_mtime < max(o.stat().st_mtime for o in gen_objs):
        tmp = GEN_LIB.with_suffix(".so.tmp")
        cmd = ["g++", "-shared", "-o", str(tmp), *map(str, gen_objs), "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, GEN_LIB)
    if verbose:
        print(f"built {LIB} and {GEN_LIB.name}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
