"""
Build the CUDA library ``libfasterlmm_gb300.so`` in-tree for sm_103a (GB300).

Each ``csrc/*.cu`` translation unit is compiled by nvcc in parallel into ``_build/`` and linked into the package
directory; cuSOLVER (for the FP64 eigendecomposition and the covariate SVD) is linked as a shared library with an
rpath to the toolkit.  Objects are rebuilt only when a source or header is newer.
"""

from __future__ import annotations

import os
import platform
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent                      # fast-er-lmm_gb300/
REPO = ROOT.parent
CSRC = ROOT / "csrc"
INCLUDE = REPO / "include"
BUILD = ROOT / "_build"
LIB = PKG / "libfasterlmm_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parents[1]
    raise RuntimeError("nvcc not found: set CUDA_HOME to a CUDA 13 toolkit")


def _newest(paths) -> float:
    return max((p.stat().st_mtime for p in paths), default=0.0)


def build(verbose: bool = False, jobs: int | None = None, force: bool = False) -> Path:
    home = cuda_home()
    nvcc = str(home / "bin" / "nvcc")
    BUILD.mkdir(exist_ok=True)
    # objects from another host architecture (a checkout copied between x86 and Arm machines) are never reused
    stamp = BUILD / "host_arch.txt"
    if not stamp.exists() or stamp.read_text().strip() != platform.machine():
        force = True
        stamp.write_text(platform.machine())
    sources = sorted(CSRC.glob("*.cu"))
    headers = list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    hdr_time = _newest(headers)
    cflags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
                     "-I", str(INCLUDE), "-I", str(CSRC)]

    def compile_one(src: Path) -> Path:
        obj = BUILD / (src.stem + ".o")
        if not force and obj.exists() and obj.stat().st_mtime >= max(src.stat().st_mtime, hdr_time):
            return obj
        cmd = [nvcc, *cflags, "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, flush=True)
        return obj

    with ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(compile_one, sources))
    if force or not LIB.exists() or LIB.stat().st_mtime < _newest(objs):
        libdir = home / "lib64"
        if not libdir.exists():
            libdir = home / "lib"
        cmd = [nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-L", str(libdir), "-lcusolver",
               "-Xlinker", f"-rpath,{libdir}"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
