"""In-tree build of libgrgx.so (the CUDA kernels + C ABI) for sm_103a.

Compiles every translation unit under grgl_gb300/csrc in parallel (g++ for host C++, nvcc for
CUDA with one -gencode for compute_103a/sm_103a) and links them with the static CUDA runtime
into grgl_gb300/libgrgx.so.  Objects go to grgl_gb300/_build and are reused when they are
newer than every source and header.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libgrgx.so"
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

CXXFLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
            f"-I{ROOT / 'include'}", f"-I{CSRC}", f"-I{CUDA_HOME / 'include'}"]
NVCCFLAGS = ["-O3", "-std=c++17", ARCH, "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
             f"-I{ROOT / 'include'}", f"-I{CSRC}"]


def _headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "grgx.h"])


def _stale(obj: Path, src: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *deps])


def _compile(src: Path, deps: list[Path], verbose: bool) -> Path:
    obj = BUILD / (src.name + ".o")
    if not _stale(obj, src, deps):
        return obj
    if src.suffix == ".cu":
        cmd = [str(CUDA_HOME / "bin" / "nvcc"), *NVCCFLAGS, "-c", str(src), "-o", str(obj)]
    else:
        cmd = ["g++", *CXXFLAGS, "-c", str(src), "-o", str(obj)]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compile failed: {src.name}\n{res.stdout}\n{res.stderr}")
    return obj


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compile and link libgrgx.so; returns its path."""
    BUILD.mkdir(exist_ok=True)
    deps = _headers()
    srcs = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    jobs = jobs or max(2, min(16, os.cpu_count() or 4))
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, deps, verbose), srcs))
    if LIB.exists() and all(LIB.stat().st_mtime >= o.stat().st_mtime for o in objs):
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["g++", "-shared", "-o", str(tmp), *map(str, objs), f"-L{CUDA_HOME / 'lib64'}", "-lcudart_static",
           "-ldl", "-lrt", "-lpthread", "-Wl,--no-undefined"]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
