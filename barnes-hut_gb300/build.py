"""Builds libbh_gpu.so in-tree (``barnes-hut_gb300/_build/``) with nvcc for
sm_103a, then the reference-API shim (libbh_reference_api.so) and the
``simulate`` driver over it with g++.  Each translation unit compiles in its
own process, in parallel; objects newer than their sources and headers are
reused.

Usage: ``python barnes-hut_gb300/build.py`` or ``build.build()``.
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
OUT = PKG / "_build"
LIB = OUT / "libbh_gpu.so"
SHIM = PKG / "shim"
SHIM_LIB = OUT / "libbh_reference_api.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", f"-I{INCLUDE}"]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", f"-I{INCLUDE}"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA extension cannot be built")


def _headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h")))


def _compile(src: Path, obj: Path, nvcc: str) -> tuple[Path, str]:
    if src.suffix == ".cu":
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
    else:
        cmd = [shutil.which("g++") or "g++", *CXX_FLAGS, "-I" + str(Path(nvcc).parent.parent / "include"),
               "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose: bool = False, force: bool = False) -> Path:
    nvcc = _nvcc()
    OUT.mkdir(exist_ok=True)
    sources = sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))
    hdr_mtime = max((h.stat().st_mtime for h in _headers()), default=0.0)
    jobs = []
    objs = []
    for src in sources:
        obj = OUT / (src.name + ".o")
        objs.append(obj)
        if force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, hdr_mtime):
            jobs.append((src, obj))
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for obj, err in ex.map(lambda j: _compile(j[0], j[1], nvcc), jobs):
            if verbose:
                print(f"built {obj.name}", err.strip(), file=sys.stderr)
    if force or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    # The reference's C++ call surface over the library, and the
    # reference-compatible driver.
    _host_link(SHIM_LIB, [SHIM / "bh_reference_api.cpp"], ["-shared"], force)
    _host_link(OUT / "simulate", [SHIM / "simulate.cpp"], ["-pthread"], force)
    return LIB


def _host_link(out: Path, srcs: list[Path], extra: list[str], force: bool) -> None:
    deps = [*srcs, *SHIM.glob("*.hpp"), LIB]
    if not force and out.exists() and out.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return
    cmd = [shutil.which("g++") or "g++", *CXX_FLAGS, f"-I{SHIM}", *extra, *map(str, srcs), "-o", str(out),
           f"-L{OUT}", "-lbh_gpu", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
