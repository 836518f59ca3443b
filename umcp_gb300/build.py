"""Builds the engine's shared library (CUDA for sm_103a + host C++) and the
hd-style driver. Objects are rebuilt only when a source is newer. (The
checker, under oracle/, has its own recipe: oracle/build.py.)

Outputs (all git-ignored):
  umcp_gb300/lib/libumcp_gb300.so   engine: kernels + C ABI (include/umcp_gpu.h)
  umcp_gb300/lib/hd_gb300           the hd-style dynamics driver on the engine
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "umcp_gb300" / "csrc"
BUILD = ROOT / "umcp_gb300" / "_build"
LIB_DIR = ROOT / "umcp_gb300" / "lib"
ENGINE_LIB = LIB_DIR / "libumcp_gb300.so"
HD_EXE = LIB_DIR / "hd_gb300"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]
CXX_FLAGS = ["-O2", "-fPIC", "-std=c++17", "-Wall", "-Wextra"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "umcp_gpu.h"]


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def build_engine(verbose: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    cuda_inc = str(Path(nvcc).resolve().parent.parent / "include")
    hdrs = _headers()
    jobs = []
    objs = []
    for src in sorted(CSRC.glob("*.cu")):
        obj = BUILD / (src.stem + ".cu.o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            jobs.append([nvcc] + NVCC_FLAGS + ["-c", str(src), "-o", str(obj)])
    for src in sorted(CSRC.glob("*.cpp")):
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            jobs.append(["g++"] + CXX_FLAGS + ["-I", cuda_inc, "-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        for fut in [ex.submit(_run, j) for j in jobs]:
            fut.result()
    if jobs or _stale(ENGINE_LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-cudart", "static", "-o", str(ENGINE_LIB)] + [str(o) for o in objs] + ["-ldl"])
    hd_src = ROOT / "umcp_gb300" / "hd" / "hd_main.cpp"
    if _stale(HD_EXE, [hd_src, ENGINE_LIB, ROOT / "include" / "umcp_gpu.h"]):
        _run(["g++", "-O2", "-std=c++17", "-Wall", "-o", str(HD_EXE), str(hd_src), "-L", str(LIB_DIR), "-lumcp_gb300",
              "-Wl,-rpath,$ORIGIN"])
    if verbose:
        print(f"built {ENGINE_LIB}")
    return ENGINE_LIB


def build_all(verbose: bool = False) -> None:
    build_engine(verbose)


if __name__ == "__main__":
    build_all(verbose=True)
    sys.exit(0)
