"""Build recipe for libemc_gb300.so (sm_103a) and the host driver.

Compiles every CUDA translation unit under csrc/ with nvcc for sm_103a and the
host C++ sources with g++, in parallel, and links them into
emc_gb300/_build/libemc_gb300.so (in-tree, git-ignored).  Host code is built
with -ffp-contract=off so float results match between x86-64 and aarch64.
Rebuilds only what changed (by modification time).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libemc_gb300.so"
EXE = BUILD / "emc"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "--expt-relaxed-constexpr", f"-I{INCLUDE}"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", f"-I{INCLUDE}"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _headers() -> list[Path]:
    return sorted(CSRC.rglob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def _stale(obj: Path, src: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return src.stat().st_mtime > t or any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build(verbose: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    deps = _headers()
    jobs = []
    objs = []
    for src in sorted(CSRC.glob("*.cu")):
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if _stale(obj, src, deps):
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)])
    for src in sorted((CSRC / "host").glob("*.cpp")):
        if src.name == "emc_main.cpp":
            continue
        obj = BUILD / (src.stem + ".host.o")
        objs.append(obj)
        if _stale(obj, src, deps):
            jobs.append(["g++", *CXX_FLAGS, "-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    if jobs or not LIB.exists():
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs)])
    main = CSRC / "host" / "emc_main.cpp"
    if main.exists() and (jobs or not EXE.exists() or _stale(EXE, main, deps)):
        _run(["g++", *CXX_FLAGS, str(main), "-o", str(EXE), f"-L{BUILD}", "-lemc_gb300",
              f"-Wl,-rpath,{BUILD}", "-ldl"])
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
