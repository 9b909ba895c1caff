"""Builds the reference-side binding of INTEGRATION.md, section 1 (test code).

emc_cuda_gb300.cpp implements the reference's cuda_* signatures on
libemc_gb300; it is compiled against the reference's own emc_cuda_help.h (from
$EMC_REF_DIR or the staged baseline/_ref/src, with the stand-in headers of
oracle/shim), so a signature that drifts from the reference fails to compile.
drive_iteration.cpp runs one iteration through those signatures for the GPU
test.  Output: tests/refshim/_build/libemc_refshim.so (git-ignored), linked
against emc_gb300/_build/libemc_gb300.so."""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
OUT = HERE / "_build"
SO = OUT / "libemc_refshim.so"
SOURCES = [HERE / "emc_cuda_gb300.cpp", HERE / "drive_iteration.cpp"]


def _flags(ref: Path) -> list[str]:
    return ["-std=c++17", "-O2", "-fPIC", "-w", f"-I{ROOT / 'oracle' / 'shim'}", f"-I{ref}",
            f"-I{ROOT / 'include'}"]


def compile_objects(ref: Path) -> list[Path]:
    """Compiles both sources against the reference header; returns the objects."""
    OUT.mkdir(parents=True, exist_ok=True)
    objs = []
    for src in SOURCES:
        obj = OUT / (src.stem + ".o")
        subprocess.run(["g++", *_flags(ref), "-c", str(src), "-o", str(obj)], check=True,
                       capture_output=True, text=True)
        objs.append(obj)
    return objs


def build(ref: Path) -> Path:
    objs = compile_objects(ref)
    lib_dir = ROOT / "emc_gb300" / "_build"
    subprocess.run(["g++", "-shared", *map(str, objs), "-o", str(SO), f"-L{lib_dir}",
                    "-lemc_gb300", f"-Wl,-rpath,{lib_dir}"], check=True, capture_output=True,
                   text=True)
    return SO
