"""Builds the oracle (test infrastructure): oracle/_build/liboracle.so from
emc_oracle.c, and -- when the reference tree is present -- the reference's own
rotations.c KAT binary and host helper (emc_helper.cpp) via build_ref.sh.
Nothing in the product links these."""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
LIB = OUT / "liboracle.so"


STAGED = HERE.parent / "baseline" / "_ref" / "src"


def ref_dir():
    """The reference source tree used by the checkers: $EMC_REF_DIR when set,
    else the staged copy under baseline/_ref/src (git-ignored; it travels with
    the working tree), else None."""
    env = os.environ.get("EMC_REF_DIR")
    if env and Path(env, "rotations.c").exists():
        return Path(env)
    if Path(STAGED, "rotations.c").exists():
        return STAGED
    return None


def stage(src) -> None:
    """Copies the reference files the checkers compile from `src` into the
    staged tree (build_ref.sh --stage)."""
    subprocess.run(["bash", str(HERE / "build_ref.sh"), "--stage"], check=True,
                   capture_output=True, env={**os.environ, "EMC_REF_DIR": str(src)})


def build() -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    src = HERE / "emc_oracle.c"
    if not LIB.exists() or src.stat().st_mtime > LIB.stat().st_mtime:
        subprocess.run(["gcc", "-O2", "-std=gnu99", "-fPIC", "-shared", "-fopenmp",
                        "-ffp-contract=off", str(src), "-o", str(LIB), "-lm"], check=True)
    ref = ref_dir()
    if ref is not None:
        subprocess.run(["bash", str(HERE / "build_ref.sh"), "--helper"], check=True,
                       capture_output=True, env={**os.environ, "EMC_REF_DIR": str(ref)})
    return LIB


def ref_helper():
    """ctypes handle of oracle/_ref/libemc_ref_helper.so (the reference's own
    emc_helper.cpp behind ref_helper_harness.cpp), or None when the reference
    tree was not available to build it."""
    import ctypes
    so = HERE / "_ref" / "libemc_ref_helper.so"
    if not so.exists():
        return None
    lib = ctypes.CDLL(str(so), mode=os.RTLD_NOW)
    P, I, F, U = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_ulonglong
    sig = {"refh_calculate_coordinates": [I, F, F, F, P, P, P],
           "refh_read_images": [P, P, I, I, I, I, I, P, P],
           "refh_normalize_images": [P, P, P, I, I, I, F],
           "refh_mask_model": [P, P, I, I],
           "refh_model_init": [I, P, P, I, I, P, P, P, U, P, P],
           "refh_quaternion_random": [U, I, P]}
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = I
    return lib


if __name__ == "__main__":
    print(build())
