"""Builds the oracle (test infrastructure): oracle/_build/liboracle.so from
emc_oracle.c, and -- when the reference tree is present -- the reference's own
rotations.c KAT binary via build_ref.sh.  Nothing in the product links these."""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
LIB = OUT / "liboracle.so"


def build() -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    src = HERE / "emc_oracle.c"
    if not LIB.exists() or src.stat().st_mtime > LIB.stat().st_mtime:
        subprocess.run(["gcc", "-O2", "-std=gnu99", "-fPIC", "-shared", "-fopenmp",
                        "-ffp-contract=off", str(src), "-o", str(LIB), "-lm"], check=True)
    ref = os.environ.get("EMC_REF_DIR", "/root/reference")
    if Path(ref, "rotations.c").exists():
        subprocess.run(["bash", str(HERE / "build_ref.sh")], check=True,
                       capture_output=True, env={**os.environ, "EMC_REF_DIR": ref})
    return LIB


if __name__ == "__main__":
    print(build())
