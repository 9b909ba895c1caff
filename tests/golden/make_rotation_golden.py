"""Generates tests/golden/rotations_ref.npz from the reference's own
rotations.c (oracle/_ref/ref_rotations, built by oracle/build_ref.sh from the
reference tree).  Run from the repository root:
    python tests/golden/make_rotation_golden.py
Stores the full quaternion/weight lists for n = 1..4 and, for n = 6, 8, 12,
the count, the first/last quaternions, the float weight sum and a float64
checksum of every value."""
from __future__ import annotations

import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
BIN = ROOT / "oracle" / "_ref" / "ref_rotations"


def run_ref(n: int):
    with tempfile.TemporaryDirectory() as d:
        subprocess.run([str(BIN), str(n), f"{d}/o.bin"], cwd=d, check=True, capture_output=True)
        b = Path(d, "o.bin").read_bytes()
    R = int(np.frombuffer(b[:4], np.int32)[0])
    q = np.frombuffer(b[4:4 + 16 * R], np.float32).reshape(R, 4).copy()
    w = np.frombuffer(b[4 + 16 * R:], np.float32).copy()
    return q, w


def main():
    if not BIN.exists():
        subprocess.run(["bash", str(ROOT / "oracle" / "build_ref.sh")], check=True)
    out = {}
    for n in (1, 2, 3, 4):
        q, w = run_ref(n)
        out[f"q{n}"], out[f"w{n}"] = q, w
    for n in (6, 8, 12):
        q, w = run_ref(n)
        out[f"summary{n}"] = np.array([q.shape[0], float(np.sum(w, dtype=np.float32)),
                                       float(np.abs(q.astype(np.float64)).sum()),
                                       float(w.astype(np.float64).sum()),
                                       float((q.astype(np.float64) * np.arange(1, 5)).sum())])
        out[f"ends{n}"] = np.concatenate([q[0], q[-1], w[:1], w[-1:]])
    np.savez_compressed(ROOT / "tests" / "golden" / "rotations_ref.npz", **out)
    print("wrote tests/golden/rotations_ref.npz")


if __name__ == "__main__":
    sys.exit(main())
