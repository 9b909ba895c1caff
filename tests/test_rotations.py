"""Rotation sampling (row A1) against the reference's own rotations.c.

Pins: tests/golden/rotations_ref.npz was produced by the reference build
(tests/golden/make_rotation_golden.py); the counts, first quaternion and
float weight sums below were also read off that build."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import emc_gb300 as E

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = np.load(os.path.join(ROOT, "tests", "golden", "rotations_ref.npz"))


@pytest.mark.parametrize("n", [1, 2, 3, 4])
def test_bit_identical_to_reference_golden(built, n):
    q, w = E.generate_rotations(n)
    assert np.array_equal(q, GOLD[f"q{n}"])
    assert np.array_equal(w, GOLD[f"w{n}"])


@pytest.mark.parametrize("n", [6, 8, 12])
def test_large_levels_match_reference_summary(built, n):
    q, w = E.generate_rotations(n)
    s = GOLD[f"summary{n}"]
    assert q.shape[0] == int(s[0])
    assert np.float32(np.sum(w, dtype=np.float32)) == np.float32(s[1])
    assert float(np.abs(q.astype(np.float64)).sum()) == s[2]
    assert float(w.astype(np.float64).sum()) == s[3]
    assert float((q.astype(np.float64) * np.arange(1, 5)).sum()) == s[4]
    e = GOLD[f"ends{n}"]
    assert np.array_equal(np.concatenate([q[0], q[-1], w[:1], w[-1:]]), e)


@pytest.mark.parametrize("n,R,wsum", [(3, 1380, 1.00000401), (4, 3240, 1.00001671),
                                      (6, 10860, 0.999939927), (8, 25680, 1.00013991),
                                      (12, 86520, 0.999893175)])
def test_known_answers(built, n, R, wsum):
    assert E.rotation_count(n) == R
    q, w = E.generate_rotations(n)
    assert q.shape == (R, 4)
    assert np.array_equal(q[0], np.array([0.5, -0.5, -0.5, -0.5], np.float32))
    assert abs(float(np.sum(w, dtype=np.float32)) - wsum) < 2e-7
    # hemisphere q0 > 0 with lexicographic tie-break; unit norm
    first_nz = np.array([r[np.nonzero(r)[0][0]] for r in q])
    assert (first_nz > 0).all()
    assert np.allclose(np.linalg.norm(q.astype(np.float64), axis=1), 1.0, atol=1e-6)


def test_live_reference_build_if_present(built):
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_rotations")
    if not os.path.exists(exe):
        pytest.skip("reference rotations.c build not present (no reference tree here)")
    for n in (5, 7):
        with tempfile.TemporaryDirectory() as d:
            subprocess.run([exe, str(n), f"{d}/o.bin"], cwd=d, check=True, capture_output=True)
            b = open(f"{d}/o.bin", "rb").read()
        R = int(np.frombuffer(b[:4], np.int32)[0])
        q, w = E.generate_rotations(n)
        assert np.array_equal(q, np.frombuffer(b[4:4 + 16 * R], np.float32).reshape(R, 4))
        assert np.array_equal(w, np.frombuffer(b[4 + 16 * R:], np.float32))


def test_bad_level_rejected(built):
    assert E.rotation_count(0) < 0
    with pytest.raises(E.EmcError):
        E.generate_rotations(0)
