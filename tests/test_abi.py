"""The C ABI library: every symbol declared in include/emc_gb300.h is
exported, host-side entry points work, device entry points fail cleanly
(status codes, no crash) when given bad arguments."""
import ctypes as C
import os
import re

import numpy as np

import emc_gb300 as E
from emc_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "emc_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(emc_[a-z0-9_]+)\s*\(", src)))


def test_every_declared_symbol_is_exported(built):
    names = declared_functions()
    assert len(names) >= 30
    lib = C.CDLL(str(_lib.LIB_PATH))
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header(built):
    assert set(declared_functions()) == set(_lib.SIGNATURES)


def test_null_context_is_rejected(built):
    lib = _lib.load()
    assert lib.emc_sync(None) == -1
    assert lib.emc_get_slices(None, None, 8, None, None, None, None, None, 0, 1, 0) == -1
    assert lib.emc_last_error(None) == b"null context"
    assert lib.emc_plan_bind(None, None, None, None, None, None, None, None) == -1
    # option access on a null plan (no device work) is refused, not dereferenced
    import ctypes
    v = ctypes.c_int(7)
    assert lib.emc_plan_get_option(None, 3, ctypes.byref(v)) == -1 and v.value == 7
    assert lib.emc_plan_set_option(None, 3, 1) == -1


def test_sigma_schedule_matches_main_cpp(built):
    # main.cpp:251 with emc.conf's 0.4 / 0.12 / 25
    for t in (0, 1, 10, 25, 49):
        want = np.float32(0.12 + (0.4 - 0.12) * np.exp(np.float64(np.float32(-t / np.float32(25))) * np.log(2.0)))
        assert np.float32(E.sigma_schedule(t, 0.4, 0.12, 25)) == want
    assert abs(E.sigma_schedule(25, 0.4, 0.12, 25) - 0.26) < 1e-6


def test_coordinates_geometry(built):
    x, y, z = E.calculate_coordinates(64, 75e-6, 0.74, 1.03e-9)
    X = x.reshape(64, 64)
    Y = y.reshape(64, 64)
    # [y*side + x] layout, half-integer pixel centres
    assert X[0, 0] == -31.5 and X[0, 63] == 31.5 and Y[63, 0] == 31.5
    r = np.sqrt(x.astype(np.float64) ** 2 + y ** 2)
    theta = np.arctan2(r * 75e-6, 0.74)
    want = (1 - np.cos(theta)) / np.sin(theta) * r
    # float evaluation of 1 - cos(angle), as in emc_helper.cpp:55-79, leaves
    # ~1e-3 voxels of cancellation noise on z (a tenth of a voxel at the rim)
    assert np.abs(z - want).max() < 1e-3
    assert (z >= 0).all()  # 1 - cos rounds to 0 in float near the beam


def test_option_numbers_match_the_header(built):
    """Plan.OPT_* carries the header's EMC_OPT_* numbers."""
    import re
    from pathlib import Path

    import emc_gb300 as E
    hdr = (Path(__file__).resolve().parents[1] / "include" / "emc_gb300.h").read_text()
    opts = {m.group(1): int(m.group(2))
            for m in re.finditer(r"#define EMC_OPT_([A-Z0-9_]+) (-?\d+)", hdr)}
    assert len(opts) >= 7
    for name, value in opts.items():
        assert getattr(E.Plan, "OPT_" + name) == value, name
    # insertion modes likewise (EMC_INSERT_* -> emc_gb300.INSERT_*)
    modes = {m.group(1): int(m.group(2))
             for m in re.finditer(r"#define EMC_INSERT_([A-Z0-9_]+) (-?\d+)", hdr)}
    assert set(modes) == {"ATOMIC", "DETERMINISTIC", "SORTED"}
    for name, value in modes.items():
        assert getattr(E, "INSERT_" + name) == value, name


def test_heldout_patterns_share_the_particle():
    """pattern_seed draws new orientations, scales and counts of the same
    particle and detector."""
    from emc_gb300 import synthetic as S
    import dataclasses
    cfg = dataclasses.replace(S.tiny(side=24, n_images=20, rot_n=1), photons=300)
    rot = (np.zeros((1, 4), np.float32), np.ones(1, np.float32))
    coords = tuple(np.zeros(24 * 24, np.float32) + v for v in (0.0, 0.0, 0.0))
    a = S.make_problem(cfg, coords=coords, rotations=rot)
    b = S.make_problem(cfg, coords=coords, rotations=rot, pattern_seed=1)
    c = S.make_problem(cfg, coords=coords, rotations=rot, pattern_seed=1)
    assert np.array_equal(a.true_model, b.true_model) and np.array_equal(a.mask, b.mask)
    assert not np.allclose(a.true_quats, b.true_quats)
    assert np.array_equal(b.true_quats, c.true_quats) and np.array_equal(b.images, c.images)
