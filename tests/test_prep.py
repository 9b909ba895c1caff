"""Host-side pieces of the preprocessing and model initialisation (no GPU):
the seeded quaternion generator and the oracle's restatements of the
reference's host code (emc_helper.cpp:226-243, 389-438, 458-518, 567-575)."""
import numpy as np

import emc_gb300 as E
from emc_gb300 import synthetic as S
from oracle import oracle as O


def test_random_rotations_are_unit_and_seeded():
    q = E.random_rotations(7, 4000)
    assert q.shape == (4000, 4) and q.dtype == np.float32
    assert np.allclose(np.linalg.norm(q.astype(np.float64), axis=1), 1.0, atol=1e-6)
    assert np.array_equal(q, E.random_rotations(7, 4000))
    assert not np.array_equal(q, E.random_rotations(8, 4000))
    # Shoemake sampling is uniform on SO(3): every component has mean 0, E[q_k^2] = 1/4
    assert np.abs(q.mean(0)).max() < 0.03
    assert np.abs((q.astype(np.float64) ** 2).mean(0) - 0.25).max() < 0.02
    assert E.random_rotations(1, 0).shape == (0, 4)


def test_binning_sums_blocks_and_counts_masks():
    rng = np.random.default_rng(0)
    side, stride = 8, 2
    raw = rng.normal(size=(3, side * stride, side * stride)).astype(np.float32)
    rmask = (rng.random(raw.shape) > 0.3).astype(np.int32)
    img, msk = O.bin_images(raw, rmask, side, stride)
    # the block of output (x, y) is rows y*s..y*s+s-1, columns x*s..x*s+s-1 for a frame of side*s
    blk = np.abs(raw).reshape(3, side, stride, side, stride)
    msum = rmask.reshape(3, side, stride, side, stride).sum((2, 4)).reshape(3, -1)
    with np.errstate(divide="ignore", invalid="ignore"):
        want = blk.sum((2, 4)).reshape(3, -1) / msum
    ok = msum > 0
    np.testing.assert_allclose(img[ok], want[ok], rtol=1e-6)
    assert np.array_equal(msk, (msum > 1).astype(np.int32))


def test_stride_one_masks_everything():
    # a one-pixel block has a mask sum of at most 1, and the reference keeps
    # pixels whose mask sum is > 1 (emc_helper.cpp:236-240)
    raw = np.ones((1, 4, 4), np.float32)
    img, msk = O.bin_images(raw, np.ones((1, 4, 4), np.int32), 4, 1)
    assert np.array_equal(img, np.ones((1, 16), np.float32))
    assert not msk.any()


def test_normalisation_makes_mean_one():
    prob = S.make_problem(S.tiny(side=16, n_images=5, rot_n=1))
    out, fac = O.normalize_images(prob.images, prob.mask)
    sel = prob.mask == 1
    np.testing.assert_allclose(out[:, sel].sum(1), 16 * 16, rtol=1e-5)
    assert np.all(fac > 0)


def test_radial_init_float_and_double_sums_agree():
    prob = S.make_problem(S.tiny(side=16, n_images=40, rot_n=1))
    mf, rf = O.model_init_radial(prob.images, 16, float_sums=True)
    md, rd = O.model_init_radial(prob.images, 16, float_sums=False)
    np.testing.assert_allclose(rf, rd, rtol=1e-5)
    assert rf[-1] == 0.0
    inside = mf >= 0
    np.testing.assert_allclose(mf[inside], md[inside], rtol=1e-5)
    assert np.array_equal(mf < 0, md < 0)


def test_orientation_init_weights_count_insertions():
    prob = S.make_problem(S.tiny(side=16, n_images=30, rot_n=1))
    q = E.random_rotations(3, 30)
    m, w = O.model_init_orientations(prob.images, prob.mask, 16, q, prob.x, prob.y, prob.z)
    assert w.sum() <= 30 * prob.mask.sum()
    assert np.all(w == np.round(w))
    assert np.all(m[w == 0] == 0)
