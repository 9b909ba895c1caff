"""GPU preprocessing and model initialisation against the oracle's
restatements of the reference host code: binning, normalisation and
per-pattern masks bit for bit; the radial-average model to the float
rounding of its ring sums; the random-orientation model with identical
weights (same voxel for every pixel) and sums to float rounding."""
import numpy as np
import pytest
import torch

import emc_gb300 as E
from emc_gb300 import synthetic as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def T(a, dev, dt=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)


@pytest.mark.parametrize("side,stride,raw_w,raw_h", [(16, 2, 32, 32), (12, 4, 48, 48),
                                                     (10, 3, 31, 29), (8, 1, 8, 8),
                                                     (9, 2, 12, 20)])
def test_bin_images_bit_exact(ctx, cuda, side, stride, raw_w, raw_h):
    rng = np.random.default_rng(side * 100 + stride)
    n = 7
    raw = rng.poisson(3.0, size=(n, raw_h, raw_w)).astype(np.float32)
    raw[:, 0, 0] = -2.5  # |value| is summed
    rmask = (rng.random(raw.shape) > 0.25).astype(np.int32)
    rmask[0] = 0  # a pattern with nothing unmasked: 0 / 0
    want_i, want_m = O.bin_images(raw, rmask, side, stride)
    img = torch.empty((n, side * side), device=cuda)
    msk = torch.empty((n, side * side), dtype=torch.int32, device=cuda)
    ctx.bin_images(T(raw, cuda), T(rmask, cuda, torch.int32), raw_w, raw_h, n, side, stride,
                   img, msk)
    ctx.sync()  # the context's stream is not torch's
    got = img.cpu().numpy()
    assert np.array_equal(np.isnan(got), np.isnan(want_i))
    assert np.array_equal(got[~np.isnan(got)].view(np.uint32),
                          want_i[~np.isnan(want_i)].view(np.uint32))
    assert np.array_equal(msk.cpu().numpy(), want_m)


@pytest.mark.parametrize("individual", [False, True])
def test_normalize_and_mask_bit_exact(ctx, cuda, individual):
    prob = S.make_problem(S.tiny(side=24, n_images=50, rot_n=1))
    n, n2 = prob.images.shape
    rng = np.random.default_rng(3)
    masks = (rng.random((n, n2)) > 0.1).astype(np.int32)
    want, _ = O.normalize_images(prob.images, prob.mask, masks if individual else None)
    img = T(prob.images, cuda)
    ctx.normalize_images(img, T(prob.mask, cuda, torch.int32), n2, n,
                         masks=T(masks, cuda, torch.int32) if individual else None)
    ctx.sync()
    assert np.array_equal(img.cpu().numpy().view(np.uint32), want.view(np.uint32))
    want_m = O.mask_images(want, masks)
    ctx.mask_model(img, T(masks, cuda, torch.int32), n2, n)
    ctx.sync()
    assert np.array_equal(img.cpu().numpy().view(np.uint32), want_m.view(np.uint32))


def test_model_init_radial(ctx, cuda):
    side = 32
    prob = S.make_problem(S.tiny(side=side, n_images=200, rot_n=1))
    model = torch.empty(side ** 3, device=cuda)
    ctx.model_init_radial(T(prob.images, cuda), prob.images.shape[0], side, model)
    ctx.sync()
    got = model.cpu().numpy()
    want_d, _ = O.model_init_radial(prob.images, side, float_sums=False)
    want_f, _ = O.model_init_radial(prob.images, side, float_sums=True)
    assert np.array_equal(got < 0, want_d < 0)
    assert np.all(got[got < 0] == -1.0)
    inside = want_d >= 0
    # FP64 ring sums in a different order: equal after rounding to float up to an ulp
    np.testing.assert_allclose(got[inside], want_d[inside], rtol=3e-7, atol=0)
    # the reference's sequential float sums differ by their own rounding
    np.testing.assert_allclose(got[inside], want_f[inside], rtol=1e-4, atol=0)


def test_model_init_orientations(ctx, cuda):
    side = 32
    prob = S.make_problem(S.tiny(side=side, n_images=300, rot_n=1))
    n = prob.images.shape[0]
    q = E.random_rotations(11, n)
    model = torch.empty(side ** 3, device=cuda)
    weight = torch.empty(side ** 3, device=cuda)
    ctx.model_init_orientations(T(prob.images, cuda), T(prob.mask, cuda, torch.int32), n, side,
                                T(q, cuda), T(prob.x, cuda), T(prob.y, cuda), T(prob.z, cuda),
                                model, weight)
    ctx.sync()
    want_m, want_w = O.model_init_orientations(prob.images, prob.mask, side, q, prob.x, prob.y,
                                               prob.z)
    assert np.array_equal(weight.cpu().numpy(), want_w)
    np.testing.assert_allclose(model.cpu().numpy(), want_m, rtol=2e-6, atol=1e-6)
