"""Pins the detector geometry (A2) and the preprocessing/model-initialisation
restatements (F2, F3) to the reference's own host code: emc_helper.cpp and
rotations.c compiled unchanged by oracle/build_ref.sh --helper (stand-ins for
libspimage, HDF5 and GSL in oracle/shim and oracle/ref_helper_harness.cpp).

* emc_calculate_coordinates (the library's host function) against
  calculate_coordinates (emc_helper.cpp:55-79): bit-identical.
* the oracle's binning, normalisation, masking and model initialisation
  (oracle/emc_oracle.c, which the GPU tests hold the CUDA kernels to) against
  read_images (:198-248), normalize_images* (:369-438), mask_model (:567-575)
  and model_init (:445-518).

No GPU is needed; skipped when the reference tree was not available to build
the helper."""
import ctypes as C

import numpy as np
import pytest

import emc_gb300 as E
from emc_gb300 import synthetic as S
from oracle import build as OB
from oracle import oracle as O


@pytest.fixture(scope="module")
def ref(built):
    lib = OB.ref_helper()
    if lib is None:
        pytest.skip("reference host helper not built (no reference tree)")
    return lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def ref_coordinates(ref, side, pixel, distance, wavelength):
    x, y, z = (np.zeros(side * side, np.float32) for _ in range(3))
    assert ref.refh_calculate_coordinates(side, pixel, distance, wavelength, _p(x), _p(y),
                                          _p(z)) == 0
    return x, y, z


@pytest.mark.parametrize("side", [1, 2, 24, 63, 64, 128, 256])
@pytest.mark.parametrize("geometry", [(S.PIXEL_SIZE, S.DISTANCE, S.WAVELENGTH),
                                      (600e-6, 0.3, 1.5e-10)], ids=["emc.conf", "wide"])
def test_coordinates_bit_identical_to_reference(ref, side, geometry):
    want = ref_coordinates(ref, side, *geometry)
    got = E.calculate_coordinates(side, *geometry)
    for g, w in zip(got, want):
        assert np.array_equal(g, w, equal_nan=True)


@pytest.mark.parametrize("side,stride,raw", [(16, 2, 32), (12, 4, 50), (8, 1, 8), (10, 3, 29)])
def test_binning_bit_identical_to_reference(ref, side, stride, raw):
    rng = np.random.default_rng(side * stride + raw)
    n = 5
    frames = rng.poisson(3.0, size=(n, raw, raw)).astype(np.float32)
    frames[0, :3] = -2.5  # |raw| is summed
    fmask = (rng.random(frames.shape) > 0.25).astype(np.int32)
    fmask[1] = 0  # a frame with no unmasked pixel: 0/0 everywhere
    want_i = np.zeros((n, side * side), np.float32)
    want_m = np.zeros((n, side * side), np.int32)
    assert ref.refh_read_images(_p(frames), _p(fmask), raw, raw, n, side, stride, _p(want_i),
                                _p(want_m)) == 0
    got_i, got_m = O.bin_images(frames, fmask, side, stride)
    assert np.array_equal(got_i, want_i, equal_nan=True)
    assert np.array_equal(got_m, want_m)


@pytest.mark.parametrize("individual", [False, True])
def test_normalisation_bit_identical_to_reference(ref, individual):
    rng = np.random.default_rng(3)
    side, n = 20, 7
    images = rng.poisson(4.0, size=(n, side * side)).astype(np.float32)
    mask = (rng.random(side * side) > 0.2).astype(np.int32)
    masks = (rng.random((n, side * side)) > 0.3).astype(np.int32)
    got, _ = O.normalize_images(images, mask, masks if individual else None)
    for mode in ((2,) if individual else (0, 1)):  # 0 and 1: common mask, central part all ones
        want = images.copy()
        assert ref.refh_normalize_images(_p(want), _p(mask), _p(masks), n, side, mode, 5.0) == 0
        assert np.array_equal(got, want)


def test_mask_model_identical_to_reference(ref):
    rng = np.random.default_rng(4)
    side, n = 16, 4
    images = rng.random((n, side * side)).astype(np.float32)
    masks = (rng.random((n, side * side)) > 0.5).astype(np.int32)
    want = images.copy()
    assert ref.refh_mask_model(_p(want), _p(masks), n, side) == 0
    assert np.array_equal(O.mask_images(images, masks), want)


@pytest.mark.parametrize("side", [16, 24, 33])
def test_radial_model_matches_reference(ref, side):
    rng = np.random.default_rng(side)
    n = 6
    images = rng.poisson(5.0, size=(n, side * side)).astype(np.float32)
    want = np.zeros(side ** 3, np.float32)
    weight = np.zeros(side ** 3, np.float32)
    x, y, z = E.calculate_coordinates(side, S.PIXEL_SIZE, S.DISTANCE, S.WAVELENGTH)
    mask = np.ones(side * side, np.int32)
    assert ref.refh_model_init(3, _p(images), _p(mask), n, side, _p(x), _p(y), _p(z), 0,
                               _p(want), _p(weight)) == 0
    got, _ = O.model_init_radial(images, side, float_sums=True)
    # voxels of the outermost rings read radavg[side/2], one past the
    # reference's array (emc_helper.cpp:494; for an odd side its ring sums also
    # write there): its value is whatever follows the allocation, so voxels
    # with r >= side/2 - 1 are left out
    c = np.arange(side, dtype=np.float64) - side / 2.0 + 0.5
    rad = np.sqrt(c[None, None, :] ** 2 + c[None, :, None] ** 2 + c[:, None, None] ** 2)
    keep = (rad.astype(np.float32).astype(np.int32) < side // 2 - 1).reshape(-1)
    assert keep.sum() > side ** 3 // 3
    np.testing.assert_array_equal(got[keep], want[keep])


def test_orientation_model_identical_to_reference(ref):
    """model_input 1: each pattern inserted once at a random orientation.  The
    reference draws the orientations from GSL's taus generator; here both
    sides take them from the same stand-in stream (rotations.c's own
    quaternion_random on it), so what is compared is the insertion and the
    division."""
    side, n = 24, 40
    prob = S.make_problem(S.tiny(side=side, n_images=n, rot_n=1, photons=800, seed=5))
    seed = 1234
    quats = np.zeros((n, 4), np.float32)
    assert ref.refh_quaternion_random(seed, n, _p(quats)) == 0
    want = np.zeros(side ** 3, np.float32)
    want_w = np.zeros(side ** 3, np.float32)
    images = np.ascontiguousarray(prob.images, np.float32)
    mask = np.ascontiguousarray(prob.mask, np.int32)
    assert ref.refh_model_init(1, _p(images), _p(mask), n, side, _p(prob.x), _p(prob.y),
                               _p(prob.z), seed, _p(want), _p(want_w)) == 0
    got, got_w = O.model_init_orientations(images, mask, side, quats, prob.x, prob.y, prob.z)
    assert want_w.sum() > 0
    assert np.array_equal(got_w, want_w)
    assert np.array_equal(got, want)
