"""The reference-side binding: the reference's
cuda_* signatures implemented on libemc_gb300 (tests/refshim/).

CPU: the binding compiles against the reference's own emc_cuda_help.h and
links against the library.  GPU: one EMC iteration driven through those
signatures in main.cpp's order (rank set-up, scaling and likelihood passes
over rotation chunks, max / sum-exp / normalise, M-step with insertion over
chunks, divide, normalise) matches the oracle's restatement of the reference
iteration; cuda_set_device's context is the one every later call uses."""
import ctypes as C
import importlib.util
import os

import numpy as np
import pytest

from emc_gb300 import synthetic as S
from oracle import build as OB
from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))


def _recipe():
    spec = importlib.util.spec_from_file_location("refshim_build",
                                                  os.path.join(HERE, "refshim", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="module")
def shim(built):
    ref = OB.ref_dir()
    if ref is None:
        pytest.skip("no reference tree (EMC_REF_DIR or baseline/_ref/src)")
    so = _recipe().build(ref)
    lib = C.CDLL(str(so))
    P, I, F = C.c_void_p, C.c_int, C.c_float
    lib.shim_run_iteration.argtypes = [I, I, I, I, I, I, F] + [P] * 11
    lib.shim_run_iteration.restype = I
    lib.shim_device_after_set.argtypes = [I, I]
    lib.shim_device_after_set.restype = I
    return lib


def test_binding_compiles_against_reference_header(shim):
    for name in ("shim_run_iteration", "shim_device_after_set"):
        assert hasattr(shim, name)


@pytest.mark.gpu
def test_one_iteration_through_reference_signatures(shim, cuda):
    prob = S.make_problem(S.tiny(side=24, n_images=96, rot_n=2, photons=1200, seed=11))
    s, N, R = prob.cfg.side, prob.images.shape[0], prob.quats.shape[0]
    chunk = 100  # several chunks, the last one ragged
    sigma = O.sigma_at(0)
    f = lambda a: np.ascontiguousarray(a, np.float32)
    images, x, y, z = f(prob.images), f(prob.x), f(prob.y), f(prob.z)
    rot, rw = f(prob.quats), f(prob.weights)
    mask = np.ascontiguousarray(prob.mask, np.int32)
    model = f(prob.init_model).copy()
    weight = np.zeros(s ** 3, np.float32)
    respons = np.zeros((R, N), np.float32)
    scaling = np.zeros((R, N), np.float32)
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    dev = shim.shim_run_iteration(0, 5, s, N, R, chunk, sigma, p(images), p(mask), p(x), p(y),
                                  p(z), p(rot), p(rw), p(model), p(weight), p(respons),
                                  p(scaling))
    assert dev == 0
    want = O.ref_iteration(prob.init_model, prob.images, prob.mask, prob.x, prob.y, prob.z,
                           prob.quats, prob.weights, sigma, s, chunk=chunk)
    assert np.array_equal(scaling, want["scaling"], equal_nan=True)
    np.testing.assert_allclose(respons, want["respons"], rtol=2e-5, atol=1e-30)
    wm, ww = want["model"], want["weight"]
    np.testing.assert_allclose(weight, ww, rtol=2e-5, atol=1e-6 * ww.max())
    np.testing.assert_allclose(model, wm, rtol=2e-5, atol=1e-5 * np.abs(wm).max())


@pytest.mark.gpu
def test_set_device_context_is_used(shim, cuda):
    # main.cpp:127 sets the device once per rank; the binding keeps one context
    # on that device and replaces it when set again (no leaked second context)
    assert shim.shim_device_after_set(0, 3) == 0
    assert shim.shim_device_after_set(0, 4) == 0
