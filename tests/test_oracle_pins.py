"""Pins the oracle to the reference's own kernels.

tests/golden/ref_kernels_golden.npz holds the outputs of the reference's
emc_cuda.cu / emc_atomic.cu compiled unchanged for sm_103a and run on a GB300
(tests/golden/make_ref_kernel_golden.py), on a seeded 24^3 problem with 96
rotations and 64 patterns.  The C restatement in oracle/emc_oracle.c must
reproduce them: bit for bit where the reference's arithmetic is fixed
(slicing, the int-truncated scaling, the M-step slices, max, divide,
normalise), to one float ulp where CUDA's logf/expf/pow and glibc's differ
or the reference's atomics fix no order."""
import os

import numpy as np
import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
G = np.load(os.path.join(ROOT, "tests", "golden", "ref_kernels_golden.npz"))
S = int(G["side"])
Q = G["quats"]
R, N = Q.shape[0], G["images"].shape[0]


def test_slices_bit_exact(built):
    assert np.array_equal(O.get_slices(G["model"], S, Q, G["x"], G["y"], G["z"]), G["slices"])
    assert (G["slices"] == -1).any()


def test_scaling_bit_exact_including_int_truncation(built):
    got = np.ones((R, N), np.float32)
    O.update_scaling_full(G["images"], G["slices"], G["mask"], got, 0)
    assert np.array_equal(got, G["scaling"], equal_nan=True)


@pytest.mark.parametrize("diff,name", [(1, "respons_poisson"), (0, "respons_absolute")])
def test_likelihood_within_one_ulp(built, diff, name):
    got = np.zeros((R, N), np.float32)
    O.calculate_responsabilities(G["slices"], G["images"], G["mask"], np.float32(0.3),
                                 G["scaling"], got, G["weights"], 0, diff)
    np.testing.assert_allclose(got, G[name], rtol=2.4e-7, atol=0)


def test_log_sum_exp_chain(built):
    resp = G["respons_poisson"]
    mx = O.max_vector(resp, N)
    assert np.array_equal(mx, G["maxr"])
    sums = O.respons_max_expf(resp, G["maxr"], N)
    np.testing.assert_allclose(sums, G["sums"], rtol=2.4e-7)
    r = resp.copy()
    lse = O.normalize_respons(r, G["sums"], G["maxr"], N)
    assert np.array_equal(lse, G["lse_host"])
    np.testing.assert_allclose(r, G["respons_norm"], rtol=4e-7, atol=1e-30)


def test_mstep_slices_bit_exact_and_insert(built):
    act = np.ones(N, np.int32)
    sl, tot = O.update_slices(G["images"], G["mask"], G["respons_norm"], G["scaling"], act, 16, 60)
    assert np.array_equal(sl, G["upd_slices"])
    m = np.zeros(S ** 3, np.float32)
    w = np.zeros(S ** 3, np.float32)
    O.insert_slices(G["upd_slices"], G["mask"], tot, Q[16:76], G["x"], G["y"], G["z"], S, m, w)
    assert np.array_equal(m != 0, G["ins_model"] != 0)  # same voxels touched
    np.testing.assert_allclose(m, G["ins_model"], rtol=1e-6, atol=1e-6 * G["ins_model"].max())
    np.testing.assert_allclose(w, G["ins_weight"], rtol=1e-6, atol=1e-6 * G["ins_weight"].max())


def test_divide_average_normalize_bit_exact(built):
    d = G["ins_model"].copy()
    O.divide_model(d, G["ins_weight"])
    assert np.array_equal(d, G["divided"])
    assert np.float32(O.model_average(G["divided"])) == G["avg_before"]
    n = G["divided"].copy()
    O.normalize_model(n)
    assert np.array_equal(n, G["normalized"])
