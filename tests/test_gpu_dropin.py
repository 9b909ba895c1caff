"""Parity of the drop-in entry points (reference semantics) against the oracle.

Every call goes through the C ABI (emc_gb300.Context -> libemc_gb300.so).
Bit-exact where the reference's arithmetic has no transcendental function
and no order freedom (slicing, scaling, update_slices, max, divide); within
the stated float tolerances where logf/expf differ by an ulp between CUDA
and glibc or where the reference's float atomics make the order free."""
import numpy as np
import pytest
import torch

import emc_gb300 as E
from emc_gb300 import synthetic as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def T(a, dev, dt=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)


@pytest.fixture(scope="module")
def prob():
    return S.make_problem(S.tiny(side=24, n_images=70, rot_n=2, photons=2000))


@pytest.fixture(scope="module")
def dev_prob(prob, cuda):
    p = prob
    return dict(model=T(p.init_model, cuda), x=T(p.x, cuda), y=T(p.y, cuda), z=T(p.z, cuda),
                rot=T(p.quats, cuda), w=T(p.weights, cuda), images=T(p.images, cuda),
                mask=T(p.mask, cuda, torch.int32))


@pytest.mark.parametrize("interp", [E.INTERP_NEAREST, E.INTERP_TRILINEAR])
def test_get_slices_bit_exact(ctx, prob, dev_prob, interp):
    d, s = dev_prob, prob.cfg.side
    R = prob.quats.shape[0]
    out = torch.full((R - 7, s * s), 7.0, device=d["model"].device)
    ctx.get_slices(d["model"], s, out, d["rot"], d["x"], d["y"], d["z"], 5, R - 7, interp)
    ctx.sync()
    ref = O.get_slices(prob.init_model, s, prob.quats[5:R - 2], prob.x, prob.y, prob.z, interp)
    assert np.array_equal(out.cpu().numpy(), ref)
    if interp == E.INTERP_NEAREST:
        assert (ref == -1).any()  # out-of-volume sentinel exercised


def test_get_slices_odd_side_and_empty_chunk(ctx, cuda):
    s = 7
    model = np.random.default_rng(1).random(s ** 3).astype(np.float32)
    x, y, z = E.calculate_coordinates(s, 75e-6, 0.74, 1.03e-9)
    q, _ = E.generate_rotations(1)
    out = torch.empty((q.shape[0], s * s), device=cuda)
    ctx.get_slices(T(model, cuda), s, out, T(q, cuda), T(x, cuda), T(y, cuda), T(z, cuda), 0,
                   q.shape[0])
    ctx.get_slices(T(model, cuda), s, out, T(q, cuda), T(x, cuda), T(y, cuda), T(z, cuda), 0, 0)
    ctx.sync()
    assert np.array_equal(out.cpu().numpy(), O.get_slices(model, s, q, x, y, z))


def test_scaling_bit_exact_with_int_truncation(ctx, prob, dev_prob):
    d, s = dev_prob, prob.cfg.side
    R, N = prob.quats.shape[0], prob.images.shape[0]
    sl = O.get_slices(prob.init_model, s, prob.quats, prob.x, prob.y, prob.z)
    start, chunk = 3, R - 10
    got = torch.ones((R, N), device=d["model"].device)
    ctx.update_scaling_full(d["images"], T(sl[start:start + chunk], d["model"].device), d["mask"],
                            got, s * s, N, start, chunk)
    ctx.sync()
    want = np.ones((R, N), np.float32)
    O.update_scaling_full(prob.images, sl[start:start + chunk], prob.mask, want, start)
    assert np.array_equal(got.cpu().numpy(), want)
    # the quirk is real: a float denominator gives a different answer
    K = prob.images.astype(np.float64)
    Sd = sl[start].astype(np.float64)
    m = (prob.mask > 0) & (Sd > 1e-10)
    num = ((K ** 2) * (m & (K > 1e-10))).sum(1)
    den = (K * Sd * (m & (K > 1e-10))).sum(1)
    assert not np.allclose(want[start], num / den, rtol=1e-3)


@pytest.mark.parametrize("diff", [E.DIFF_POISSON, E.DIFF_ABSOLUTE, E.DIFF_RELATIVE])
def test_responsabilities(ctx, prob, dev_prob, diff):
    d, s = dev_prob, prob.cfg.side
    R, N = prob.quats.shape[0], prob.images.shape[0]
    sl = O.get_slices(prob.init_model, s, prob.quats, prob.x, prob.y, prob.z)
    scal = np.ones((R, N), np.float32)
    O.update_scaling_full(prob.images, sl, prob.mask, scal, 0)
    want = np.zeros((R, N), np.float32)
    sigma = np.float32(0.3)
    O.calculate_responsabilities(sl, prob.images, prob.mask, sigma, scal, want, prob.weights, 0, diff)
    got = torch.zeros((R, N), device=d["model"].device)
    ctx.calculate_responsabilities(T(sl, d["model"].device), d["images"], d["mask"], sigma,
                                   T(scal, d["model"].device), got, d["w"], s * s, N, 0, R, diff)
    ctx.sync()
    g = got.cpu().numpy()
    # the per-pair sums are identical; only logf(w) may differ by an ulp
    np.testing.assert_allclose(g, want, rtol=2e-6, atol=2e-6)


def test_lse_chain(ctx, prob, cuda):
    rng = np.random.default_rng(3)
    R, N = 1300, 37
    L = (rng.standard_normal((R, N)) * 30 - 200).astype(np.float32)
    L[5, :] = -1e12  # below the -1e10 cut
    L[:, 3] = np.nan  # NaN entries are skipped by the max
    L[7, 3] = -50.0
    dL = T(L, cuda)
    mx = torch.empty(N, device=cuda)
    ctx.max_vector(dL, N, R, mx)
    ctx.sync()
    want_max = O.max_vector(L, N)
    assert np.array_equal(mx.cpu().numpy(), want_max)
    sm = torch.empty(N, device=cuda)
    ctx.respons_max_expf(dL, mx, N, R, sm)
    want_sum = O.respons_max_expf(L, want_max, N)
    ok = np.isfinite(want_sum)
    np.testing.assert_allclose(sm.cpu().numpy()[ok], want_sum[ok], rtol=1e-5)
    lse = torch.empty(N, device=cuda)
    ctx.log_sum_max(sm, mx, lse, N)
    ctx.norm_respons_sumexpf(dL, lse, mx, N, R)
    ctx.sync()
    Lw = L.copy()
    O.normalize_respons(Lw, want_sum, want_max, N)
    g = dL.cpu().numpy()
    fin = np.isfinite(Lw)
    np.testing.assert_allclose(g[fin], Lw[fin], rtol=2e-5, atol=1e-30)


def test_update_slices_and_insert(ctx, prob, dev_prob):
    d, s = dev_prob, prob.cfg.side
    dev = d["model"].device
    R, N = prob.quats.shape[0], prob.images.shape[0]
    ref = O.ref_iteration(prob.init_model, prob.images, prob.mask, prob.x, prob.y, prob.z,
                          prob.quats, prob.weights, O.sigma_at(0), s)
    resp, scal = ref["respons"], ref["scaling"]
    active = np.ones(N, np.int32)
    active[4] = 0
    start, chunk = 11, R - 20
    slices = torch.zeros((chunk, s * s), device=dev)
    model = torch.zeros(s ** 3, device=dev)
    weight = torch.zeros(s ** 3, device=dev)
    ctx.update_slices(d["images"], slices, d["mask"], T(resp, dev), T(scal, dev),
                      T(active, dev, torch.int32), N, start, chunk, s * s, s, model, d["x"],
                      d["y"], d["z"], d["rot"][start:start + chunk].contiguous(), weight)
    ctx.sync()
    want_sl, tot = O.update_slices(prob.images, prob.mask, resp, scal, active, start, chunk)
    assert np.array_equal(slices.cpu().numpy(), want_sl)
    wm = np.zeros(s ** 3, np.float32)
    ww = np.zeros(s ** 3, np.float32)
    O.insert_slices(want_sl, prob.mask, tot, prob.quats[start:start + chunk], prob.x, prob.y,
                    prob.z, s, wm, ww)
    np.testing.assert_allclose(model.cpu().numpy(), wm, rtol=2e-5, atol=1e-6 * wm.max())
    np.testing.assert_allclose(weight.cpu().numpy(), ww, rtol=2e-5, atol=1e-6 * ww.max())
    assert (ww > 0).sum() > 100


def test_divide_normalize_max_average(ctx, cuda):
    rng = np.random.default_rng(5)
    s = 20
    m = (rng.random(s ** 3) * 3).astype(np.float32)
    w = rng.random(s ** 3).astype(np.float32)
    w[rng.random(s ** 3) < 0.2] = 0.0
    dm, dw = T(m, cuda), T(w, cuda)
    ctx.divide_model_by_weight(s, dm, dw)
    ctx.sync()
    want = m.copy()
    O.divide_model(want, w)
    assert np.array_equal(dm.cpu().numpy(), want)
    avg = ctx.model_average(dm)
    assert abs(avg - O.model_average(want)) <= 2e-6 * avg
    mx = ctx.model_max(dm)
    assert mx == max(0.0, float(want.max()))
    before = ctx.normalize_model(s, dm)
    ctx.sync()
    O.normalize_model(want)
    assert abs(before - avg) <= 1e-6 * avg
    np.testing.assert_allclose(dm.cpu().numpy(), want, rtol=2e-6)


@pytest.mark.parametrize("side,sigma", [(24, 1.0), (17, 0.7), (32, 3.0), (16, 40.0)])
def test_blur_matches_fft(ctx, cuda, side, sigma):
    rng = np.random.default_rng(side)
    m = (rng.random(side ** 3) * 2).astype(np.float32)
    m[rng.random(side ** 3) < 0.1] = -1.0
    dm = T(m, cuda)
    ctx.blur_model(dm, side, sigma)
    ctx.sync()
    want = O.blur_fft_fp64(m, side, sigma)
    got = dm.cpu().numpy()
    assert np.array_equal(got == -1.0, want == -1.0)
    np.testing.assert_allclose(got, want, atol=2e-6 * np.abs(want).max())


def test_degenerate_inputs_follow_reference(ctx, cuda):
    """count == 0 gives NaN and a zero-photon pattern NaN scaling, as in the
    reference (emc_cuda.cu:274, 453)."""
    s = 8
    N, R = 3, 4
    images = np.zeros((N, s * s), np.float32)
    images[1, 10] = 5.0
    mask = np.zeros(s * s, np.int32)
    mask[8:40] = 1
    sl = np.full((R, s * s), -1.0, np.float32)
    sl[:2, 8:40] = 0.5
    scal = np.ones((R, N), np.float32)
    d_scal = T(scal, cuda)
    ctx.update_scaling_full(T(images, cuda), T(sl, cuda), T(mask, cuda, torch.int32), d_scal,
                            s * s, N, 0, R)
    O.update_scaling_full(images, sl, mask, scal, 0)
    ctx.sync()
    np.testing.assert_array_equal(d_scal.cpu().numpy(), scal)
    assert np.isnan(scal[0, 0]) and np.isnan(scal[3, 1])
    resp = np.zeros((R, N), np.float32)
    O.calculate_responsabilities(sl, images, mask, np.float32(0.3), np.ones((R, N), np.float32),
                                 resp, np.full(R, 0.25, np.float32), 0, 1)
    d_resp = torch.zeros((R, N), device=cuda)
    ctx.calculate_responsabilities(T(sl, cuda), T(images, cuda), T(mask, cuda, torch.int32), 0.3,
                                   torch.ones((R, N), device=cuda), d_resp,
                                   T(np.full(R, 0.25, np.float32), cuda), s * s, N, 0, R)
    ctx.sync()
    np.testing.assert_allclose(d_resp.cpu().numpy(), resp, rtol=2e-6, equal_nan=True)
    assert np.isnan(resp[2:]).all()


def test_against_reference_kernel_golden(ctx, cuda):
    """The drop-ins against the reference's own kernels (run on a GB300,
    tests/golden/ref_kernels_golden.npz): bit-exact slicing, scaling and
    M-step slices, likelihood within one float ulp."""
    import os
    G = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_kernels_golden.npz"))
    s = int(G["side"])
    q = G["quats"]
    R, N = q.shape[0], G["images"].shape[0]
    d = {k: T(G[k], cuda) for k in ("model", "x", "y", "z", "quats", "weights", "images")}
    mask = T(G["mask"], cuda, torch.int32)
    sl = torch.empty((R, s * s), device=cuda)
    ctx.get_slices(d["model"], s, sl, d["quats"], d["x"], d["y"], d["z"], 0, R)
    scal = torch.ones((R, N), device=cuda)
    ctx.update_scaling_full(d["images"], sl, mask, scal, s * s, N, 0, R)
    resp = torch.zeros((R, N), device=cuda)
    ctx.calculate_responsabilities(sl, d["images"], mask, 0.3, scal, resp, d["weights"], s * s, N,
                                   0, R)
    upd = torch.zeros((60, s * s), device=cuda)
    m = torch.zeros(s ** 3, device=cuda)
    w = torch.zeros(s ** 3, device=cuda)
    ctx.update_slices(d["images"], upd, mask, T(G["respons_norm"], cuda), scal,
                      T(np.ones(N, np.int32), cuda, torch.int32), N, 16, 60, s * s, s, m, d["x"],
                      d["y"], d["z"], d["quats"][16:76].contiguous(), w)
    ctx.sync()
    assert np.array_equal(sl.cpu().numpy(), G["slices"])
    assert np.array_equal(scal.cpu().numpy(), G["scaling"], equal_nan=True)
    np.testing.assert_allclose(resp.cpu().numpy(), G["respons_poisson"], rtol=2.4e-7)
    assert np.array_equal(upd.cpu().numpy(), G["upd_slices"])
    np.testing.assert_allclose(m.cpu().numpy(), G["ins_model"], rtol=1e-6,
                               atol=1e-6 * G["ins_model"].max())
    np.testing.assert_allclose(w.cpu().numpy(), G["ins_weight"], rtol=1e-6,
                               atol=1e-6 * G["ins_weight"].max())


def test_bad_arguments_raise(ctx, cuda):
    z = torch.zeros(16, device=cuda)
    with pytest.raises(E.EmcError):
        ctx.get_slices(z, 0, z, z, z, z, z, 0, 1)
    with pytest.raises(E.EmcError):
        ctx.calculate_responsabilities(z, z, torch.zeros(4, dtype=torch.int32, device=cuda), 0.3,
                                       z, z, z, 4, 1, 0, 1, diff=9)
    with pytest.raises(E.EmcError):
        ctx.blur_model(z, 2000, 1.0)
