"""The likelihood kernel on CTA pairs (EMC_OPT_ESTEP_PAIR) against the
single-CTA kernel.

Both compute every (pattern, rotation) element from the same FP16 operands
with the same 16-pixel MMA steps; the pair runs them as 256-row MMAs with the
rotation-side operands split between two CTAs.  Cases: an odd number of
pattern tiles (the last pair's second CTA has no patterns), ragged pattern
and rotation counts, counts above 45 (K^2 lo blocks), known intensity (H lo
halves), normalised images, and the tile orders of the autotuner."""
import numpy as np
import pytest
import torch

import emc_gb300 as E
from emc_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


def T(a, dev, dt=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)


def run(ctx, prob, dev, pair, raster=8, **kw):
    s, R, N = prob.cfg.side, prob.quats.shape[0], prob.images.shape[0]
    plan = E.Plan(ctx, s, N, R, precision=E.PREC_MIXED, insert_mode=E.INSERT_DETERMINISTIC, **kw)
    plan.set_option(E.Plan.OPT_ESTEP_PAIR, pair)
    plan.bind(T(prob.images, dev), T(prob.mask, dev, torch.int32), T(prob.x, dev), T(prob.y, dev),
              T(prob.z, dev), T(prob.quats, dev), T(prob.weights, dev))
    plan.set_option(E.Plan.OPT_ESTEP_RASTER, raster)
    m = T(prob.init_model, dev)
    w = torch.empty_like(m)
    st = plan.iterate(m, w, 0.3)
    r_ptr, s_ptr, _ = plan.results()
    ctx.sync()
    L = ctx.copy_real_to_host(r_ptr, R * N)
    phi = ctx.copy_real_to_host(s_ptr, R * N)
    plan.close()
    return m.cpu().numpy(), L, phi, st


CASES = {
    # 3 pattern tiles (odd), 1,380 rotations (ragged), bright patterns
    "odd_tiles": (dict(side=32, n_images=300, rot_n=3, photons=6000, n_atoms=120, radius=7.0), {}),
    "known_intensity": (dict(side=32, n_images=260, rot_n=3, photons=4000, n_atoms=120,
                             radius=7.0), dict(known_intensity=1)),
    "normalised": (dict(side=48, n_images=700, rot_n=4, photons=3000, n_atoms=150, radius=9.0,
                        seed=3), dict(normalize_images=1)),
}


@pytest.mark.parametrize("case", list(CASES))
def test_pair_matches_single_cta(ctx, cuda, case):
    cfg_kw, plan_kw = CASES[case]
    prob = S.make_problem(S.tiny(**cfg_kw))
    if case == "odd_tiles":
        assert prob.images.max() > 45  # K^2 lo blocks are used
    m1, L1, p1, st1 = run(ctx, prob, cuda, 0, **plan_kw)
    for raster in (8, -19, 2):
        m2, L2, p2, st2 = run(ctx, prob, cuda, 1, raster, **plan_kw)
        ok = np.isfinite(L1)
        assert np.array_equal(ok, np.isfinite(L2))
        assert np.abs(L2[ok] - L1[ok]).max() <= 1e-6 * max(1.0, np.abs(L1[ok]).max())
        np.testing.assert_allclose(p2, p1, rtol=1e-6)
        np.testing.assert_allclose(m2, m1, rtol=1e-5, atol=1e-7)
        assert abs(st2.total_loglik - st1.total_loglik) <= 1e-6 * abs(st1.total_loglik)
        assert st2.bad_pairs == st1.bad_pairs


def test_pair_autotune_and_window(ctx, cuda):
    prob = S.make_problem(S.tiny(side=32, n_images=900, rot_n=4, photons=3000, n_atoms=120,
                                 radius=7.0))
    s, R, N = prob.cfg.side, prob.quats.shape[0], prob.images.shape[0]
    plan = E.Plan(ctx, s, N, R, precision=E.PREC_MIXED)
    plan.bind(T(prob.images, cuda), T(prob.mask, cuda, torch.int32), T(prob.x, cuda),
              T(prob.y, cuda), T(prob.z, cuda), T(prob.quats, cuda), T(prob.weights, cuda))
    m = T(prob.init_model, cuda)
    ms, total = plan.time_likelihood(8, model=m, sigma=0.3)
    assert total == ((N + 127) // 128 + 1) // 2 * ((R + 127) // 128) and ms > 0
    raster, t = plan.autotune(m, 0.3)
    assert raster != 0 and t > 0
    plan.close()


def run_mstep(ctx, prob, dev, pair, q_lo=0, raster=-16):
    s, R, N = prob.cfg.side, prob.quats.shape[0], prob.images.shape[0]
    plan = E.Plan(ctx, s, N, R, precision=E.PREC_MIXED, insert_mode=E.INSERT_DETERMINISTIC)
    plan.set_option(E.Plan.OPT_MSTEP_PAIR, pair)
    plan.set_option(E.Plan.OPT_MSTEP_QLO, q_lo)
    plan.set_option(E.Plan.OPT_MSTEP_RASTER, raster)
    plan.bind(T(prob.images, dev), T(prob.mask, dev, torch.int32), T(prob.x, dev), T(prob.y, dev),
              T(prob.z, dev), T(prob.quats, dev), T(prob.weights, dev))
    m = T(prob.init_model, dev)
    w = torch.empty_like(m)
    st = plan.iterate(m, w, 0.3)
    plan.close()
    return m.cpu().numpy(), w.cpu().numpy(), st


@pytest.mark.parametrize("q_lo", [0, 1])
def test_mstep_pair_matches_single_cta(ctx, cuda, q_lo):
    """The M-step on CTA pairs (EMC_OPT_MSTEP_PAIR) against single CTAs: an odd
    number of 128-rotation tiles (the last pair's second CTA has no
    rotations), a ragged pixel count, Q hi and Q hi + lo, two tile orders;
    deterministic insertion, so equal sums give equal models."""
    prob = S.make_problem(S.tiny(side=40, n_images=500, rot_n=3, photons=3000, n_atoms=120,
                                 radius=8.0, seed=4))
    R = prob.quats.shape[0]
    assert ((R + 127) // 128) % 2 == 1
    m1, w1, st1 = run_mstep(ctx, prob, cuda, 0, q_lo)
    for raster in (-16, 3):
        m2, w2, st2 = run_mstep(ctx, prob, cuda, 1, q_lo, raster)
        np.testing.assert_allclose(w2, w1, rtol=1e-6, atol=1e-6 * np.abs(w1).max())
        np.testing.assert_allclose(m2, m1, rtol=1e-5, atol=1e-6 * np.abs(m1).max())
        assert abs(st2.total_loglik - st1.total_loglik) <= 1e-9 * abs(st1.total_loglik)
