"""Pruned iterations against full scans from the same start.

Problem: 64^3, 4,000 patterns, 25,680 rotations (level 8): 32 pattern tiles x
201 rotation tiles.  Started from the true particle, the counts x log-slice
Poisson likelihood is peaked from the first iteration, so every iteration
after the first evaluates a subset of the (pattern, rotation) tiles.  The
pruned iteration stays within 1e-4 relative L2 (model) and 1e-5 (total
log-likelihood) of a full scan from the same input model, and its
responsibilities (mapped back to the input pattern and rotation order)
within 1e-3 of the full scan's.  The
reference's likelihood is peaked only at a very small sigma; a jump to a wide
sigma spreads the mass into the margin tiles and the iteration is repeated as
a full scan."""
import numpy as np
import pytest
import torch

import emc_gb300 as E
from emc_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def prob():
    cfg = S.Config("prune64", 64, 400, 1.5, 12, 4000, 3000, (0.5, 1.5), 4, 8, 1, seed=3)
    return S.make_problem(cfg, device="cuda")


def T(a, dev, dt=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)


def make_plan(ctx, prob, dev, diff):
    s, R, N = prob.cfg.side, prob.quats.shape[0], prob.images.shape[0]
    plan = E.Plan(ctx, s, N, R, diff=diff, precision=E.PREC_MIXED,
                  insert_mode=E.INSERT_DETERMINISTIC)
    inputs = (T(prob.images, dev), T(prob.mask, dev, torch.int32), T(prob.x, dev), T(prob.y, dev),
              T(prob.z, dev), T(prob.quats, dev), T(prob.weights, dev))
    plan.bind(*inputs)
    plan._inputs = inputs
    return plan


def start_model(ctx, prob, dev):
    m = T(prob.true_model, dev)
    ctx.normalize_model(prob.cfg.side, m)
    return m, torch.empty_like(m)


def respons(ctx, plan, R, N):
    r_ptr, _, _ = plan.results()
    ctx.sync()
    return ctx.copy_real_to_host(r_ptr, R * N).reshape(R, N)


def rel(a, b):
    a, b = a.cpu().numpy().astype(np.float64), b.cpu().numpy().astype(np.float64)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_pruned_iterations_match_full_scans(ctx, cuda, prob):
    """Each iteration of the pruned run against a full scan from the same
    input model: the only differences are the skipped mass (< 1 - min_mass)
    and the FP32 summation order of the re-sorted patterns."""
    R, N = prob.quats.shape[0], prob.images.shape[0]
    full = make_plan(ctx, prob, cuda, E.DIFF_TRUE_POISSON)
    pr = make_plan(ctx, prob, cuda, E.DIFF_TRUE_POISSON)
    pr.set_pruning(True, min_mass=0.999, dilate=1.0)
    mp, wp = start_model(ctx, prob, cuda)
    wf = torch.empty_like(wp)
    infos = []
    for it in range(6):
        mf = mp.clone()
        torch.cuda.synchronize()
        sf = full.iterate(mf, wf, 0.1)
        sp = pr.iterate(mp, wp, 0.1)
        info = pr.prune_info()
        infos.append(info)
        assert rel(mp, mf) < 1e-4
        assert abs(sp.total_loglik - sf.total_loglik) <= 1e-5 * abs(sf.total_loglik)
        order, rorder = pr.pattern_order(), pr.rotation_order()
        assert sorted(order.tolist()) == list(range(N))
        assert sorted(rorder.tolist()) == list(range(R))
        pf = respons(ctx, full, R, N)
        pp = np.empty_like(pf)
        pp[np.ix_(rorder, order)] = respons(ctx, pr, R, N)
        assert np.abs(pp - pf).max() < 1e-3
        assert abs(sp.captured_mass - 1.0) < 1e-4
    assert infos[0]["full_iterations"] == 1 and infos[0]["pruned"] == 0
    assert infos[-1]["pruned_iterations"] >= 2
    assert min(i["active_fraction"] for i in infos) < 0.75
    full.close()
    pr.close()


def test_fallback_repeats_as_full_scan(ctx, cuda, prob):
    """The reference's likelihood prunes at a very small sigma; its mass then
    moves between iterations (or spreads, after the jump to sigma 4) beyond
    the margin, and the attempts are repeated as full scans."""
    full = make_plan(ctx, prob, cuda, E.DIFF_POISSON)
    pr = make_plan(ctx, prob, cuda, E.DIFF_POISSON)
    pr.set_pruning(True, min_mass=0.999, dilate=1.0)
    mp, wp = start_model(ctx, prob, cuda)
    wf = torch.empty_like(wp)
    for sg in (0.005, 0.005, 4.0):
        mf = mp.clone()
        torch.cuda.synchronize()
        sf = full.iterate(mf, wf, sg)
        sp = pr.iterate(mp, wp, sg)
        assert rel(mp, mf) < 1e-4
        assert abs(sp.total_loglik - sf.total_loglik) <= 1e-5 * abs(sf.total_loglik)
    info = pr.prune_info()
    assert info["pruned"] == 1 and info["fallback"] == 1
    assert info["fallback_iterations"] >= 1 and info["margin_mass"] > 1e-3
    pr.set_pruning(False)  # back to the input order
    assert np.array_equal(pr.pattern_order(), np.arange(prob.images.shape[0]))
    assert np.array_equal(pr.rotation_order(), np.arange(prob.quats.shape[0]))
    full.close()
    pr.close()


def test_periodic_full_scan(ctx, cuda, prob):
    pr = make_plan(ctx, prob, cuda, E.DIFF_TRUE_POISSON)
    pr.set_pruning(True, min_mass=0.999, dilate=1.0, full_every=2)
    m, w = start_model(ctx, prob, cuda)
    kinds = []
    for _ in range(8):
        pr.iterate(m, w, 0.1)
        i = pr.prune_info()
        kinds.append((i["pruned"], i["active_fraction"] < 0.75))
    # never two pruned attempts in a row; a full scan whose mask is sparse
    # enough is followed by a pruned attempt
    for (a, _), (b, _) in zip(kinds, kinds[1:]):
        assert not (a and b)
    for (a, sparse), (b, _) in zip(kinds, kinds[1:]):
        if not a and sparse:
            assert b
    assert any(a for a, _ in kinds)
    pr.close()


def test_pruning_needs_the_tensor_path(ctx, cuda, prob):
    s, R, N = prob.cfg.side, prob.quats.shape[0], prob.images.shape[0]
    plan = E.Plan(ctx, s, N, R, precision=E.PREC_FP32)
    with pytest.raises(E.EmcError):
        plan.set_pruning(True)  # not bound
    plan.bind(T(prob.images, cuda), T(prob.mask, cuda, torch.int32), T(prob.x, cuda),
              T(prob.y, cuda), T(prob.z, cuda), T(prob.quats, cuda), T(prob.weights, cuda))
    with pytest.raises(E.EmcError):
        plan.set_pruning(True)
    plan.close()
