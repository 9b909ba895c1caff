"""The learned rotation proposal on the GPU.

* inputs, loss and every parameter gradient of the CUDA network against the
  FP64 oracle (oracle/proposal.py) on the same parameters and patterns;
* labels: emc_plan_best_quaternions equals the argmax of the results;
* seeding a pruned iteration from proposals: true orientations (and their
  Friedel mates) give a pruned iteration that matches the full scan; random
  proposals put mass in the margin and the iteration is repeated as a full
  scan, which then equals the full scan;
* training on EMC's own labels lowers the loss and predicts held-out
  patterns' rotations far better than chance."""
import numpy as np
import pytest
import torch

import emc_gb300 as E
from emc_gb300 import synthetic as S
from oracle import proposal as PO

pytestmark = pytest.mark.gpu


def T(a, dev, dt=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)


@pytest.fixture(scope="module")
def prob():
    # 64^3, 4,000 patterns, 25,680 rotations (level 8)
    cfg = S.Config("prop64", 64, 400, 1.5, 12, 4000, 3000, (0.5, 1.5), 4, 8, 1, seed=3)
    return S.make_problem(cfg, device="cuda")


@pytest.fixture(scope="module")
def dense():
    # the same particle, 12,000 patterns: 94 pattern tiles, each spanning ~1 %
    # of the rotations, few enough tiles per pattern tile to prune
    cfg = S.Config("prop64", 64, 400, 1.5, 12, 12000, 3000, (0.5, 1.5), 4, 8, 1, seed=3)
    return S.make_problem(cfg, device="cuda", pattern_seed=1)


def rel_l2(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_inputs_and_gradients_match_oracle(ctx, cuda, prob):
    net = E.Proposal(ctx, seed=11)
    imgs, mask = T(prob.images, cuda), T(prob.mask, cuda, torch.int32)
    net.set_data(imgs, mask, 64)
    X = net.inputs(0, 16)
    raw = PO.inputs(prob.images, prob.mask, 64)
    st = PO.input_stats(raw)
    np.testing.assert_allclose(net.stats(), st, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(X, PO.inputs(prob.images[:16], prob.mask, 64, net.stats()),
                               rtol=1e-5, atol=1e-5)
    rng = np.random.default_rng(0)
    q = rng.normal(size=(prob.images.shape[0], 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    quats = T(q, cuda)
    rows = np.array([3, 0, 7, 12, 5, 9, 1, 15], np.int32)
    loss, g = net.loss_grad(rows, quats)
    params = net.params().astype(np.float64)
    L, gw = PO.loss_and_grads(params, X[rows].astype(np.float64),
                              quats.cpu().numpy()[rows].astype(np.float64))
    assert abs(loss - L) <= 1e-5 * abs(L)
    lay, _ = PO.layout()
    for o, shape in lay:
        n = int(np.prod(shape))
        assert rel_l2(g[o:o + n], gw[o:o + n]) < 2e-4, (o, shape)
    net.close()


def bound_plan(ctx, prob, dev, diff=E.DIFF_TRUE_POISSON, rows=None):
    s, R = prob.cfg.side, prob.quats.shape[0]
    images = prob.images if rows is None else prob.images[rows]
    plan = E.Plan(ctx, s, images.shape[0], R, diff=diff, precision=E.PREC_MIXED,
                  insert_mode=E.INSERT_DETERMINISTIC)
    inputs = (T(images, dev), T(prob.mask, dev, torch.int32), T(prob.x, dev), T(prob.y, dev),
              T(prob.z, dev), T(prob.quats, dev), T(prob.weights, dev))
    plan.bind(*inputs)
    plan._inputs = inputs
    return plan


def true_model(ctx, prob, dev):
    m = T(prob.true_model, dev)
    ctx.normalize_model(prob.cfg.side, m)
    return m


def test_best_quaternions_is_the_argmax(ctx, cuda, prob):
    R, N = prob.quats.shape[0], prob.images.shape[0]
    plan = bound_plan(ctx, prob, cuda)
    m = true_model(ctx, prob, cuda)
    w = torch.empty_like(m)
    plan.iterate(m, w, 0.1)
    r_ptr, _, _ = plan.results()
    ctx.sync()
    P = ctx.copy_real_to_host(r_ptr, R * N).reshape(R, N)
    out = torch.empty((N, 4), device=cuda)
    plan.best_quaternions(out)
    np.testing.assert_array_equal(out.cpu().numpy(), prob.quats[P.argmax(0)])
    plan.close()


def seeded_vs_full(ctx, prob, dev, proposals, fraction=0.0005):
    full = bound_plan(ctx, prob, dev)
    pr = bound_plan(ctx, prob, dev)
    pr.set_pruning(True, min_mass=0.999, dilate=1.0)
    pr.set_proposals(proposals, fraction)
    seeded = pr.prune_info()["active_fraction"]
    m0 = true_model(ctx, prob, dev)
    mf, mp = m0.clone(), m0.clone()
    w = torch.empty_like(m0)
    sf = full.iterate(mf, w, 0.1)
    sp = pr.iterate(mp, w, 0.1)
    info = pr.prune_info()
    full.close()
    pr.close()
    info["seeded_active_fraction"] = seeded
    return mf.cpu().numpy(), mp.cpu().numpy(), sf, sp, info


def with_mates(q):
    return np.stack([q, PO.friedel_mate(q)], 1).astype(np.float32)


def test_true_orientations_seed_a_pruned_iteration(ctx, cuda, dense):
    props = T(with_mates(dense.true_quats), cuda)
    mf, mp, sf, sp, info = seeded_vs_full(ctx, dense, cuda, props)
    print(f"\ntrue orientations: {info}")
    assert info["pruned"] == 1 and info["fallback"] == 0
    assert info["seeded_active_fraction"] < 1.0
    assert rel_l2(mp, mf) < 1e-4
    assert abs(sp.total_loglik - sf.total_loglik) <= 1e-5 * abs(sf.total_loglik)


def test_random_proposals_fall_back_to_the_full_scan(ctx, cuda, dense):
    rng = np.random.default_rng(5)
    q = rng.normal(size=(dense.images.shape[0], 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    q = np.where(q[:, :1] < 0, -q, q)
    mf, mp, sf, sp, info = seeded_vs_full(ctx, dense, cuda, T(with_mates(q), cuda))
    print(f"\nrandom proposals: {info}")
    assert info["pruned"] == 1 and info["fallback"] == 1
    assert rel_l2(mp, mf) < 1e-6


def angle_to_label(pred, label):
    """Rotation angle (degrees) from the label to the nearer of the
    prediction and its mate."""
    c = np.maximum(np.abs((pred[:, 0] * label).sum(1)), np.abs((pred[:, 1] * label).sum(1)))
    return np.degrees(2 * np.arccos(np.clip(c, -1, 1)))


def test_training_on_emc_labels(ctx, cuda, prob):
    N = prob.images.shape[0]
    plan = bound_plan(ctx, prob, cuda)
    m = true_model(ctx, prob, cuda)
    w = torch.empty_like(m)
    plan.iterate(m, w, 0.1)
    labels = torch.empty((N, 4), device=cuda)
    plan.best_quaternions(labels)
    plan.close()
    net = E.Proposal(ctx, seed=2)
    net.set_data(T(prob.images, cuda), T(prob.mask, cuda, torch.int32), 64)
    train, held = np.arange(0, 3500), np.arange(3500, N)
    pred0 = net.predict(torch.empty((N, 2, 4), device=cuda)).cpu().numpy()
    losses = net.train(labels, rows=train, epochs=40, batch=128, lr=1e-3, seed=1)
    pred = net.predict(torch.empty((N, 2, 4), device=cuda)).cpu().numpy()
    lab = labels.cpu().numpy()
    a0 = angle_to_label(pred0[held], lab[held])
    a1 = angle_to_label(pred[held], lab[held])
    print(f"\nproposal: loss {losses[0]:.4f} -> {losses[-1]:.4f}; held-out median angle "
          f"{np.median(a0):.1f} -> {np.median(a1):.1f} deg; within 41.8 deg "
          f"{(a0 < 41.8).mean():.3f} -> {(a1 < 41.8).mean():.3f}; train median "
          f"{np.median(angle_to_label(pred[train], lab[train])):.1f} deg")
    assert losses[-1] < 0.5 * losses[0]
    assert np.median(a1) < 0.5 * np.median(a0)
    # the 2 % ball (41.8 degrees) around the prediction or its mate holds the
    # label for far more held-out patterns than for the untrained network
    assert (a1 < 41.8).mean() > 4 * max((a0 < 41.8).mean(), 0.02)
    net.close()
