"""Accuracy at the low-count stress configuration's geometry against the FP64
oracle, and deterministic insertion bit-identical across runs.

128^3 model, all 10,860 rotations (n = 6), 128x128 detector with half of it
masked (seeded panel gaps plus the beamstop), ~80 photons per pattern, scales
U(0.2, 2.0); 2,000 of the 50,000 patterns so that the FP64 oracle finishes in
about a minute (a pattern's E-step does not depend on the others).  At 80
photons most counts are 0 or 1.  Two regimes: the schedule's first sigma
(0.4) from the random start, where responsibilities are broad, and two
iterations at its final sigma (0.12) from the true particle, where they are
peaked around each pattern's orientation.  (At sigma 0.12 from a model one
iteration old -- nearly isotropic, so the likelihood is almost flat across
rotations -- the responsibilities go to whichever rotation is marginally
best: there the plain FP32 path's model already differs from FP64 by 0.9 %,
a measure of that chaos rather than of precision.)

At sigma 0.12 with 2,000 peaked patterns most of the 10,860 rotations get
responsibilities at underflow level, and the voxels only those reach hold
values below 1e-6: 247,209 of the FP64 oracle's 363,359 positive voxels, of
which FP32 arithmetic (the reference's own) keeps about half and the FP16
M-step operand about a sixth, the rest rounding to exactly 0.  The model's
normalisation divides by the mean over positive voxels, so their count sets a
global scale (0.65 for FP32, 0.42 for the tensor path against FP64).  With
per-pattern scaling the likelihood does not depend on the model's scale, and
the log-likelihoods agree; the model is compared up to that scale, weighted
by the FP64 weight grid (the voxels the data determine).  Targets: weighted
scale-free model error within 1e-3 and total log-likelihood within 1e-4
relative of FP64."""
import dataclasses

import numpy as np
import pytest
import torch

import emc_gb300 as E
from emc_gb300 import synthetic as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu

# (sigma, start from the true particle)
STEPS = ((0.4, False), (0.12, True), (0.12, False))


@pytest.fixture(scope="module")
def prob():
    cfg = dataclasses.replace(S.CONFIGS["lowcount"], n_images=2000, name="lowcount-2000")
    return S.make_problem(cfg, device="cuda")


def true_start(prob):
    m = prob.true_model.astype(np.float64)
    return (m / m[m > 0].mean()).astype(np.float32)


def oracle_step(prob, m, sigma):
    w = O.fused_iteration_fp64(m.astype(np.float32), prob.images, prob.mask, prob.x, prob.y,
                               prob.z, prob.quats, prob.weights, sigma, prob.cfg.side)
    return w["model"], w["weight"], w["total_loglik"]


def T(a, dev, dt=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)


def make_plan(ctx, prob, dev, precision, insert=E.INSERT_ATOMIC):
    s, R, N = prob.cfg.side, prob.quats.shape[0], prob.images.shape[0]
    plan = E.Plan(ctx, s, N, R, precision=precision, insert_mode=insert)
    plan.bind(T(prob.images, dev), T(prob.mask, dev, torch.int32), T(prob.x, dev), T(prob.y, dev),
              T(prob.z, dev), T(prob.quats, dev), T(prob.weights, dev))
    return plan


@pytest.mark.parametrize("precision", [E.PREC_FP32, E.PREC_MIXED], ids=["fp32", "mixed"])
def test_lowcount_geometry_accuracy(ctx, cuda, prob, precision):
    """Each iteration against the FP64 oracle run from the same input model."""
    assert prob.mask.sum() < 0.55 * np.pi * 64 ** 2
    plan = make_plan(ctx, prob, cuda, precision)
    m = T(prob.init_model, cuda)
    w = torch.empty_like(m)
    for it, (sigma, restart) in enumerate(STEPS):
        if restart:
            m.copy_(T(true_start(prob), cuda))
        want, wt, want_ll = oracle_step(prob, m.cpu().numpy(), sigma)
        st = plan.iterate(m, w, sigma)
        got = m.cpu().numpy().astype(np.float64)
        rel = np.linalg.norm(got - want) / np.linalg.norm(want)
        wt = np.maximum(wt, 0.0)
        wc = (wt * got * want).sum() / (wt * want ** 2).sum()
        wrel = np.sqrt((wt * (got - wc * want) ** 2).sum() / (wt * (wc * want) ** 2).sum())
        ll_rel = abs(st.total_loglik - want_ll) / abs(want_ll)
        pos = want > 0
        print(f"lowcount precision {precision} step {it} sigma {sigma}: weighted scale-free "
              f"model rel L2 {wrel:.3e} (plain {rel:.3e}, scale {wc:.4f}), LL rel {ll_rel:.3e}; "
              f"positive voxels {int((got > 0).sum())} vs {int(pos.sum())} (FP64), below 1e-6 "
              f"{int(((got > 0) & (got < 1e-6)).sum())} vs {int((pos & (want < 1e-6)).sum())}")
        assert wrel < 1e-3
        assert ll_rel < 1e-4
    plan.close()


def test_lowcount_deterministic_insertion_bit_identical(ctx, cuda, prob):
    outs = []
    for _ in range(2):
        plan = make_plan(ctx, prob, cuda, E.PREC_MIXED, E.INSERT_DETERMINISTIC)
        m = T(prob.init_model, cuda)
        w = torch.empty_like(m)
        for sigma, restart in STEPS:
            if restart:
                m.copy_(T(true_start(prob), cuda))
            plan.iterate(m, w, sigma)
        outs.append((m.cpu().numpy(), w.cpu().numpy()))
        plan.close()
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])
