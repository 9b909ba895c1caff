"""Accuracy at the mid configuration's geometry against the FP64 oracle.

128^3 model, all 25,680 rotations (n = 8), 128x128 detector with the 6-px
beamstop, ~5,000 photons per pattern; 2,000 of the 20,000 patterns so that the
FP64 oracle (numpy GEMMs on the host) finishes in about a minute.  The E-step of
a pattern does not depend on the other patterns, so the per-pattern log-sum-exp
and responsibilities are exactly those of the full problem; the model is that of
the 2,000-pattern problem.  Targets: final model within 1e-3 relative L2 and
total log-likelihood within 1e-4 relative of FP64, for the plain FP32 and the
mixed-precision (tensor-core) paths, over the first six iterations of the sigma
schedule (0.4 -> 0.12, half-life 25); each path and the oracle run their own
chain from the same random start."""
import dataclasses

import numpy as np
import pytest
import torch

import emc_gb300 as E
from emc_gb300 import synthetic as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu

ITERATIONS = 6


@pytest.fixture(scope="module")
def prob():
    cfg = dataclasses.replace(S.CONFIGS["mid"], n_images=2000, name="mid-2000")
    return S.make_problem(cfg, device="cuda")


@pytest.fixture(scope="module")
def oracle_run(prob):
    s = prob.cfg.side
    models, lls = [], []
    m = prob.init_model.astype(np.float32)
    for it in range(ITERATIONS):
        sigma = E.sigma_schedule(it, 0.4, 0.12, 25)
        w = O.fused_iteration_fp64(m, prob.images, prob.mask, prob.x, prob.y, prob.z, prob.quats,
                                   prob.weights, sigma, s)
        models.append(w["model"])
        lls.append(w["total_loglik"])
        m = w["model"].astype(np.float32)
    return models, lls


# mixed: the defaults (G hi + lo up to the pattern tile's 0.1 % count tail,
# H hi, Q hi); mixed-glo-all: G lo on every pixel block; mixed-hilo: every
# factor hi + lo; mixed-hi: every factor hi only (close to the log-likelihood
# target: the G lo term matters, the H and Q lo terms do not)
@pytest.mark.parametrize("precision,q_lo,gh_lo,tail",
                         [(E.PREC_FP32, 1, -1, 1000), (E.PREC_MIXED, 0, -1, 1000),
                          (E.PREC_MIXED, 0, -1, 0), (E.PREC_MIXED, 1, 3, 0),
                          (E.PREC_MIXED, 0, 0, 1000)],
                         ids=["fp32", "mixed", "mixed-glo-all", "mixed-hilo", "mixed-hi"])
def test_mid_geometry_accuracy(ctx, cuda, prob, oracle_run, precision, q_lo, gh_lo, tail):
    want_models, want_lls = oracle_run
    s, R, N = prob.cfg.side, prob.quats.shape[0], prob.images.shape[0]
    T = lambda a, dt=torch.float32: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=cuda)
    plan = E.Plan(ctx, s, N, R, precision=precision)
    plan.set_option(E.Plan.OPT_MSTEP_QLO, q_lo)
    plan.set_option(E.Plan.OPT_ESTEP_GHLO, gh_lo)
    plan.set_option(E.Plan.OPT_GLO_TAIL, tail)
    plan.bind(T(prob.images), T(prob.mask, torch.int32), T(prob.x), T(prob.y), T(prob.z),
              T(prob.quats), T(prob.weights))
    m = T(prob.init_model)
    w = torch.empty_like(m)
    for it in range(ITERATIONS):
        st = plan.iterate(m, w, E.sigma_schedule(it, 0.4, 0.12, 25))
        got = m.cpu().numpy().astype(np.float64)
        want = want_models[it]
        rel = np.linalg.norm(got - want) / np.linalg.norm(want)
        ll_rel = abs(st.total_loglik - want_lls[it]) / abs(want_lls[it])
        print(f"precision {precision} q_lo {q_lo} gh_lo {gh_lo} tail {tail} iteration {it}: "
              f"model rel L2 {rel:.3e}, LL rel {ll_rel:.3e}")
        assert rel < 1e-3
        assert ll_rel < 1e-4
    plan.close()
