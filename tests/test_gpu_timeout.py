"""The bounded-wait exit path of the tensor-core pipelines, made to run out.

EMC_OPT_DEBUG_SPIN caps every pipeline wait (TMA ring, MMA completion,
accumulator hand-over) at one poll, so the likelihood and M-step kernels give
up at once: emc_iterate must report EMC_ERR_TIMEOUT (the status word, not a
fault), the kernels must leave with no copy or MMA in flight (their exit
waits are not capped), and the next iteration on the same plan with the
default limit must equal, bit for bit, an iteration of a fresh plan from the
same model (deterministic insertion).  Nothing here faults or hangs a GPU:
every wait is bounded, and the failure is a status the host reads."""
import time

import numpy as np
import pytest
import torch

import emc_gb300 as E
from emc_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def prob():
    return S.make_problem(S.tiny(side=32, n_images=600, rot_n=3, photons=1500, seed=3))


@pytest.mark.parametrize("diff,pair", [(E.DIFF_POISSON, 1), (E.DIFF_POISSON, 0),
                                       (E.DIFF_TRUE_POISSON, 0)],
                         ids=["pairs", "single", "true-poisson"])
def test_timeout_is_reported_and_plan_recovers(ctx, cuda, prob, diff, pair):
    s, R, N = prob.cfg.side, prob.quats.shape[0], prob.images.shape[0]
    T = lambda a, dt=torch.float32: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=cuda)
    inputs = (T(prob.images), T(prob.mask, torch.int32), T(prob.x), T(prob.y), T(prob.z),
              T(prob.quats), T(prob.weights))

    def plan_for():
        p = E.Plan(ctx, s, N, R, diff=diff, precision=E.PREC_MIXED,
                   insert_mode=E.INSERT_DETERMINISTIC)
        p.set_option(E.Plan.OPT_ESTEP_PAIR, pair)
        p.bind(*inputs)
        return p

    sigma = 0.3
    fresh = plan_for()
    m_ref = T(prob.init_model)
    w_ref = torch.empty_like(m_ref)
    fresh.iterate(m_ref, w_ref, sigma)
    fresh.close()

    plan = plan_for()
    plan.set_option(E.Plan.OPT_DEBUG_SPIN, 1)
    m = T(prob.init_model)
    w = torch.empty_like(m)
    t0 = time.perf_counter()
    with pytest.raises(E.EmcError, match="EMC_ERR_TIMEOUT"):
        plan.iterate(m, w, sigma)
    assert time.perf_counter() - t0 < 60.0
    plan.set_option(E.Plan.OPT_DEBUG_SPIN, 0)
    m = T(prob.init_model)
    w = torch.empty_like(m)
    st = plan.iterate(m, w, sigma)
    assert np.isfinite(st.total_loglik)
    assert torch.equal(m, m_ref)
    assert torch.equal(w, w_ref)
    plan.close()
