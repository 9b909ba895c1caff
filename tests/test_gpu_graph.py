"""The iteration's asynchronous and CUDA-graph forms against emc_iterate.

emc_iterate_async + emc_plan_wait and emc_plan_capture + emc_plan_replay run
the same kernels as emc_iterate; with deterministic insertion every result is
bit-identical, for both arithmetic paths, across changes of sigma between
replays."""
import numpy as np
import pytest
import torch

import emc_gb300 as E
from emc_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def prob():
    return S.make_problem(S.tiny(side=32, n_images=300, rot_n=2, photons=3000, n_atoms=120,
                                 radius=7.0))


def bound_plan(ctx, prob, dev, **kw):
    T = lambda a, dt=torch.float32: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    s, R, N = prob.cfg.side, prob.quats.shape[0], prob.images.shape[0]
    plan = E.Plan(ctx, s, N, R, insert_mode=E.INSERT_DETERMINISTIC, **kw)
    inputs = (T(prob.images), T(prob.mask, torch.int32), T(prob.x), T(prob.y), T(prob.z),
              T(prob.quats), T(prob.weights))
    plan.bind(*inputs)
    plan._inputs = inputs
    return plan, T(prob.init_model)


SIGMAS = (0.4, 0.31, 0.25)
KINDS = [dict(precision=E.PREC_FP32), dict(precision=E.PREC_MIXED),
         dict(precision=E.PREC_MIXED, diff=E.DIFF_TRUE_POISSON),
         dict(precision=E.PREC_FP32, blur_sigma=1.0)]


def kind_id(k):
    return "-".join(f"{a}{b}" for a, b in k.items())


@pytest.mark.parametrize("kw", KINDS, ids=kind_id)
def test_graph_replay_matches_iterate(ctx, cuda, prob, kw):
    plan, m_direct = bound_plan(ctx, prob, cuda, **kw)
    w_direct = torch.empty_like(m_direct)
    direct = []
    for sg in SIGMAS:
        st = plan.iterate(m_direct, w_direct, sg)
        direct.append((m_direct.cpu().numpy().copy(), w_direct.cpu().numpy().copy(),
                       st.total_loglik, st.captured_mass))
    m = torch.as_tensor(np.ascontiguousarray(prob.init_model), device=cuda)
    w = torch.empty_like(m)
    plan.capture(m, w)
    # capturing enqueues nothing: the buffers still hold the start model
    assert np.array_equal(m.cpu().numpy(), prob.init_model.astype(np.float32))
    for sg, (dm, dw, ll, mass) in zip(SIGMAS, direct):
        plan.replay(sg)
        st = plan.wait()
        assert np.array_equal(m.cpu().numpy(), dm)
        assert np.array_equal(w.cpu().numpy(), dw)
        assert st.total_loglik == ll
        assert st.captured_mass == mass
    plan.close()


def test_async_then_wait_matches_iterate(ctx, cuda, prob):
    plan, m1 = bound_plan(ctx, prob, cuda, precision=E.PREC_MIXED)
    w1 = torch.empty_like(m1)
    st1 = plan.iterate(m1, w1, 0.3)
    m2 = torch.as_tensor(np.ascontiguousarray(prob.init_model), device=cuda)
    w2 = torch.empty_like(m2)
    plan.iterate_async(m2, w2, 0.3)
    st2 = plan.wait()
    assert np.array_equal(m1.cpu().numpy(), m2.cpu().numpy())
    assert st1.total_loglik == st2.total_loglik
    # several queued iterations, one wait
    for sg in SIGMAS:
        plan.iterate_async(m2, w2, sg)
    st3 = plan.wait()
    assert np.isfinite(st3.total_loglik)
    plan.close()


def test_replay_without_capture_is_an_error(ctx, cuda, prob):
    plan, _ = bound_plan(ctx, prob, cuda, precision=E.PREC_FP32)
    with pytest.raises(E.EmcError):
        plan.replay(0.3)
    with pytest.raises(E.EmcError):
        plan.iterate_async(None, None, 0.3)
    plan.close()


def test_batch_matches_each_plan(ctx, cuda):
    """Three uneven problems in one graph launch: every model, weight and
    log-likelihood equals that problem's own direct iteration."""
    probs = [S.make_problem(S.tiny(side=s, n_images=n, rot_n=r, seed=k))
             for k, (s, n, r) in enumerate([(16, 70, 1), (24, 200, 2), (32, 130, 2)])]
    ctxs = [E.Context(0) for _ in probs]
    kinds = [E.PREC_FP32, E.PREC_MIXED, E.PREC_MIXED]
    direct, plans, models, weights = [], [], [], []
    for c, p, prec in zip(ctxs, probs, kinds):
        plan, m = bound_plan(c, p, cuda, precision=prec)
        w = torch.empty_like(m)
        st = plan.iterate(m, w, 0.35)
        direct.append((m.cpu().numpy(), w.cpu().numpy(), st.total_loglik))
        m2 = torch.as_tensor(np.ascontiguousarray(p.init_model), device=cuda)
        plans.append(plan)
        models.append(m2)
        weights.append(torch.empty_like(m2))
    batch = E.Batch(plans, models, weights)
    batch.run([0.35] * 3)
    stats = batch.wait()
    for (dm, dw, ll), m, w, st in zip(direct, models, weights, stats):
        assert np.array_equal(m.cpu().numpy(), dm)
        assert np.array_equal(w.cpu().numpy(), dw)
        assert st.total_loglik == ll
    batch.close()
    for plan, c in zip(plans, ctxs):
        plan.close()
        c.close()
