"""The likelihood kernel's tile order (EMC_OPT_ESTEP_RASTER) and its
autotuner (emc_plan_autotune).

Every (pattern tile, rotation tile) CTA computes its tile independently, so
the order changes which operand panels share L2, never the numbers: with
deterministic insertion a whole iteration is bit-identical under every order,
for both likelihood kernels (the reference's Poisson form and counts x log
slice).  The autotuner picks one of its candidates and leaves the model
untouched."""
import numpy as np
import pytest
import torch

import emc_gb300 as E
from emc_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

ORDERS = (8, 2, 16, -8, -19, -76, 64, -4096)
CANDIDATES_MAX = 76


@pytest.fixture(scope="module")
def prob():
    # 2,000 patterns (16 tiles) x 3,240 rotations (26 tiles of 128, 13 of 256)
    return S.make_problem(S.tiny(side=48, n_images=2000, rot_n=4, photons=2500, n_atoms=150,
                                 radius=9.0))


def bound(ctx, prob, dev, **kw):
    T = lambda a, dt=torch.float32: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    s, R, N = prob.cfg.side, prob.quats.shape[0], prob.images.shape[0]
    plan = E.Plan(ctx, s, N, R, insert_mode=E.INSERT_DETERMINISTIC, **kw)
    inputs = (T(prob.images), T(prob.mask, torch.int32), T(prob.x), T(prob.y), T(prob.z),
              T(prob.quats), T(prob.weights))
    plan.bind(*inputs)
    plan._inputs = inputs
    return plan, T(prob.init_model)


@pytest.mark.parametrize("diff", [E.DIFF_POISSON, E.DIFF_TRUE_POISSON], ids=["poisson", "true"])
def test_every_order_gives_identical_iterations(ctx, cuda, prob, diff):
    plan, m0 = bound(ctx, prob, cuda, precision=E.PREC_MIXED, diff=diff)
    outs = []
    for g in ORDERS:
        plan.set_option(E.Plan.OPT_ESTEP_RASTER, g)
        m, w = m0.clone(), torch.empty_like(m0)
        st = plan.iterate(m, w, 0.3)
        st2 = plan.iterate(m, w, 0.25)
        outs.append((g, m.cpu().numpy(), w.cpu().numpy(), st.total_loglik, st2.total_loglik))
    g0, m_ref, w_ref, ll_ref, ll2_ref = outs[0]
    for g, m, w, ll, ll2 in outs[1:]:
        assert np.array_equal(m, m_ref), f"raster {g}"
        assert np.array_equal(w, w_ref), f"raster {g}"
        assert (ll, ll2) == (ll_ref, ll2_ref), f"raster {g}"
    plan.close()


@pytest.mark.parametrize("diff", [E.DIFF_POISSON, E.DIFF_TRUE_POISSON], ids=["poisson", "true"])
def test_autotune_picks_a_candidate(ctx, cuda, prob, diff):
    plan, m0 = bound(ctx, prob, cuda, precision=E.PREC_MIXED, diff=diff)
    m = m0.clone()
    raster, ms = plan.autotune(m, 0.3)
    assert raster != 0 and abs(raster) <= CANDIDATES_MAX and ms > 0.0
    assert torch.equal(m, m0)  # the model is only read
    # the tuned plan iterates like one with the default order and the tile
    # shape the tuner kept (CTA pairs or single CTAs)
    ref, _ = bound(ctx, prob, cuda, precision=E.PREC_MIXED, diff=diff)
    shape = plan.get_option(E.Plan.OPT_ESTEP_PAIR)
    assert shape in (0, 1)
    ref.set_option(E.Plan.OPT_ESTEP_PAIR, shape)
    m1, w1 = m0.clone(), torch.empty_like(m0)
    w = torch.empty_like(m0)
    st = plan.iterate(m, w, 0.3)
    st1 = ref.iterate(m1, w1, 0.3)
    assert torch.equal(m, m1) and torch.equal(w, w1)
    assert st.total_loglik == st1.total_loglik and st.bad_pairs == st1.bad_pairs == 0
    plan.close()
    ref.close()


def test_autotune_fp32_plan_and_bad_orders(ctx, cuda, prob):
    plan, m0 = bound(ctx, prob, cuda, precision=E.PREC_FP32)
    assert plan.autotune(m0, 0.3) == (0, 0.0)
    for bad in (0, 4097, -4097):
        with pytest.raises(E.EmcError):
            plan.set_option(E.Plan.OPT_ESTEP_RASTER, bad)
    plan.close()


def test_mstep_orders_give_identical_iterations(ctx, cuda, prob):
    """The M-step's tile order (EMC_OPT_MSTEP_RASTER) changes which CTA
    inserts which tile when, never the deterministic sums."""
    plan, m0 = bound(ctx, prob, cuda, precision=E.PREC_MIXED)
    outs = []
    for g in (8, 1, 3, -2, -64, 4096):
        plan.set_option(E.Plan.OPT_MSTEP_RASTER, g)
        m, w = m0.clone(), torch.empty_like(m0)
        plan.iterate(m, w, 0.3)
        outs.append((m.cpu().numpy(), w.cpu().numpy()))
    for m, w in outs[1:]:
        assert np.array_equal(m, outs[0][0]) and np.array_equal(w, outs[0][1])
    for bad in (0, 4097):
        with pytest.raises(E.EmcError):
            plan.set_option(E.Plan.OPT_MSTEP_RASTER, bad)
    plan.close()


def test_option_values_read_back(ctx, cuda, prob):
    """emc_plan_get_option returns what emc_plan_set_option set (and the
    defaults before)."""
    plan, _ = bound(ctx, prob, cuda, precision=E.PREC_MIXED)
    assert plan.get_option(E.Plan.OPT_ESTEP_PAIR) == 1
    assert plan.get_option(E.Plan.OPT_MSTEP_PAIR) == 1
    assert plan.get_option(E.Plan.OPT_GLO_TAIL) == 1000
    for opt, val in ((E.Plan.OPT_ESTEP_RASTER, -19), (E.Plan.OPT_MSTEP_RASTER, 8),
                     (E.Plan.OPT_ESTEP_PAIR, 0), (E.Plan.OPT_GLO_TAIL, 0),
                     (E.Plan.OPT_MSTEP_QLO, 1)):
        plan.set_option(opt, val)
        assert plan.get_option(opt) == val
    with pytest.raises(E.EmcError):
        plan.get_option(999)
    plan.close()
