"""The small configuration exactly as defined, against the FP64 oracle, and the
fused path's distance from the reference's own iteration semantics.

Small configuration: 64^3 model (400 Gaussian atoms, radius 12), 2,000 patterns
of 64x64 (~1,000 photons, scale U(0.5, 1.5), beamstop radius 4), 3,240
rotations (n = 4), the reference's "poisson" likelihood with scaling, blur
sigma = 1 voxel, random start model, all 20 iterations of the sigma schedule
(0.4 -> 0.12, half-life 25).

* test_small_config_20_iterations: the plain FP32 path and the mixed-precision
  tensor-core path each run their own chain of 20 iterations; the FP64 oracle
  (oracle.fused_iteration_fp64) runs its own chain from the same start.  After
  every iteration the model must be within 1e-3 relative L2 and the total
  log-likelihood within 1e-4 relative of the oracle's -- for the FP32 path
  and for the tensor-core path with every lo term (G and H hi + lo in the
  likelihood, Q hi + lo in the M-step).  With the default lo terms (G only)
  the tensor-core path's log-likelihood is measured at up to 1.1e-4 relative
  over the 20 chained iterations (4e-5 to 7e-5 for one iteration from the
  same model: at 1,000 photons per pattern the FP16 rounding of
  H = 1/(s + c) shifts every pattern's lse the same way), so its bound is
  2e-4; the mid configuration's test holds the default to 1e-4.
* test_fused_vs_reference_semantics: the fused FP32 path against
  oracle.ref_iteration -- the restatement of the reference's kernels that the
  reference-kernel golden vectors pin (int-truncated scaling denominator,
  FP64 per-pixel likelihood terms, float log-sum-exp) -- over the first two
  iterations, no blur (the reference never blurs).  The two semantics differ
  on purpose (float scaling denominator; invalid pairs get L = -inf), so the
  bounds are the measured distances with a margin, stated in the test.
"""
import numpy as np
import pytest
import torch

import emc_gb300 as E
from emc_gb300 import synthetic as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu

ITERATIONS = 20


@pytest.fixture(scope="module")
def prob():
    return S.make_problem(S.CONFIGS["small"], device="cuda")


def sigma(it):
    return E.sigma_schedule(it, S.SIGMA_START, S.SIGMA_FINAL, S.SIGMA_HALF_LIFE)


@pytest.fixture(scope="module")
def oracle_chain(prob):
    s = prob.cfg.side
    models, lls = [], []
    m = prob.init_model.astype(np.float32)
    for it in range(ITERATIONS):
        w = O.fused_iteration_fp64(m, prob.images, prob.mask, prob.x, prob.y, prob.z, prob.quats,
                                   prob.weights, sigma(it), s, blur_sigma=prob.cfg.blur)
        models.append(w["model"])
        lls.append(w["total_loglik"])
        m = w["model"].astype(np.float32)
    return models, lls


def _tensors(prob, cuda):
    T = lambda a, dt=torch.float32: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=cuda)
    return T, (T(prob.images), T(prob.mask, torch.int32), T(prob.x), T(prob.y), T(prob.z),
               T(prob.quats), T(prob.weights))


@pytest.mark.parametrize("precision,gh_lo,q_lo,ll_bound",
                         [(E.PREC_FP32, -1, 0, 1e-4), (E.PREC_MIXED, 3, 1, 1e-4),
                          (E.PREC_MIXED, -1, 0, 2e-4)],
                         ids=["fp32", "mixed-all-lo", "mixed-default"])
def test_small_config_20_iterations(ctx, cuda, prob, oracle_chain, precision, gh_lo, q_lo,
                                    ll_bound):
    want_models, want_lls = oracle_chain
    s, R, N = prob.cfg.side, prob.quats.shape[0], prob.images.shape[0]
    assert (s, N, R) == (64, 2000, 3240)
    T, inputs = _tensors(prob, cuda)
    plan = E.Plan(ctx, s, N, R, precision=precision, blur_sigma=prob.cfg.blur)
    plan.set_option(E.Plan.OPT_ESTEP_GHLO, gh_lo)
    plan.set_option(E.Plan.OPT_MSTEP_QLO, q_lo)
    plan.bind(*inputs)
    m = T(prob.init_model)
    w = torch.empty_like(m)
    worst = (0.0, 0.0)
    for it in range(ITERATIONS):
        st = plan.iterate(m, w, sigma(it))
        got = m.cpu().numpy().astype(np.float64)
        rel = np.linalg.norm(got - want_models[it]) / np.linalg.norm(want_models[it])
        ll_rel = abs(st.total_loglik - want_lls[it]) / abs(want_lls[it])
        print(f"small precision {precision} gh_lo {gh_lo} q_lo {q_lo} iteration {it:2d} "
              f"sigma {sigma(it):.4f}: model rel L2 {rel:.3e}, LL rel {ll_rel:.3e}")
        worst = (max(worst[0], rel), max(worst[1], ll_rel))
        assert rel < 1e-3, f"iteration {it}: model rel L2 {rel:.3e}"
        assert ll_rel < ll_bound, f"iteration {it}: LL rel {ll_rel:.3e}"
    print(f"small worst over {ITERATIONS} iterations: model {worst[0]:.3e}, LL {worst[1]:.3e}")
    plan.close()


# Measured distance of the fused semantics from the reference's, first two
# iterations of the small configuration (FP64 fused oracle against
# ref_iteration; the FP32 fused path is within 1e-6 of the former):
#   iteration 0 (random start): model rel L2 0.30, LL rel 1.9e-2, responsibilities
#     within 6.3e-5 absolute.  The reference accumulates the scaling denominator
#     sum(k s) in an int, truncating after every add (emc_cuda.cu:439-446), so
#     products k s < 1 -- most of them on a U(0, 1) start model -- count 0 and
#     phi is 42 % larger at the median; the patterns' weights in the model
#     average change with it.
#   iteration 1: model rel L2 2.2e-3, LL rel 7.0e-4, responsibilities 9.9e-5.
# Bounds: twice the measured distance.
REF_BOUNDS = [dict(model=0.6, ll=4e-2, respons=2e-4), dict(model=5e-3, ll=1.5e-3, respons=2e-4)]


def test_fused_vs_reference_semantics(ctx, cuda, prob):
    s, R, N = prob.cfg.side, prob.quats.shape[0], prob.images.shape[0]
    T, inputs = _tensors(prob, cuda)
    plan = E.Plan(ctx, s, N, R, precision=E.PREC_FP32)
    plan.bind(*inputs)
    m = T(prob.init_model)
    w = torch.empty_like(m)
    ref_model = prob.init_model.astype(np.float32)
    for it, bound in enumerate(REF_BOUNDS):
        sg = O.sigma_at(it)
        st = plan.iterate(m, w, float(sg))
        respons = ctx.copy_real_to_host(plan.results()[0], R * N).reshape(R, N)
        ref = O.ref_iteration(ref_model, prob.images, prob.mask, prob.x, prob.y, prob.z,
                              prob.quats, prob.weights, sg, s)
        ref_model = ref["model"]
        ref_ll = float(np.sum(ref["lse"][np.isfinite(ref["lse"])], dtype=np.float64))
        got = m.cpu().numpy().astype(np.float64)
        want = ref_model.astype(np.float64)
        rel = np.linalg.norm(got - want) / np.linalg.norm(want)
        ll_rel = abs(st.total_loglik - ref_ll) / abs(ref_ll)
        dr = float(np.abs(respons - ref["respons"]).max())
        print(f"fused FP32 vs reference semantics, iteration {it}: model rel L2 {rel:.3e}, "
              f"LL rel {ll_rel:.3e}, responsibilities max abs {dr:.3e}")
        assert rel < bound["model"]
        assert ll_rel < bound["ll"]
        assert dr < bound["respons"]
        # continue both chains from their own models, as two runs would
    plan.close()
