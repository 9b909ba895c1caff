"""Parity of the fused iteration (emc_plan_* / emc_iterate) against the FP64
oracle of its semantics, plus its properties at larger sizes.

Tolerances (FP32 path vs FP64): model relative L2 1e-4, total log-likelihood
relative 1e-5, responsibilities absolute 1e-4, scaling relative 1e-5."""
import numpy as np
import pytest
import torch

import emc_gb300 as E
from emc_gb300 import synthetic as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def T(a, dev, dt=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)


def run_plan(ctx, prob, dev, model=None, sigma=0.3, options=None, **kw):
    s, R, N = prob.cfg.side, prob.quats.shape[0], prob.images.shape[0]
    plan = E.Plan(ctx, s, N, R, **kw)
    for opt, val in (options or {}).items():
        plan.set_option(opt, val)
    plan.bind(T(prob.images, dev), T(prob.mask, dev, torch.int32), T(prob.x, dev), T(prob.y, dev),
              T(prob.z, dev), T(prob.quats, dev), T(prob.weights, dev))
    m = T(prob.init_model if model is None else model, dev)
    w = torch.empty_like(m)
    st = plan.iterate(m, w, sigma)
    r_ptr, s_ptr, _ = plan.results()
    resp = ctx.copy_real_to_host(r_ptr, R * N).reshape(R, N)
    phi = ctx.copy_real_to_host(s_ptr, R * N).reshape(R, N)
    out = dict(model=m.cpu().numpy().astype(np.float64), weight=w.cpu().numpy().astype(np.float64),
               respons=resp.astype(np.float64), phi=phi, stats=st)
    plan.close()
    return out


def rel_l2(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


# (plan keywords, well-conditioned): the true-Poisson likelihood and the
# known-intensity scaling give near one-hot responsibilities on this problem,
# where FP32 rounding may move mass between neighbouring rotations; those
# cases are checked stage by stage (log-likelihood, scaling, and the M-step
# from the kernel's own responsibilities) instead of end to end.
CASES = [
    (dict(diff=E.DIFF_POISSON, interp=E.INTERP_NEAREST), True),
    (dict(diff=E.DIFF_POISSON, interp=E.INTERP_TRILINEAR), True),
    (dict(diff=E.DIFF_POISSON, interp=E.INTERP_NEAREST, normalize_images=1), True),
    (dict(diff=E.DIFF_POISSON, interp=E.INTERP_NEAREST, known_intensity=1), False),
    (dict(diff=E.DIFF_TRUE_POISSON, interp=E.INTERP_NEAREST), False),
    (dict(diff=E.DIFF_TRUE_POISSON, interp=E.INTERP_TRILINEAR), False),
    (dict(diff=E.DIFF_POISSON, interp=E.INTERP_NEAREST, blur_sigma=1.0), True),
    (dict(diff=E.DIFF_POISSON, interp=E.INTERP_NEAREST, insert_mode=E.INSERT_DETERMINISTIC), True),
]
MIXED_CASES = [
    (dict(interp=E.INTERP_NEAREST), True),
    (dict(interp=E.INTERP_TRILINEAR), True),
    (dict(interp=E.INTERP_NEAREST, normalize_images=1), True),
    (dict(interp=E.INTERP_NEAREST, known_intensity=1), False),
    (dict(interp=E.INTERP_NEAREST, insert_mode=E.INSERT_DETERMINISTIC), True),
    (dict(diff=E.DIFF_TRUE_POISSON, interp=E.INTERP_NEAREST), False),
    (dict(diff=E.DIFF_TRUE_POISSON, interp=E.INTERP_TRILINEAR), False),
    (dict(diff=E.DIFF_TRUE_POISSON, interp=E.INTERP_NEAREST, known_intensity=1), False),
    (dict(diff=E.DIFF_TRUE_POISSON, interp=E.INTERP_NEAREST, normalize_images=1), False),
    # warp-aggregated insertion atomics
    (dict(interp=E.INTERP_NEAREST, options={E.Plan.OPT_MSTEP_AGGREGATE: 1}), True),
    # FP16 hi-only rotation-side factors and M-step operand
    (dict(interp=E.INTERP_NEAREST, options={E.Plan.OPT_ESTEP_GHLO: 0, E.Plan.OPT_MSTEP_QLO: 0}),
     True),
    # every factor hi + lo
    (dict(interp=E.INTERP_NEAREST, options={E.Plan.OPT_ESTEP_GHLO: 3, E.Plan.OPT_MSTEP_QLO: 1}),
     True),
    # G lo on every pixel block (no count tail dropped)
    (dict(interp=E.INTERP_NEAREST, options={E.Plan.OPT_GLO_TAIL: 0}), True),
]
# tolerances: (log-likelihood rel, scaling rel, model rel L2, respons abs)
TOL = {E.PREC_FP32: (1e-5, 1e-5, 1e-4, 1e-4), E.PREC_MIXED: (2e-5, 5e-4, 5e-4, 1e-3)}


@pytest.fixture(scope="module")
def prob():
    # ragged sizes: N and P_eff not multiples of the 128 tiles
    return S.make_problem(S.tiny(side=32, n_images=300, rot_n=2, photons=3000, n_atoms=120,
                                 radius=7.0))


def check_against_oracle(ctx, cuda, prob, kw, wellcond, precision):
    sigma = 0.3
    tl, tphi, tm, tr = TOL[precision]
    s = prob.cfg.side
    got = run_plan(ctx, prob, cuda, sigma=sigma, precision=precision, **kw)
    diff = kw.get("diff", E.DIFF_POISSON)
    norm = bool(kw.get("normalize_images", 0))
    want = O.fused_iteration_fp64(prob.init_model, prob.images, prob.mask, prob.x, prob.y, prob.z,
                                  prob.quats, prob.weights, sigma, s, diff=diff,
                                  interp=kw["interp"],
                                  known_intensity=bool(kw.get("known_intensity", 0)),
                                  normalize_images=norm, blur_sigma=kw.get("blur_sigma", 0.0))
    st = got["stats"]
    # E-step + normaliser
    assert abs(st.total_loglik - want["total_loglik"]) <= tl * abs(want["total_loglik"])
    np.testing.assert_allclose(got["phi"], want["phi"], rtol=tphi)
    np.testing.assert_allclose(got["respons"].sum(0), 1.0, atol=1e-4)
    assert abs(st.captured_mass - 1.0) < 1e-5
    # M-step from the kernel's own responsibilities and scaling
    K = O.compacted_counts(prob.images, prob.mask, s, norm)
    pm = prob.mask == 1
    m = O.mstep_fp64(got["respons"], got["phi"], K, prob.x[pm], prob.y[pm], prob.z[pm],
                     prob.quats, s, kw["interp"], kw.get("blur_sigma", 0.0))
    assert rel_l2(got["weight"], m["weight"]) < tm
    if wellcond:
        assert rel_l2(got["model"], m["model"]) < tm
        assert abs(st.model_mean_before - m["mean_before"]) <= tm * m["mean_before"]
    elif kw.get("blur_sigma", 0.0) == 0.0:
        # one-hot responsibilities: voxels reached only by underflowing
        # contributions are "positive" in FP64 and exactly 0 in FP32, which
        # moves the mean-over-positive-voxels normalisation; compare the
        # un-normalised model U/T where the weight is significant
        sel = m["weight"] > 1e-6 * m["weight"].max()
        a = got["model"][sel] * st.model_mean_before
        b = m["model"][sel] * m["mean_before"]
        assert rel_l2(a, b) < tm
    if wellcond:  # end to end
        assert np.abs(got["respons"] - want["respons"]).max() < tr
        assert rel_l2(got["model"], want["model"]) < 2 * tm
        assert rel_l2(got["weight"], want["weight"]) < 2 * tm


def case_id(c):
    names = {E.Plan.OPT_MSTEP_AGGREGATE: "aggregate", E.Plan.OPT_ESTEP_GHLO: "ghlo",
             E.Plan.OPT_MSTEP_QLO: "qlo", E.Plan.OPT_GLO_TAIL: "glotail"}
    return "-".join(f"{a}{b}" if a != "options" else
                    "-".join(f"{names[o]}{v}" for o, v in b.items()) for a, b in c[0].items())


@pytest.mark.parametrize("case", CASES, ids=case_id)
def test_fp32_iteration_matches_fp64_oracle(ctx, cuda, prob, case):
    check_against_oracle(ctx, cuda, prob, case[0], case[1], E.PREC_FP32)


@pytest.mark.parametrize("case", MIXED_CASES, ids=case_id)
def test_mixed_iteration_matches_fp64_oracle(ctx, cuda, prob, case):
    """Tensor-core path: FP16 hi+lo operands, FP32 accumulation."""
    check_against_oracle(ctx, cuda, prob, case[0], case[1], E.PREC_MIXED)


@pytest.mark.parametrize("n,k", [(128, 96), (256, 192)])
def test_tc_gemm_building_blocks(ctx, cuda, n, k):
    """TMA + descriptors + tcgen05.mma + TMEM loads for the E-step (n=128)
    and M-step (n=256) tile shapes, against an FP32 matmul."""
    import ctypes
    g = torch.Generator(device="cpu").manual_seed(n + k)
    A = (torch.randint(-8, 9, (128, k), generator=g).float() / 4).half().to(cuda)
    B = (torch.randint(-8, 9, (n, k), generator=g).float() / 8).half().to(cuda)
    D = torch.zeros((128, n), device=cuda)
    lib = E._lib.load()
    rc = lib.emc_tc_gemm_selftest(ctx.handle, A.data_ptr(), B.data_ptr(), D.data_ptr(), n, k)
    assert rc == 0, lib.emc_last_error(ctx.handle)
    ref = A.float() @ B.float().T
    torch.cuda.synchronize()
    assert torch.equal(D, ref), (D - ref).abs().max().item()


def test_mixed_rejects_non_integer_counts(ctx, cuda, prob):
    p = S.Problem(**{**prob.__dict__})
    p.images = prob.images + 0.5
    with pytest.raises(E.EmcError, match="UNSUPPORTED"):
        run_plan(ctx, p, cuda, precision=E.PREC_MIXED)


@pytest.mark.parametrize("pair", [1, 0], ids=["pairs", "single"])
def test_glo_tail_bounds(ctx, cuda, prob, pair):
    """EMC_OPT_GLO_TAIL 1e6 (every block in the tail) drops the G lo term
    everywhere: bit-identical to gh_lo = 0.  0 keeps it on every block that
    holds a count; the default lies between and within the oracle bounds."""
    kw = dict(precision=E.PREC_MIXED, insert_mode=E.INSERT_DETERMINISTIC)
    base = {E.Plan.OPT_ESTEP_PAIR: pair}
    none = run_plan(ctx, prob, cuda, options={**base, E.Plan.OPT_GLO_TAIL: 1000000}, **kw)
    off = run_plan(ctx, prob, cuda, options={**base, E.Plan.OPT_ESTEP_GHLO: 0}, **kw)
    assert np.array_equal(none["model"], off["model"])
    assert none["stats"].total_loglik == off["stats"].total_loglik
    every = run_plan(ctx, prob, cuda, options={**base, E.Plan.OPT_GLO_TAIL: 0}, **kw)
    dflt = run_plan(ctx, prob, cuda, options=base, **kw)
    ll_e, ll_d = every["stats"].total_loglik, dflt["stats"].total_loglik
    assert abs(ll_d - ll_e) <= 1e-5 * abs(ll_e)
    assert rel_l2(dflt["model"], every["model"]) < 1e-4


def test_deterministic_insert_is_bit_identical(ctx, cuda, prob):
    for prec in (E.PREC_FP32, E.PREC_MIXED):
        a = run_plan(ctx, prob, cuda, insert_mode=E.INSERT_DETERMINISTIC, precision=prec)
        b = run_plan(ctx, prob, cuda, insert_mode=E.INSERT_DETERMINISTIC, precision=prec)
        assert np.array_equal(a["model"], b["model"]) and np.array_equal(a["weight"], b["weight"])
        c = run_plan(ctx, prob, cuda, insert_mode=E.INSERT_ATOMIC, precision=prec)
        assert rel_l2(a["model"], c["model"]) < 1e-5


def test_two_iterations_track_oracle(ctx, cuda, prob):
    s = prob.cfg.side
    m = prob.init_model.copy()
    want = prob.init_model.copy()
    for it in range(2):
        sigma = E.sigma_schedule(it, 0.4, 0.12, 25)
        got = run_plan(ctx, prob, cuda, model=m, sigma=sigma)
        w = O.fused_iteration_fp64(want, prob.images, prob.mask, prob.x, prob.y, prob.z,
                                   prob.quats, prob.weights, sigma, s)
        m = got["model"].astype(np.float32)
        want = w["model"].astype(np.float32)
        assert rel_l2(got["model"], w["model"]) < 2e-4


def test_zero_photon_pattern_gets_no_responsibility(ctx, cuda, prob):
    p = S.Problem(**{**prob.__dict__})
    p.images = prob.images.copy()
    p.images[7] = 0.0
    got = run_plan(ctx, p, cuda)
    assert (got["respons"][:, 7] == 0).all()
    assert abs(got["stats"].captured_mass - (p.images.shape[0] - 1) / p.images.shape[0]) < 1e-5
    assert got["stats"].bad_pairs >= p.quats.shape[0]


def test_bind_rejects_bad_inputs(ctx, cuda, prob):
    s, R, N = prob.cfg.side, prob.quats.shape[0], prob.images.shape[0]
    args = [T(prob.x, cuda), T(prob.y, cuda), T(prob.z, cuda), T(prob.quats, cuda),
            T(prob.weights, cuda)]
    bad = prob.images.copy()
    bad[3, np.nonzero(prob.mask)[0][10]] = np.nan  # a pixel the mask keeps
    plan = E.Plan(ctx, s, N, R)
    with pytest.raises(E.EmcError, match="NONFINITE"):
        plan.bind(T(bad, cuda), T(prob.mask, cuda, torch.int32), *args)
    m2 = prob.mask.copy()
    m2[0] = 2
    plan = E.Plan(ctx, s, N, R)
    with pytest.raises(E.EmcError, match="mask"):
        plan.bind(T(prob.images, cuda), T(m2, cuda, torch.int32), *args)
    plan = E.Plan(ctx, s, N, R)
    m = T(prob.init_model, cuda)
    with pytest.raises(E.EmcError, match="not bound"):
        plan.iterate(m, torch.empty_like(m), 0.3)
    with pytest.raises(E.EmcError):
        E.Plan(ctx, s, N, R, diff=E.DIFF_ABSOLUTE)


def test_properties_at_small_config(ctx, cuda):
    """The small benchmark configuration (64^3, 2,000 patterns, 3,240
    rotations): responsibilities normalise per pattern, the model has mean 1
    over its positive voxels, the weight sums to sum_r T_r x inserted pixels,
    and deterministic reruns are bit-identical."""
    prob = S.make_problem(S.CONFIGS["small"], device="cuda")
    s, R, N = prob.cfg.side, prob.quats.shape[0], prob.images.shape[0]
    a = run_plan(ctx, prob, cuda, sigma=0.4, insert_mode=E.INSERT_DETERMINISTIC)
    b = run_plan(ctx, prob, cuda, sigma=0.4, insert_mode=E.INSERT_DETERMINISTIC)
    assert np.array_equal(a["model"], b["model"])
    colsum = a["respons"].sum(0)
    np.testing.assert_allclose(colsum, 1.0, atol=2e-4)
    pos = a["model"][a["model"] > 0]
    assert abs(pos.mean() - 1.0) < 1e-5
    T_r = a["respons"].sum(1)
    vox = O.nearest_voxels(prob.quats, prob.x[prob.mask == 1], prob.y[prob.mask == 1],
                           prob.z[prob.mask == 1], s, 0)
    inserted = (vox >= 0).sum(1)
    assert abs(a["weight"].sum() - (T_r * inserted).sum()) <= 1e-4 * a["weight"].sum()
    assert abs(a["stats"].captured_mass - 1.0) < 1e-5


@pytest.fixture(scope="module")
def lowcount():
    # the low-count stress configuration's character at a size the FP64 oracle
    # finishes quickly: 80 photons per pattern, scales U(0.2, 2.0), half of the
    # detector masked by seeded panel gaps plus the beamstop
    cfg = S.Config("lowcount-tiny", 32, 120, 1.2, 7.0, 400, 80.0, (0.2, 2.0), 2, 2, 1,
                   masked_fraction=0.5)
    return S.make_problem(cfg)


@pytest.mark.parametrize("precision", [E.PREC_FP32, E.PREC_MIXED], ids=["fp32", "mixed"])
def test_lowcount_matches_oracle_and_reruns_bit_identical(ctx, cuda, lowcount, precision):
    assert lowcount.mask.sum() < 0.55 * (np.pi * 16 ** 2)
    check_against_oracle(ctx, cuda, lowcount, dict(interp=E.INTERP_NEAREST), False, precision)
    a = run_plan(ctx, lowcount, cuda, precision=precision, insert_mode=E.INSERT_DETERMINISTIC)
    b = run_plan(ctx, lowcount, cuda, precision=precision, insert_mode=E.INSERT_DETERMINISTIC)
    assert np.array_equal(a["model"], b["model"]) and np.array_equal(a["weight"], b["weight"])
    assert np.array_equal(a["respons"], b["respons"])


def test_qlo_switched_on_after_bind(ctx, cuda, prob):
    """The FP16 lo half of the M-step operand exists only once asked for; asking
    after bind allocates it and the iteration uses it."""
    s, R, N = prob.cfg.side, prob.quats.shape[0], prob.images.shape[0]
    plan = E.Plan(ctx, s, N, R, precision=E.PREC_MIXED, insert_mode=E.INSERT_DETERMINISTIC)
    plan.bind(T(prob.images, cuda), T(prob.mask, cuda, torch.int32), T(prob.x, cuda),
              T(prob.y, cuda), T(prob.z, cuda), T(prob.quats, cuda), T(prob.weights, cuda))
    before = plan.workspace_bytes
    plan.set_option(E.Plan.OPT_MSTEP_QLO, 1)
    assert plan.workspace_bytes > before
    m = T(prob.init_model, cuda)
    w = torch.empty_like(m)
    plan.iterate(m, w, 0.3)
    ref = run_plan(ctx, prob, cuda, precision=E.PREC_MIXED, insert_mode=E.INSERT_DETERMINISTIC,
                   options={E.Plan.OPT_MSTEP_QLO: 1})
    assert np.array_equal(m.cpu().numpy().astype(np.float64), ref["model"])
    plan.close()


def test_counts_above_2048_rounded_to_fp16(ctx, cuda, prob):
    """Bright patterns: counts up to ~30,000.  Without EMC_OPT_COUNTS_ROUND the
    tensor path refuses them; with it, it matches the FP64 oracle run on the
    counts rounded to FP16 (the K^2 operand scale follows the largest count)."""
    p = S.Problem(**{**prob.__dict__})
    p.images = (prob.images * 37.0).astype(np.float32)
    assert p.images.max() > 4096
    with pytest.raises(E.EmcError, match="UNSUPPORTED"):
        run_plan(ctx, p, cuda, precision=E.PREC_MIXED)
    got = run_plan(ctx, p, cuda, precision=E.PREC_MIXED, options={E.Plan.OPT_COUNTS_ROUND: 1})
    rounded = p.images.astype(np.float16).astype(np.float32)
    s = p.cfg.side
    want = O.fused_iteration_fp64(p.init_model, rounded, p.mask, p.x, p.y, p.z, p.quats,
                                  p.weights, 0.3, s)
    tl, tphi, tm, tr = TOL[E.PREC_MIXED]
    assert abs(got["stats"].total_loglik - want["total_loglik"]) <= tl * abs(want["total_loglik"])
    np.testing.assert_allclose(got["phi"], want["phi"], rtol=tphi)
    assert rel_l2(got["model"], want["model"]) < 2 * tm
