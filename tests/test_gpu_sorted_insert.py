"""The sorted-voxel insertion (EMC_INSERT_SORTED): the M-step stores every
(rotation, pixel) value and a segmented reduction over the pairs sorted by
voxel adds them in a fixed order (the reference adds them with float atomics,
emc_atomic.cu:72-73).

* bit-identical models and weights from fresh plans, FP32 and mixed
  precision, nearest and trilinear insertion, and the same sums as the float
  atomics up to rounding;
* against the FP64 oracle of one iteration (model, weight);
* a re-bind with the same geometry keeps the voxel map, a re-bind with other
  rotations rebuilds it (bit-identical to a fresh plan on those rotations),
  and so does turning pruning on (which reorders the plan's rotations);
* the rotation split (emc_rank_mstep) with sorted insertion;
* pair codes that do not fit 32 bits are refused at bind."""
import numpy as np
import pytest
import torch

import emc_gb300 as E
from emc_gb300 import synthetic as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def T(a, dev, dt=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)


@pytest.fixture(scope="module")
def prob():
    return S.make_problem(S.tiny(side=32, n_images=300, rot_n=3, photons=3000, n_atoms=120,
                                 radius=7.0, seed=5))


def bind(plan, prob, dev, quats=None, weights=None):
    q = prob.quats if quats is None else quats
    w = prob.weights if weights is None else weights
    plan.bind(T(prob.images, dev), T(prob.mask, dev, torch.int32), T(prob.x, dev),
              T(prob.y, dev), T(prob.z, dev), T(q, dev), T(w, dev))


def iterate(plan, prob, dev, n_iter=1, sigma=0.3):
    m = T(prob.init_model, dev)
    w = torch.empty_like(m)
    st = None
    for _ in range(n_iter):
        st = plan.iterate(m, w, sigma)
    return m.cpu().numpy(), w.cpu().numpy(), st


def run(ctx, prob, dev, n_iter=1, quats=None, **kw):
    s, N = prob.cfg.side, prob.images.shape[0]
    R = (prob.quats if quats is None else quats).shape[0]
    plan = E.Plan(ctx, s, N, R, **kw)
    bind(plan, prob, dev, quats)
    out = iterate(plan, prob, dev, n_iter)
    plan.close()
    return out


def rel_l2(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


PARAMS = [(E.PREC_FP32, E.INTERP_NEAREST), (E.PREC_FP32, E.INTERP_TRILINEAR),
          (E.PREC_MIXED, E.INTERP_NEAREST), (E.PREC_MIXED, E.INTERP_TRILINEAR)]
IDS = ["fp32-nearest", "fp32-trilinear", "mixed-nearest", "mixed-trilinear"]


@pytest.mark.parametrize("precision,interp", PARAMS, ids=IDS)
def test_sorted_is_bit_identical_and_matches_atomics(ctx, cuda, prob, precision, interp):
    kw = dict(precision=precision, interp=interp)
    a = run(ctx, prob, cuda, n_iter=2, insert_mode=E.INSERT_SORTED, **kw)
    b = run(ctx, prob, cuda, n_iter=2, insert_mode=E.INSERT_SORTED, **kw)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert a[2].total_loglik == b[2].total_loglik
    c = run(ctx, prob, cuda, n_iter=2, insert_mode=E.INSERT_ATOMIC, **kw)
    assert rel_l2(a[1], c[1]) < 1e-5
    assert rel_l2(a[0], c[0]) < 1e-4


@pytest.mark.parametrize("precision,interp", PARAMS, ids=IDS)
def test_sorted_against_fp64_oracle(ctx, cuda, prob, precision, interp):
    sigma = 0.3
    s = prob.cfg.side
    m, w, st = run(ctx, prob, cuda, insert_mode=E.INSERT_SORTED, precision=precision,
                   interp=interp)
    want = O.fused_iteration_fp64(prob.init_model, prob.images, prob.mask, prob.x, prob.y,
                                  prob.z, prob.quats, prob.weights, sigma, s, interp=interp)
    tol = 1e-4 if precision == E.PREC_FP32 else 5e-4
    assert rel_l2(w, want["weight"]) < tol
    assert rel_l2(m, want["model"]) < tol


def test_rebind_keeps_or_rebuilds_the_voxel_map(ctx, cuda, prob):
    s, N, R = prob.cfg.side, prob.images.shape[0], prob.quats.shape[0]
    kw = dict(precision=E.PREC_MIXED, insert_mode=E.INSERT_SORTED)
    plan = E.Plan(ctx, s, N, R, **kw)
    bind(plan, prob, cuda)
    first = iterate(plan, prob, cuda)
    bind(plan, prob, cuda)  # same geometry: the map is kept
    again = iterate(plan, prob, cuda)
    assert np.array_equal(first[0], again[0]) and np.array_equal(first[1], again[1])
    # other rotations, same count: the map is rebuilt for them
    rng = np.random.default_rng(11)
    q2 = S.random_quaternions(R, rng).astype(np.float32)
    bind(plan, prob, cuda, quats=q2)
    other = iterate(plan, prob, cuda)
    plan.close()
    fresh = run(ctx, prob, cuda, quats=q2, **kw)
    assert np.array_equal(other[0], fresh[0]) and np.array_equal(other[1], fresh[1])
    assert not np.array_equal(other[1], first[1])


def test_sorted_with_pruning(ctx, cuda, prob):
    """Pruning reorders the plan's rotations: the voxel map follows, and the
    pruned iterations stay bit-identical between runs and near the atomics."""
    s, N, R = prob.cfg.side, prob.images.shape[0], prob.quats.shape[0]

    def go(mode):
        plan = E.Plan(ctx, s, N, R, precision=E.PREC_MIXED, insert_mode=mode)
        bind(plan, prob, cuda)
        plan.set_pruning(True, min_mass=0.999)
        out = iterate(plan, prob, cuda, n_iter=4, sigma=0.2)
        info = plan.prune_info()
        plan.set_pruning(False)  # back to the input rotation order: rebuilt again
        after = iterate(plan, prob, cuda, n_iter=1, sigma=0.2)
        plan.close()
        return out, info, after

    a, info, a2 = go(E.INSERT_SORTED)
    b, _, b2 = go(E.INSERT_SORTED)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert np.array_equal(a2[0], b2[0])
    # a pruned iteration evaluates the tiles that the previous iteration's
    # responsibilities select, so the rounding difference between the two
    # insertion orders can change a tile near the threshold: looser than the
    # full-scan comparison
    c, _, c2 = go(E.INSERT_ATOMIC)
    assert rel_l2(a[1], c[1]) < 1e-3
    assert rel_l2(a2[1], c2[1]) < 1e-3
    assert info["pruned_iterations"] + info["full_iterations"] >= 1


def test_rank_split_with_sorted_insertion(ctx, cuda, prob):
    s, N, R = prob.cfg.side, prob.images.shape[0], prob.quats.shape[0]
    full = run(ctx, prob, cuda, precision=E.PREC_MIXED, insert_mode=E.INSERT_SORTED)
    model = T(prob.init_model, cuda)
    plans, parts = [], []
    for k in range(2):
        r0, r1 = k * R // 2, (k + 1) * R // 2
        p = E.Plan(ctx, s, N, r1 - r0, precision=E.PREC_MIXED, insert_mode=E.INSERT_SORTED)
        bind(p, prob, cuda, quats=prob.quats[r0:r1], weights=prob.weights[r0:r1])
        mx = torch.empty(N, device=cuda)
        sx = torch.empty(N, device=cuda, dtype=torch.float64)
        p.rank_estep(model, 0.3, mx, sx)
        plans.append(p)
        parts.append((mx.double(), sx))
    gm = torch.stack([m for m, _ in parts]).max(0).values
    S_ = sum(sx * torch.where(torch.isfinite(m), torch.exp(m - gm), torch.zeros_like(m))
             for m, sx in parts)
    lse = torch.where(S_ > 0, gm + torch.log(S_), torch.full_like(gm, float("inf")))
    msum, wsum = torch.zeros_like(model), torch.zeros_like(model)
    for p in plans:
        pm, pw = torch.empty_like(model), torch.empty_like(model)
        p.rank_mstep(lse, pm, pw)
        msum += pm
        wsum += pw
    new_m, new_w = torch.empty_like(model), torch.empty_like(model)
    plans[0].model_from_sums(msum, wsum, 2, new_m, new_w)
    plans[0].wait()
    got_m = new_m.cpu().numpy()
    got_w = new_w.cpu().numpy() * 2
    for p in plans:
        p.close()
    assert rel_l2(got_w, full[1]) < 1e-5
    assert rel_l2(got_m, full[0]) < 1e-4


def test_pair_codes_beyond_32_bits_are_refused(ctx, cuda):
    # 32,769 rotations (16 bits) x 9,216 pixels (14 bits) x 8 corners (3 bits)
    side, N, R = 96, 4, 32769
    rng = np.random.default_rng(2)
    quats = S.random_quaternions(R, rng).astype(np.float32)
    images = rng.poisson(1.0, size=(N, side * side)).astype(np.float32)
    mask = np.ones(side * side, np.int32)
    g = (np.arange(side, dtype=np.float32) - side / 2 + 0.5) * 0.5
    x = np.tile(g, side)
    y = np.repeat(g, side)
    z = np.zeros(side * side, np.float32)
    plan = E.Plan(ctx, side, N, R, precision=E.PREC_FP32, interp=E.INTERP_TRILINEAR,
                  insert_mode=E.INSERT_SORTED)
    with pytest.raises(E.EmcError, match="UNSUPPORTED"):
        plan.bind(T(images, cuda), T(mask, cuda, torch.int32), T(x, cuda), T(y, cuda),
                  T(z, cuda), T(quats, cuda), T(np.ones(R, np.float32), cuda))
    plan.close()
