"""One rank of the reference's rotation split through the library
(emc_rank_estep / emc_rank_mstep / emc_model_from_sums).

* in one process: the rotations split into 1, 2 and 3 contiguous ranges, one
  plan per range, the partials combined as main.cpp:367-392 does (MAX, then
  SUM of the rescaled sums, FP64) and the sums as main.cpp:467-470 does; the
  model must match one plan over all rotations (emc_iterate).  One range is
  emc_iterate exactly.
* across processes: two ranks under torch.distributed (gloo over host
  tensors; both ranks on the same GPU, their kernels never wait on one
  another) run tests/rank_worker.py; rank 0's model must match the one-plan
  iteration."""
import os
import subprocess
import sys

import numpy as np
import pytest
import torch

import emc_gb300 as E
from emc_gb300 import synthetic as S

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def make(seed=9):
    return S.make_problem(S.tiny(side=32, n_images=300, rot_n=3, photons=1500, seed=seed))


def full_iteration(ctx, cuda, prob, precision, sigma=0.3):
    s, R, N = prob.cfg.side, prob.quats.shape[0], prob.images.shape[0]
    T = lambda a, dt=torch.float32: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=cuda)
    plan = E.Plan(ctx, s, N, R, precision=precision)
    plan.bind(T(prob.images), T(prob.mask, torch.int32), T(prob.x), T(prob.y), T(prob.z),
              T(prob.quats), T(prob.weights))
    m = T(prob.init_model)
    w = torch.empty_like(m)
    st = plan.iterate(m, w, sigma)
    plan.close()
    return m.cpu().numpy().astype(np.float64), w.cpu().numpy().astype(np.float64), st.total_loglik


@pytest.mark.parametrize("precision", [E.PREC_FP32, E.PREC_MIXED], ids=["fp32", "mixed"])
@pytest.mark.parametrize("n_ranks", [1, 2, 3])
def test_rotation_split_matches_one_plan(ctx, cuda, precision, n_ranks):
    prob = make()
    s, R, N = prob.cfg.side, prob.quats.shape[0], prob.images.shape[0]
    T = lambda a, dt=torch.float32: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=cuda)
    want_m, want_w, want_ll = full_iteration(ctx, cuda, prob, precision)
    model = T(prob.init_model)
    plans, parts = [], []
    for k in range(n_ranks):
        r0, r1 = k * R // n_ranks, (k + 1) * R // n_ranks
        p = E.Plan(ctx, s, N, r1 - r0, precision=precision)
        p.bind(T(prob.images), T(prob.mask, torch.int32), T(prob.x), T(prob.y), T(prob.z),
               T(prob.quats[r0:r1]), T(prob.weights[r0:r1]))
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
    plans[0].model_from_sums(msum, wsum, n_ranks, new_m, new_w)
    st = plans[0].wait()
    got_m = new_m.cpu().numpy().astype(np.float64)
    got_w = new_w.cpu().numpy().astype(np.float64) * n_ranks
    rel = np.linalg.norm(got_m - want_m) / np.linalg.norm(want_m)
    relw = np.linalg.norm(got_w - want_w) / np.linalg.norm(want_w)
    print(f"precision {precision}, {n_ranks} ranks: model rel L2 {rel:.2e}, weight {relw:.2e}, "
          f"LL {st.total_loglik:.6f} vs {want_ll:.6f}")
    assert rel < 2e-6 and relw < 2e-6
    assert abs(st.total_loglik - want_ll) <= 1e-9 * abs(want_ll)
    for p in plans:
        p.close()


def test_two_ranks_over_gloo(ctx, cuda, tmp_path):
    want_m, want_w, want_ll = full_iteration(ctx, cuda, make(), E.PREC_FP32)
    out = tmp_path / "rank0.npz"
    env = dict(os.environ, MASTER_ADDR="127.0.0.1", NCCL_NVLS_ENABLE="0")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(29400 + os.getpid() % 1000),
           os.path.join(HERE, "rank_worker.py"), str(out), str(E.PREC_FP32)]
    r = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    got = np.load(out)
    gm = got["model"].astype(np.float64)
    gw = got["weight"].astype(np.float64) * 2
    assert np.linalg.norm(gm - want_m) / np.linalg.norm(want_m) < 2e-6
    assert np.linalg.norm(gw - want_w) / np.linalg.norm(want_w) < 2e-6
    assert abs(float(got["total_loglik"]) - want_ll) <= 1e-9 * abs(want_ll)
