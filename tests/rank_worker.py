"""One rank of a rotation split, run under torch.distributed with the gloo
backend by tests/test_gpu_rank.py (not collected by pytest itself).

Every rank builds the same seeded problem, makes a plan over its contiguous
range of the rotations (main.cpp:141-154: start = rank R / n, end = (rank + 1)
R / n), runs emc_rank_estep, exchanges the per-pattern partials (MAX of the
maxima, then SUM of the rescaled sums -- main.cpp:367-392) over gloo on host
tensors, runs emc_rank_mstep with the global normaliser, all-reduces the model
and weight sums (main.cpp:467-470) and finishes with emc_model_from_sums.
Rank 0 writes the model, weight and total log-likelihood to argv[1]."""
import os
import sys

import numpy as np
import torch
import torch.distributed as dist

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import emc_gb300 as E  # noqa: E402
from emc_gb300 import synthetic as S  # noqa: E402


def run(out_path, precision):
    dist.init_process_group("gloo")
    rank, world = dist.get_rank(), dist.get_world_size()
    prob = S.make_problem(S.tiny(side=32, n_images=300, rot_n=3, photons=1500, seed=9))
    s, R, N = prob.cfg.side, prob.quats.shape[0], prob.images.shape[0]
    r0, r1 = rank * R // world, (rank + 1) * R // world
    dev = torch.device("cuda:0")
    T = lambda a, dt=torch.float32: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    ctx = E.Context(0)
    plan = E.Plan(ctx, s, N, r1 - r0, precision=precision)
    plan.bind(T(prob.images), T(prob.mask, torch.int32), T(prob.x), T(prob.y), T(prob.z),
              T(prob.quats[r0:r1]), T(prob.weights[r0:r1]))
    model = T(prob.init_model)
    mx = torch.empty(N, device=dev)
    sx = torch.empty(N, device=dev, dtype=torch.float64)
    plan.rank_estep(model, 0.3, mx, sx)
    m = mx.double().cpu()
    gm = m.clone()
    dist.all_reduce(gm, op=dist.ReduceOp.MAX)
    sc = sx.cpu() * torch.where(torch.isfinite(m), torch.exp(m - gm), torch.zeros_like(m))
    dist.all_reduce(sc, op=dist.ReduceOp.SUM)
    lse = torch.where(sc > 0, gm + torch.log(sc), torch.full_like(gm, float("inf")))
    msum = torch.empty_like(model)
    wsum = torch.empty_like(model)
    plan.rank_mstep(lse.to(dev), msum, wsum)
    hm, hw = msum.cpu(), wsum.cpu()
    dist.all_reduce(hm, op=dist.ReduceOp.SUM)
    dist.all_reduce(hw, op=dist.ReduceOp.SUM)
    new_model, new_weight = torch.empty_like(model), torch.empty_like(model)
    plan.model_from_sums(hm.to(dev), hw.to(dev), world, new_model, new_weight)
    st = plan.wait()
    if rank == 0:
        np.savez(out_path, model=new_model.cpu().numpy(), weight=new_weight.cpu().numpy(),
                 total_loglik=st.total_loglik)
    plan.close()
    ctx.close()
    dist.barrier()
    dist.destroy_process_group()


if __name__ == "__main__":
    run(sys.argv[1], int(sys.argv[2]))
