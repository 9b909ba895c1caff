"""The reference's rotation split (main.cpp:141-154) on two CPU ranks (gloo).

Each rank owns a contiguous rotation range (emc_helper.cpp:39-45 split), computes
its log-likelihoods, and the ranks exchange exactly what the reference exchanges:
the per-pattern max (Allreduce MAX, main.cpp:373), the per-pattern sum of
exp(L - max) (Allreduce SUM, main.cpp:386), and the model and weight grids
(Allreduce SUM, main.cpp:469-470).  The result must equal one process holding
every rotation.  FP64 oracle arithmetic; no GPU."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from emc_gb300 import synthetic as S
from oracle import oracle as O


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def split_range(R, ntasks, taskid):
    """emc_helper.cpp:39-45 get_allocate_len / main.cpp:141-154."""
    start = taskid * R // ntasks
    end = R if taskid == ntasks - 1 else (taskid + 1) * R // ntasks
    return start, end


def _rank_main(rank, world, port, prob, sigma, out_path):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    s = prob.cfg.side
    R = prob.quats.shape[0]
    a, b = split_range(R, world, rank)
    loc = O.fused_iteration_fp64(prob.init_model, prob.images, prob.mask, prob.x, prob.y, prob.z,
                                 prob.quats[a:b], prob.weights[a:b], sigma, s)
    L = loc["loglik"]  # [R_local, N]; a rotation's L needs no other rotation
    mx = torch.from_numpy(L.max(0))
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    with np.errstate(invalid="ignore"):
        se = torch.from_numpy(np.exp(L - mx.numpy()[None, :]).sum(0))
    dist.all_reduce(se, op=dist.ReduceOp.SUM)
    lse = mx.numpy() + np.log(se.numpy())
    P = np.exp(L - lse[None, :])
    K = O.compacted_counts(prob.images, prob.mask, s)
    pm = prob.mask == 1
    # local insertion, then the model / weight sums of the reference
    phi = loc["phi"]
    Qm = np.where(phi > 0, P / phi, 0.0)
    T32 = P.sum(1).astype(np.float32)  # the rotation totals as the kernels keep them
    T = T32.astype(np.float64)
    U = Qm @ K
    vox = O.nearest_voxels(prob.quats[a:b], prob.x[pm], prob.y[pm], prob.z[pm], s, 0)
    sel = (vox >= 0) & (T32 > np.float32(1e-10))[:, None]
    m = np.bincount(vox[sel], weights=U[sel], minlength=s ** 3)
    w = np.bincount(vox[sel], weights=np.broadcast_to(T[:, None], U.shape)[sel], minlength=s ** 3)
    mt, wt = torch.from_numpy(m), torch.from_numpy(w)
    dist.all_reduce(mt, op=dist.ReduceOp.SUM)
    dist.all_reduce(wt, op=dist.ReduceOp.SUM)
    if rank == 0:
        model = np.where(wt.numpy() > 0, mt.numpy() / np.where(wt.numpy() > 0, wt.numpy(), 1), -1.0)
        model = model / model[model > 0].mean()
        np.savez(out_path, model=model, weight=wt.numpy(), lse=lse)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_rotation_split_exchange_matches_single_process(tmp_path, world):
    prob = S.make_problem(S.tiny(side=20, n_images=40, rot_n=2, photons=1500, n_atoms=40,
                                 radius=4.0))
    sigma = 0.3
    out = str(tmp_path / "r.npz")
    mp.start_processes(_rank_main, args=(world, _free_port(), prob, sigma, out), nprocs=world,
                       join=True, start_method="spawn")
    got = np.load(out)
    want = O.fused_iteration_fp64(prob.init_model, prob.images, prob.mask, prob.x, prob.y, prob.z,
                                  prob.quats, prob.weights, sigma, prob.cfg.side)
    np.testing.assert_allclose(got["lse"], want["lse"], rtol=1e-12)
    np.testing.assert_allclose(got["weight"], want["weight"], rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(got["model"], want["model"], rtol=1e-9, atol=1e-12)
