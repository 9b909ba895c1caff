"""Records the reference's own CUDA kernels' outputs as golden fixtures.

Runs on a machine with a GB300.  Builds oracle/_ref/libemc_ref_kernels.so
from the reference sources (emc_cuda.cu, emc_atomic.cu compiled unchanged for
sm_103a behind oracle/ref_harness.cu) -- from $EMC_REF_DIR, else the
staged copy in baseline/_ref/src -- feeds it a small seeded
problem and writes inputs and outputs to the file given as the argument
(default ref_kernels_golden.npz in the working directory), which is committed
as tests/golden/ref_kernels_golden.npz.
    python tests/golden/make_ref_kernel_golden.py [out.npz]
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))


def main():
    import torch

    from emc_gb300 import synthetic as S

    from oracle.build import ref_dir
    env = dict(os.environ)
    if ref_dir() is None:
        raise SystemExit("no reference tree: set EMC_REF_DIR or stage it (build_ref.sh --stage)")
    env["EMC_REF_DIR"] = str(ref_dir())
    subprocess.run(["bash", str(ROOT / "oracle" / "build_ref.sh"), "--kernels"], check=True, env=env)
    lib = C.CDLL(str(ROOT / "oracle" / "_ref" / "libemc_ref_kernels.so"))
    lib.ref_model_average.restype = C.c_float
    dev = torch.device("cuda:0")
    prob = S.make_problem(S.tiny(side=24, n_images=64, rot_n=2, photons=1500, seed=7))
    s, N = prob.cfg.side, prob.images.shape[0]
    R = 96
    quats, weights = prob.quats[:R].copy(), prob.weights[:R].copy()
    T = lambda a, dt=torch.float32: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    ptr = lambda t: C.c_void_p(t.data_ptr())
    out = dict(model=prob.init_model, images=prob.images, mask=prob.mask, x=prob.x, y=prob.y,
               z=prob.z, quats=quats, weights=weights, side=np.int32(s))
    model, x, y, z = T(prob.init_model), T(prob.x), T(prob.y), T(prob.z)
    rot, w, images, mask = T(quats), T(weights), T(prob.images), T(prob.mask, torch.int32)
    # slices of every rotation, in two chunks (start offset exercised)
    slices = torch.empty((R, s * s), device=dev)
    assert lib.ref_get_slices(ptr(model), s, ptr(slices), ptr(rot), ptr(x), ptr(y), ptr(z), 0, 40) == 0
    tail = torch.empty((R - 40, s * s), device=dev)
    assert lib.ref_get_slices(ptr(model), s, ptr(tail), ptr(rot), ptr(x), ptr(y), ptr(z), 40, R - 40) == 0
    slices[40:] = tail
    out["slices"] = slices.cpu().numpy()
    # scaling (int-truncated denominator)
    scaling = torch.ones((R, N), device=dev)
    assert lib.ref_update_scaling_full(ptr(images), ptr(slices), ptr(mask), ptr(scaling), s * s, N,
                                       0, R, 1) == 0
    out["scaling"] = scaling.cpu().numpy()
    # likelihood, reference "poisson" and "absolute"
    sigma = C.c_float(0.3)
    for diff, name in ((1, "respons_poisson"), (0, "respons_absolute")):
        resp = torch.zeros((R, N), device=dev)
        assert lib.ref_calculate_responsabilities(ptr(slices), ptr(images), ptr(mask), sigma,
                                                  ptr(scaling), ptr(resp), ptr(w), s * s, N, 0, R,
                                                  diff) == 0
        out[name] = resp.cpu().numpy()
    resp = T(out["respons_poisson"])
    maxr = torch.empty(N, device=dev)
    assert lib.ref_max_vector(ptr(resp), N, R, ptr(maxr)) == 0
    sums = torch.empty(N, device=dev)
    assert lib.ref_respons_max_expf(ptr(resp), ptr(maxr), N, R, ptr(sums)) == 0
    out["maxr"], out["sums"] = maxr.cpu().numpy(), sums.cpu().numpy()
    lse = T(np.log(out["sums"]).astype(np.float32) + out["maxr"])  # main.cpp:388-389 on the host
    out["lse_host"] = lse.cpu().numpy()
    assert lib.ref_norm_respons_sumexpf(ptr(resp), ptr(lse), ptr(maxr), N, R) == 0
    out["respons_norm"] = resp.cpu().numpy()
    # M-step of the chunk [16, 16+60) and its insertion
    start, chunk = 16, 60
    active = T(np.ones(N, np.int32), torch.int32)
    upd = torch.zeros((chunk, s * s), device=dev)
    new_m = torch.zeros(s ** 3, device=dev)
    new_w = torch.zeros(s ** 3, device=dev)
    rot_chunk = T(quats[start:start + chunk])
    assert lib.ref_update_slices(ptr(images), ptr(upd), ptr(mask), ptr(resp), ptr(scaling),
                                 ptr(active), N, start, chunk, s * s, s, ptr(new_m), ptr(x), ptr(y),
                                 ptr(z), ptr(rot_chunk), ptr(new_w)) == 0
    out["upd_slices"] = upd.cpu().numpy()
    out["ins_model"], out["ins_weight"] = new_m.cpu().numpy(), new_w.cpu().numpy()
    # divide and normalise
    assert lib.ref_divide_model_by_weight(s, ptr(new_m), ptr(new_w)) == 0
    out["divided"] = new_m.cpu().numpy()
    out["avg_before"] = np.float32(lib.ref_model_average(ptr(new_m), s ** 3))
    assert lib.ref_normalize_model(s, ptr(new_m)) == 0
    out["normalized"] = new_m.cpu().numpy()
    dst = Path(sys.argv[1] if len(sys.argv) > 1 else "ref_kernels_golden.npz").resolve()
    dst.parent.mkdir(parents=True, exist_ok=True)
    np.savez_compressed(dst, **out)
    print(f"wrote {dst} ({dst.stat().st_size} bytes)")


if __name__ == "__main__":
    main()
