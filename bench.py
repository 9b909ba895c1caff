#!/usr/bin/env python
"""EMC iteration throughput on GB300 (one JSON line on rank 0).

Step = one full EMC iteration (expand, scaling, likelihood, log-sum-exp,
M-step, insertion, divide, normalise) of the mid-size configuration:
128^3 model, 20,000 patterns of 128x128 (~5,000 photons, scale U(0.5,1.5),
beamstop 6 px), 25,680 rotations (600-cell level n = 8), the reference's
"poisson" difference with per-pair scaling.  Synthetic, seeded data with
those shapes stands in for HDF5 patterns (none are named or available).

value     pairs/s = R * N / step time, inputs resident in HBM, CUDA events on
          the library's stream around K iterations, max over ranks.
e2e       the same metric through the public API with host buffers: every
          step copies the patterns and model from pinned host memory, binds,
          iterates and reads back model, weight and log-likelihood.
roofline  the dominant kernel (the E-step: scaling + likelihood + LSE
          partials), its algorithmic FLOPs per launch over its event-timed
          duration, against the measured peak in MEASURED_PEAKS.json.
cpu_baseline / --impl reference
          the oracle's C restatement of the reference kernels (OpenMP, all
          host threads) on a bounded sample of the same workload.
Multi-GPU: replicas only (one independent iteration per rank; the reference's
rotation split has no exchange to accelerate on single-GPU machines).
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "EMC iter/s & rot·pattern pairs/s, mixed-prec+pruned vs plain FP32, same GB300"
UNIT = "rot·pattern pairs/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", default="mid")
    ap.add_argument("--precision", choices=["auto", "mixed", "fp32"], default="auto")
    ap.add_argument("--insert", choices=["atomic", "deterministic", "sorted"], default="atomic")
    ap.add_argument("--mstep-qlo", type=int, choices=[0, 1], default=0,
                    help="tensor M-step: responsibility x scaling as FP16 hi+lo (1) or hi (0)")
    ap.add_argument("--diff", choices=["poisson", "true_poisson"], default="poisson",
                    help="likelihood: the reference's poisson (weighted least squares) or "
                         "the counts x log-slice Poisson likelihood")
    ap.add_argument("--mstep-aggregate", type=int, choices=[0, 1], default=0,
                    help="tensor M-step: warp-aggregated atomics for nearest insertion")
    ap.add_argument("--estep-ghlo", type=int, choices=[-1, 0, 1, 2, 3], default=-1,
                    help="tensor E-step: lo terms of G (bit 0) and H (bit 1); -1: the library's "
                         "default (G, and H when the intensity is known)")
    ap.add_argument("--counts-round", type=int, choices=[-1, 0, 1], default=-1,
                    help="tensor path: round counts above 2,048 to the nearest FP16 value "
                         "(relative change <= 2^-12 on those pixels); without it such "
                         "patterns run on the FP32 path.  -1: on for the large configuration "
                         "(FP16 counts by its definition), off otherwise")
    ap.add_argument("--learned-epochs", type=int, default=-1,
                    help="learned rotation proposal leg: training epochs (0: skip; -1: 30 for "
                         "the large configuration, 10 for mid, 0 otherwise)")
    ap.add_argument("--estep-pair", type=int, choices=[0, 1], default=1,
                    help="tensor path: full likelihood scans on CTA pairs (EMC_OPT_ESTEP_PAIR)")
    ap.add_argument("--mstep-pair", type=int, choices=[0, 1], default=1,
                    help="tensor path: full-scan M-step on CTA pairs (EMC_OPT_MSTEP_PAIR)")
    ap.add_argument("--mstep-raster", type=int, default=0,
                    help="tensor path: the M-step's tile order (EMC_OPT_MSTEP_RASTER); 0: the "
                         "library's default")
    ap.add_argument("--raster", type=int, default=0,
                    help="tensor path: the likelihood kernel's tile order (EMC_OPT_ESTEP_RASTER); "
                         "0 (default): chosen by emc_plan_autotune before the warm-up")
    ap.add_argument("--plain-steps", type=int, default=2)
    ap.add_argument("--e2e-steps", type=int, default=-1,
                    help="end-to-end steps (-1: max(4, steps / 2)); the first step's pattern "
                         "copy is not hidden, later ones overlap the previous step")
    ap.add_argument("--cpu-seconds", type=float, default=15.0,
                    help="target duration of the FP64 host-oracle baseline (cpu_baseline)")
    ap.add_argument("--ref-seconds", type=float, default=100.0,
                    help="--impl reference: target duration of all warm-up + timed steps")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-gpu-chunk", type=int, default=128,
                    help="--impl reference: rotations per timed chunk of the reference's own "
                         "CUDA kernels (0: skip them)")
    ap.add_argument("--prune-steps", type=int, default=4,
                    help="timed iterations of the pruned-vs-full leg (0: skip)")
    args = ap.parse_args()
    if args.counts_round < 0:
        args.counts_round = int(args.config == "large")
    if args.e2e_steps < 0:
        args.e2e_steps = max(4, args.steps // 2)
    if args.learned_epochs < 0:
        args.learned_epochs = {"large": 30, "mid": 10}.get(args.config, 0)
    return args


# ------------------------------------------------------------ helpers ----
def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return dict(hbm=d.get("hbm_gbs"), bf16=d.get("bf16_tflops"),
                    bf16_sustained=d.get("bf16_tflops_sustained"), source="measured")
    return dict(hbm=6800.0, bf16=1900.0, bf16_sustained=1700.0, source="fallback")


def profile_traffic(kernel_key):
    """traffic_bytes_per_launch recorded in the committed ncu summary for this
    kernel and workload (profiles/<kernel>_<workload>.md), else None."""
    d = os.path.join(ROOT, "profiles")
    if not os.path.isdir(d):
        return None
    path = os.path.join(d, kernel_key + ".md")
    if os.path.exists(path):
        m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", open(path).read())
        if m:
            return float(m.group(1))
    return None


REASONS = {  # clocks_event_reasons bit names (nvidia-smi)
    "hw_slowdown": 0x8, "hw_thermal_slowdown": 0x40, "sw_thermal_slowdown": 0x20,
    "sw_power_cap": 0x4, "hw_power_brake_slowdown": 0x80,
}


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed
    region (started before, stopped after)."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        import tempfile
        fd, self.path = tempfile.mkstemp(prefix="emc_clocks_", suffix=".csv")
        os.close(fd)

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 4:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
                bits = int(parts[3], 16)
            except ValueError:
                continue
            for name, b in REASONS.items():
                if bits & b:
                    reasons.add(name)
        try:
            os.remove(self.path)
        except OSError:
            pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        top = max(sm)
        loaded = [v for v in sm if v >= 0.5 * top] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(args):
    import torch
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ws, v):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_problem(cfg_name, device):
    from emc_gb300 import synthetic as S
    return S.make_problem(S.CONFIGS[cfg_name], device=device)


def workload_desc(prob, precision, insert):
    c = prob.cfg
    return {"workload": f"{c.name}: {c.side}^3 model, {c.n_images} patterns {c.side}x{c.side} "
                        f"(~{c.photons:g} photons, scale U{c.scale}, beamstop {c.beamstop} px), "
                        f"{prob.quats.shape[0]} rotations (n={c.rot_n}), one full EMC iteration",
            "side": c.side, "n_images": c.n_images, "n_rot": int(prob.quats.shape[0]),
            "p_eff": int(prob.mask.sum()), "interp": "nearest",
            "precision": precision, "insert": insert,
            "l2": f"inputs larger than L2 (patterns {prob.images.nbytes / 1e9:.1f} GB, "
                  f"responsibilities {4.0 * prob.quats.shape[0] * c.n_images / 1e9:.1f} GB "
                  f"per step)"}


# ---------------------------------------------------- CPU (oracle) legs ----
def b1_leg(prob, seconds):
    """The FP64 host oracle in GEMM form (oracle.fused_iteration_fp64: numpy /
    OpenBLAS on all host threads) on a chunk of rotations x ALL patterns of the
    workload, full detector: the fused iteration's semantics evaluated in
    FP64.  The chunk is sized from a probe so the timed run takes about
    `seconds`.  Returns the cpu_baseline object."""
    from oracle import oracle as O
    s, R, N = prob.cfg.side, prob.quats.shape[0], prob.images.shape[0]
    cores = os.cpu_count() or 1

    def run(nr):
        t0 = time.perf_counter()
        O.fused_iteration_fp64(prob.init_model, prob.images, prob.mask, prob.x, prob.y, prob.z,
                               prob.quats[:nr], prob.weights[:nr], float(O.sigma_at(0)), s)
        return time.perf_counter() - t0

    nr0 = min(R, 64)
    t0 = run(nr0)
    nr = int(min(R, max(nr0, nr0 * seconds / max(t0, 1e-3))))
    t = run(nr) if nr != nr0 else t0
    return dict(value=nr * N / t, unit=UNIT, cores=cores, kind="port",
                sample=f"{nr} rotations x all {N} patterns of the {prob.cfg.name} workload, full "
                       f"{s}x{s} detector ({int(prob.mask.sum())} mask pixels): one iteration "
                       f"of the fused semantics in FP64 (oracle.fused_iteration_fp64, numpy "
                       f"GEMMs on {cores} threads), {t:.1f} s")


def ref_chunk_leg(prob, chunk, r0):
    """One pass of the oracle's restatement of the reference iteration
    (oracle.ref_iteration -> oracle/emc_oracle.c, OpenMP on all host
    threads: int-truncated scaling denominator, FP64 per-pixel likelihood,
    float log-sum-exp, M-step with insertion, divide, normalise) over the
    rotation chunk [r0, r0 + chunk) x ALL patterns, full detector -- the unit
    of work main.cpp:284-462 loops over (slice_chunk).  Returns seconds."""
    from oracle import oracle as O
    s = prob.cfg.side
    q, w = prob.quats[r0:r0 + chunk], prob.weights[r0:r0 + chunk]
    t0 = time.perf_counter()
    O.ref_iteration(prob.init_model, prob.images, prob.mask, prob.x, prob.y, prob.z, q, w,
                    O.sigma_at(0), s, chunk=chunk)
    return time.perf_counter() - t0


# ------------------------------------------------------------ GPU leg ----
def run_ours(args):
    import numpy as np
    import torch

    import emc_gb300 as E

    ws, rank, local = dist_setup(args)
    dev = torch.device(f"cuda:{local}")
    prob = make_problem(args.config, "cuda")
    torch.cuda.empty_cache()  # the generator's buffers go back to the device for the plan
    s, R, N = prob.cfg.side, prob.quats.shape[0], prob.images.shape[0]
    ctx = E.Context(local)
    # one explicit stream for torch copies and library kernels (the legacy
    # default stream has handle 0, which the library maps to its own stream)
    torch_stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(torch_stream)
    ctx.set_stream(torch_stream.cuda_stream)
    T = lambda a, dt=torch.float32: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    images, mask = T(prob.images), T(prob.mask, torch.int32)
    x, y, z, rot, w = T(prob.x), T(prob.y), T(prob.z), T(prob.quats), T(prob.weights)
    insert = {"atomic": E.INSERT_ATOMIC, "deterministic": E.INSERT_DETERMINISTIC,
              "sorted": E.INSERT_SORTED}[args.insert]

    def new_plan(prec):
        diff = E.DIFF_TRUE_POISSON if args.diff == "true_poisson" else E.DIFF_POISSON
        # the configuration's blur of the new model (the small configuration: sigma 1)
        p = E.Plan(ctx, s, N, R, diff=diff, precision=prec, insert_mode=insert,
                   blur_sigma=prob.cfg.blur)
        p.set_option(E.Plan.OPT_MSTEP_QLO, args.mstep_qlo)
        p.set_option(E.Plan.OPT_ESTEP_GHLO, args.estep_ghlo)
        p.set_option(E.Plan.OPT_MSTEP_AGGREGATE, args.mstep_aggregate)
        if prec == E.PREC_MIXED and args.counts_round:
            p.set_option(E.Plan.OPT_COUNTS_ROUND, 1)
        p.set_option(E.Plan.OPT_ESTEP_PAIR, args.estep_pair)
        p.set_option(E.Plan.OPT_MSTEP_PAIR, args.mstep_pair)
        if args.mstep_raster:
            p.set_option(E.Plan.OPT_MSTEP_RASTER, args.mstep_raster)
        p.bind(images, mask, x, y, z, rot, w)
        return p

    precision = args.precision
    plan = None
    if precision in ("auto", "mixed"):
        try:
            plan = new_plan(E.PREC_MIXED)
            precision = "mixed"
        except E.EmcError:
            if args.precision == "mixed":
                raise
            plan = None
    if plan is None:
        plan = new_plan(E.PREC_FP32)
        precision = "fp32"
    plan.set_profiling(True)
    model = T(prob.init_model)
    weight = torch.empty_like(model)
    sig = [E.sigma_schedule(i, 0.4, 0.12, 25) for i in range(args.warmup + args.steps)]
    tuning = None
    if precision == "mixed":
        if args.raster:
            plan.set_option(E.Plan.OPT_ESTEP_RASTER, args.raster)
            tuning = {"estep_raster": args.raster, "source": "--raster"}
        else:
            t0 = time.perf_counter()
            r, ms = plan.autotune(model, sig[0])
            tuning = {"estep_raster": r, "source": "emc_plan_autotune",
                      "estep_pair": plan.get_option(E.Plan.OPT_ESTEP_PAIR),
                      "prefix_ms": ms, "tuning_s": time.perf_counter() - t0}
        # the autotuner may have chosen single-CTA likelihood tiles
        args.estep_pair = plan.get_option(E.Plan.OPT_ESTEP_PAIR)
    for i in range(args.warmup):
        plan.iterate(model, weight, sig[i], stats=False)
    torch.cuda.synchronize()

    # ---- timed region
    sampler = ClockSampler(local)
    sampler.start()
    launches0 = ctx.kernel_launches
    barrier(ws)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(torch_stream)
    estep_ms = []
    phases = []
    for k in range(args.steps):
        plan.iterate(model, weight, sig[args.warmup + k], stats=False)
        ph = plan.phase_ms()
        phases.append(ph)
        estep_ms.append(ph["estep"])
    ev1.record(torch_stream)
    torch.cuda.synchronize()
    barrier(ws)
    launches = ctx.kernel_launches - launches0
    clocks = sampler.stop()
    ms_total = ev0.elapsed_time(ev1)
    ms_step = max_over_ranks(ws, ms_total / args.steps)
    pairs = float(R) * N
    value = pairs * ws / (ms_step / 1e3)
    st = plan.iterate(model, weight, sig[-1])

    # ---- plain FP32 path on the same GPU (the x10 denominator)
    plain = None
    if precision == "mixed" and args.plain_steps > 0:
        pplan = new_plan(E.PREC_FP32)
        m2 = T(prob.init_model)
        w2 = torch.empty_like(m2)
        pplan.iterate(m2, w2, sig[0], stats=False)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(torch_stream)
        for k in range(args.plain_steps):
            pplan.iterate(m2, w2, sig[k], stats=False)
        e1.record(torch_stream)
        torch.cuda.synchronize()
        pms = e0.elapsed_time(e1) / args.plain_steps
        plain = {"ms_per_step": pms, "pairs_per_s": pairs / (pms / 1e3),
                 "iter_per_s": 1e3 / pms}
        pplan.close()
    elif precision == "fp32":
        plain = {"ms_per_step": ms_step, "pairs_per_s": pairs / (ms_step / 1e3),
                 "iter_per_s": 1e3 / ms_step, "note": "the measured path is the plain FP32 path"}

    # ---- end to end through the public API with host buffers
    e2e = None
    if args.e2e_steps > 0:
        e2e = run_e2e(args, prob, plan, images, mask, x, y, z, rot, w, model, weight, sig,
                      torch_stream, ws, pairs)
    pruned = None
    workspace = plan.workspace_bytes
    if precision == "mixed" and args.prune_steps > 0 and rank == 0:
        plan.close()  # the prune leg's plans need the device memory
        torch.cuda.synchronize()
        pruned = prune_leg(args, prob, ctx, T, (images, mask, x, y, z, rot, w), pairs)
    if precision == "mixed" and args.learned_epochs > 0 and rank == 0:
        if args.prune_steps <= 0:
            plan.close()
            torch.cuda.synchronize()
        pruned = dict(pruned or {}, learned=learned_leg(args, prob, ctx, T,
                                                        (images, mask, x, y, z, rot, w)))
    return finish(args, prob, workspace, ctx, ws, rank, precision, value, ms_step, st, plain, e2e,
                  estep_ms, phases, launches, clocks, pairs, pruned, tuning)


def prune_leg(args, prob, ctx, T, inputs, pairs):
    """Pruned against full-scan iterations of the counts x log-slice Poisson
    likelihood (the likelihood whose responsibilities are peaked enough to
    prune; the reference's sigma-tempered one is not at these sigmas), in the
    late-iteration regime: both runs start from the state after 3 full
    iterations begun at the true particle, then run 2 untimed and K timed
    iterations each.  Reports both throughputs, the evaluated share of the
    tiles, fallbacks and the final model's distance to the full-scan run."""
    import numpy as np
    import torch

    import emc_gb300 as E
    s, R, N = prob.cfg.side, prob.quats.shape[0], prob.images.shape[0]

    def plan_b(raster=0):
        p = E.Plan(ctx, s, N, R, diff=E.DIFF_TRUE_POISSON, precision=E.PREC_MIXED)
        if args.counts_round:
            p.set_option(E.Plan.OPT_COUNTS_ROUND, 1)
        p.bind(*inputs)
        if raster:
            p.set_option(E.Plan.OPT_ESTEP_RASTER, raster)
        return p
    full = plan_b(args.raster)
    m0 = T(prob.true_model)
    ctx.normalize_model(s, m0)
    raster = args.raster or full.autotune(m0, 0.12)[0]
    w0 = torch.empty_like(m0)
    for _ in range(3):
        full.iterate(m0, w0, 0.12, stats=False)
    runs = {}
    for kind in ("full", "pruned"):
        # one plan at a time: at 256^3 a plan takes most of the device memory
        plan = full if kind == "full" else plan_b(raster)
        if kind == "pruned":
            plan.set_pruning(True, min_mass=0.999, dilate=1.0)
        m = m0.clone()
        w = torch.empty_like(m)
        torch.cuda.synchronize()
        for _ in range(2):
            plan.iterate(m, w, 0.12, stats=False)
        t = []
        for _ in range(args.prune_steps):
            t0 = time.perf_counter()
            plan.iterate(m, w, 0.12, stats=False)  # returns after its own synchronise
            t.append(time.perf_counter() - t0)
        runs[kind] = (statistics.mean(t), m.cpu().numpy().astype(np.float64),
                      plan.prune_info() if kind == "pruned" else None)
        plan.close()
        torch.cuda.synchronize()
    tf, mf, _ = runs["full"]
    tp, mp, info = runs["pruned"]
    return {"likelihood": "true poisson (counts x log slice), mixed precision",
            "state": "after 3 full iterations from the true particle (late-iteration regime)",
            "timing": "host clock around emc_iterate, which ends with a synchronise",
            "full_ms_per_step": tf * 1e3, "pruned_ms_per_step": tp * 1e3,
            "speedup": tf / tp,
            "full_scan_equivalent_pairs_per_s": pairs / tp,
            "evaluated_pairs_per_s": pairs * info["active_fraction"] / tp,
            "active_fraction": info["active_fraction"], "core_fraction": info["core_fraction"],
            "pruned_iterations": info["pruned_iterations"],
            "fallback_iterations": info["fallback_iterations"],
            "full_iterations": info["full_iterations"], "estep_raster": raster,
            "model_rel_l2_vs_full_scan": float(np.linalg.norm(mp - mf) / np.linalg.norm(mf))}


def learned_leg(args, prob, ctx, T, inputs):
    """The learned rotation proposal: labels are the most probable rotations
    of one full-scan iteration (counts x log-slice likelihood, from the true
    particle); the network is trained on those patterns (GPU kernels of the
    library), then predicts a held-out set of as many new patterns of the
    same particle, whose first iteration is seeded by the proposals (2 % ball
    around the prediction and its Friedel mate, margin, probe tiles) and timed
    against its full scan.  Reports training time, held-out angular errors
    against the true orientations, the seeded tile share, whether the
    fallback ran and the model's distance to the full scan."""
    import numpy as np
    import torch

    import emc_gb300 as E
    from emc_gb300 import synthetic as S
    s, R, N = prob.cfg.side, prob.quats.shape[0], prob.images.shape[0]
    images, mask, x, y, z, rot, w = inputs

    def plan_on(images):
        p = E.Plan(ctx, s, N, R, diff=E.DIFF_TRUE_POISSON, precision=E.PREC_MIXED)
        if args.counts_round:
            p.set_option(E.Plan.OPT_COUNTS_ROUND, 1)
        p.bind(images, mask, x, y, z, rot, w)
        return p
    m0 = T(prob.true_model)
    ctx.normalize_model(s, m0)
    plan = plan_on(images)
    m, wt = m0.clone(), torch.empty_like(m0)
    plan.iterate(m, wt, 0.12, stats=False)
    labels = torch.empty((N, 4), device=m0.device)
    plan.best_quaternions(labels)
    plan.close()
    net = E.Proposal(ctx, seed=1)
    net.set_data(images, mask, s)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    losses = net.train(labels, epochs=args.learned_epochs, batch=128, lr=1e-3, seed=1)
    train_s = time.perf_counter() - t0
    held = S.make_problem(prob.cfg, device="cuda", pattern_seed=1)
    torch.cuda.empty_cache()
    himages = T(held.images)
    net.set_data(himages, mask, s, fit_stats=False)
    props = net.predict(torch.empty((N, 2, 4), device=m0.device))
    net.close()
    pq = props.cpu().numpy().astype(np.float64)
    tq = held.true_quats
    err = np.degrees(2 * np.arccos(np.clip(np.maximum(np.abs((pq[:, 0] * tq).sum(1)),
                                                      np.abs((pq[:, 1] * tq).sum(1))), 0, 1)))
    runs = {}
    for kind in ("full", "seeded"):
        plan = plan_on(himages)
        if args.raster:
            plan.set_option(E.Plan.OPT_ESTEP_RASTER, args.raster)
        seeded = None
        if kind == "seeded":
            plan.set_pruning(True, min_mass=0.999, dilate=1.0)
            plan.set_proposals(props, 0.02, 16)
            seeded = plan.prune_info()["active_fraction"]
        m = m0.clone()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        plan.iterate(m, wt, 0.12, stats=False)  # ends with a synchronise
        dt = time.perf_counter() - t0
        info = plan.prune_info() if kind == "seeded" else None
        runs[kind] = (dt, m.cpu().numpy().astype(np.float64), info, seeded)
        plan.close()
        torch.cuda.synchronize()
    tf, mf, _, _ = runs["full"]
    tp, mp, info, seeded = runs["seeded"]
    return {"network": "4 conv 3x3/2 (64 ch) + linear to 6D, FP32, trained on the GPU",
            "train_patterns": N, "epochs": args.learned_epochs,
            "train_s": train_s, "loss_first_last": [float(losses[0]), float(losses[-1])],
            "heldout_patterns": N,
            "heldout_err_deg_median": float(np.median(err)),
            "heldout_err_deg_p90": float(np.percentile(err, 90)),
            "heldout_within_2pct_ball": float((err < 41.8).mean()),
            "seeded_active_fraction": seeded, "fallback": bool(info["fallback"]),
            "margin_mass": info["margin_mass"],
            "first_iteration_ms": {"full_scan": tf * 1e3, "seeded": tp * 1e3},
            "model_rel_l2_vs_full_scan": float(np.linalg.norm(mp - mf) / np.linalg.norm(mf))}


def run_e2e(args, prob, plan, images, mask, x, y, z, rot, w, model, weight, sig, torch_stream, ws,
            pairs):
    """End to end through the public API with host buffers: every step copies
    its patterns and start model from pinned host memory, binds, iterates and
    reads model and weight back.  Like a loader of successive batches, the
    patterns of step k + 1 are copied on a second stream into a second device
    buffer while step k iterates (the first step's copy is not hidden); both
    copies and all steps are inside the timed region."""
    import torch
    h_images = torch.from_numpy(prob.images).pin_memory()
    h_model = torch.from_numpy(prob.init_model).pin_memory()
    h_out_m = torch.empty_like(h_model).pin_memory()
    h_out_w = torch.empty_like(h_model).pin_memory()
    bufs = [images, torch.empty_like(images)]
    copy_stream = torch.cuda.Stream(images.device)
    ready = [torch.cuda.Event(), torch.cuda.Event()]
    free = [torch.cuda.Event(), torch.cuda.Event()]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(torch_stream)
    with torch.cuda.stream(copy_stream):
        copy_stream.wait_event(e0)
        bufs[0].copy_(h_images, non_blocking=True)
        ready[0].record(copy_stream)
    lls = []
    for k in range(args.e2e_steps):
        b = k % 2
        torch_stream.wait_event(ready[b])
        model.copy_(h_model, non_blocking=True)
        plan.bind(bufs[b], mask, x, y, z, rot, w)
        if k + 1 < args.e2e_steps:  # the next step's patterns, into the other buffer
            with torch.cuda.stream(copy_stream):
                if k >= 1:
                    copy_stream.wait_event(free[1 - b])
                bufs[1 - b].copy_(h_images, non_blocking=True)
                ready[1 - b].record(copy_stream)
        stk = plan.iterate(model, weight, sig[k % len(sig)])
        free[b].record(torch_stream)
        h_out_m.copy_(model, non_blocking=True)
        h_out_w.copy_(weight, non_blocking=True)
        lls.append(stk.total_loglik)
    e1.record(torch_stream)
    torch.cuda.synchronize()
    wall = (time.perf_counter() - t0) / args.e2e_steps
    event_ms = e0.elapsed_time(e1) / args.e2e_steps
    e2e_ms = max(event_ms, wall * 1e3)
    e2e_ms = max_over_ranks(ws, e2e_ms)
    plan.bind(images, mask, x, y, z, rot, w)  # back to the first buffer
    del bufs
    return {"value": pairs * ws / (e2e_ms / 1e3), "unit": UNIT,
            "h2d_bytes_per_step": int(prob.images.nbytes + prob.init_model.nbytes),
            "d2h_bytes_per_step": int(2 * prob.init_model.nbytes + 8 * 4),
            "ms_per_step": e2e_ms, "event_ms_per_step": event_ms, "host_ms_per_step": wall * 1e3,
            "overlap": "patterns of the next step copied on a second stream during this step"}


def finish(args, prob, workspace, ctx, ws, rank, precision, value, ms_step, st, plain, e2e,
           estep_ms, phases, launches, clocks, pairs, pruned=None, tuning=None):
    # ---- roofline of the dominant kernel (E-step)
    peaks = load_peaks()
    p_eff = int(prob.mask.sum())
    if args.diff == "poisson":
        flops = 8.0 * p_eff * pairs  # 4 GEMM-equivalents (num, den, B, C) x 2 FLOP
        kernel = ("tc_estep_pair_kernel" if args.estep_pair else "tc_estep_kernel") \
            if precision == "mixed" else "estep_fp32_kernel"
    else:
        flops = 2.0 * p_eff * pairs  # one GEMM-equivalent (counts x log slice) x 2 FLOP
        kernel = "tc_estep_pois_kernel" if precision == "mixed" else "estep_pois_fp32_kernel"
    est = statistics.mean(estep_ms)
    achieved = flops / (est / 1e3) / 1e12
    traffic = profile_traffic(f"{kernel}_{prob.cfg.name}")
    roofline = {"bound": "tensor", "kernel": kernel, "achieved": achieved,
                "peak": peaks["bf16"], "unit": "TFLOP/s", "frac": achieved / peaks["bf16"],
                "peak_source": f"bf16_tflops of {peaks['source']} peaks",
                "flops_per_launch": flops, "ms_per_launch": est,
                "traffic": traffic}
    if precision == "fp32":
        roofline["note"] = ("plain FP32 SIMT kernel; against the FP32 FMA pipe "
                            "(152 SMs x 128 lanes x 2 x sm clock) it runs at "
                            f"{achieved / (152 * 128 * 2 * (clocks.get('sm_mhz') or 1900) * 1e6 / 1e12):.2f}")
    phase_mean = {k: statistics.mean(p[k] for p in phases) for k in phases[0]}

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cpu = b1_leg(prob, args.cpu_seconds)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if precision == "fp32" else "f16/f32",
            "data": f"synthetic (seeded; shapes of the {args.config} configuration)",
            "config": dict(workload_desc(prob, precision, args.insert),
                           diff="poisson (reference)" if args.diff == "poisson"
                           else "true poisson (counts x log slice)",
                           mstep_q="fp16 hi+lo" if args.mstep_qlo else "fp16 hi",
                           estep_gh={-1: "G fp16 hi+lo, H fp16 hi", 3: "G, H fp16 hi+lo",
                                     2: "G hi, H hi+lo", 1: "G hi+lo, H hi",
                                     0: "G, H fp16 hi"}[args.estep_ghlo],
                           mstep_atomics="warp-aggregated" if args.mstep_aggregate else "per pair",
                           estep_kernel="CTA pairs (256-row MMAs)" if args.estep_pair
                           else "single CTAs",
                           mstep_kernel="CTA pairs (256-row MMAs)" if args.mstep_pair
                           else "single CTAs",
                           counts="counts above 2048 rounded to fp16" if
                           (args.counts_round and precision == "mixed") else "exact"),
            "iter_per_s": ws * 1e3 / ms_step,
            "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "plain_fp32": plain,
            "pruned": pruned,
            "speedup_vs_plain_fp32": (plain["ms_per_step"] / ms_step) if plain else None,
            "phase_ms": phase_mean, "gpu_launches": launches, "clocks": clocks,
            "total_loglik": st.total_loglik, "captured_mass": st.captured_mass,
            "workspace_gb": workspace / 1e9, "tile_order": tuning,
        }
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_reference(args):
    """The reference arm.  The reference's own code for this path is CUDA
    (emc_cuda.cu, emc_atomic.cu) driven by an MPI host that cannot be built
    here; its CPU stand-in is the oracle's restatement of those kernels
    (kind "port"), timed on a rotation chunk x all patterns per step, with
    inputs built from the reference's own rotations.c and
    calculate_coordinates (oracle/_ref) -- nothing of this project's library
    is loaded.  The reference's CUDA kernels, built unchanged for sm_103a, are
    timed beside it on one chunk (reference_gpu)."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from emc_gb300 import synthetic as S  # data generation only: numpy / torch
    from oracle import oracle as O
    cfg = S.CONFIGS[args.config]
    rotations = O.ref_rotations(cfg.rot_n)
    coords = O.ref_coordinates(cfg.side, S.PIXEL_SIZE, S.DISTANCE, S.WAVELENGTH)
    if rotations is None or coords is None:
        print(json.dumps({"impl": "reference", "metric": METRIC,
                          "unavailable": "the reference's rotations.c / emc_helper.cpp builds "
                                         "(oracle/_ref) are missing: no reference tree staged"}),
              flush=True)
        return
    try:
        import torch
        dev = "cuda" if torch.cuda.is_available() else None
    except Exception:
        dev = None
    prob = S.make_problem(cfg, device=dev, coords=coords, rotations=rotations)
    R, N = prob.quats.shape[0], prob.images.shape[0]
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    # chunk sized so that warm-up + timed steps take about args.ref_seconds
    probe = min(R, 4)
    t_probe = ref_chunk_leg(prob, probe, 0)
    per_step = max(1.0, args.ref_seconds / max(1, args.warmup + args.steps))
    chunk = int(min(R, max(1, probe * per_step / max(t_probe, 1e-3))))
    times = []
    for k in range(args.warmup + args.steps):
        r0 = (k * chunk) % max(1, R - chunk + 1)
        t = ref_chunk_leg(prob, chunk, r0)
        if k >= args.warmup:
            times.append(t)
    t_step = statistics.mean(times)
    v = chunk * N / t_step
    ref_gpu = None
    if dev == "cuda" and args.ref_gpu_chunk > 0:
        ref_gpu = ref_gpu_leg(prob, args.ref_gpu_chunk)
    c = prob.cfg
    sample = (f"per step: rotations [r0, r0 + {chunk}) x all {N} patterns, full {c.side}x{c.side} "
              f"detector, one reference-semantics iteration of that chunk (oracle.ref_iteration "
              f"-> oracle/emc_oracle.c, OpenMP, {cores} threads)")
    workload = workload_desc(prob, "reference (quirk-exact CPU restatement)", "sequential")
    workload["workload"] = (f"{c.name}: {c.side}^3 model, {N} patterns {c.side}x{c.side}, "
                            f"{R} rotations (n={c.rot_n}); each step one slice_chunk of {chunk} "
                            f"rotations x all {N} patterns (main.cpp:284-462)")
    workload["rotation_chunk"] = chunk
    workload["inputs"] = ("rotations from the reference's rotations.c and detector coordinates "
                          "from its calculate_coordinates (oracle/_ref builds)")
    line = {"metric": METRIC, "impl": "reference", "value": v, "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64",
            "data": f"synthetic (seeded; shapes of the {args.config} configuration)",
            "config": workload,
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "full_iteration_ms_implied": R * N / v * 1e3,
            "reference_gpu": ref_gpu}
    print(json.dumps(line), flush=True)


def ref_gpu_leg(prob, chunk):
    """The reference's own CUDA kernels (emc_cuda.cu, emc_atomic.cu compiled
    unchanged for sm_103a by oracle/build_ref.sh --kernels) on one chunk of
    `chunk` rotations x all patterns of the workload, in main.cpp's order for
    one chunk: slices, scaling, slices, likelihood, max, sum exp, normalise,
    slices + insertion.  Each reference call synchronises, as it does in the
    reference.  Returns pairs/s and the full-iteration time it implies."""
    import ctypes as C

    import numpy as np
    import torch
    from oracle.build import ref_dir
    env = dict(os.environ)
    if ref_dir() is not None:
        env["EMC_REF_DIR"] = str(ref_dir())
    so = os.path.join(ROOT, "oracle", "_ref", "libemc_ref_kernels.so")
    if not os.path.exists(so):
        r = subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref.sh"), "--kernels"],
                           env=env, capture_output=True, text=True)
        if r.returncode != 0 or not os.path.exists(so):
            tail = (r.stderr or r.stdout).strip().splitlines()[-1:] or ["no output"]
            return {"unavailable": f"reference kernels did not build: {tail[0][:200]}"}
    lib = C.CDLL(so)
    dev = torch.device("cuda:0")
    s, N = prob.cfg.side, prob.images.shape[0]
    R = prob.quats.shape[0]
    n2 = s * s
    chunk = min(chunk, R)
    T = lambda a, dt=torch.float32: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    ptr = lambda t: C.c_void_p(t.data_ptr())
    model, x, y, z = T(prob.init_model), T(prob.x), T(prob.y), T(prob.z)
    rot, w = T(prob.quats[:chunk]), T(prob.weights[:chunk])
    images, mask = T(prob.images), T(prob.mask, torch.int32)
    slices = torch.empty((chunk, n2), device=dev)
    scaling = torch.ones((chunk, N), device=dev)
    respons = torch.empty((chunk, N), device=dev)
    maxr, sums = torch.empty(N, device=dev), torch.empty(N, device=dev)
    active = torch.ones(N, dtype=torch.int32, device=dev)
    new_model, weight = torch.zeros_like(model), torch.zeros_like(model)
    sigma = C.c_float(0.4)
    steps = []

    def one():
        t = {}
        def timed(name, fn):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            rc = fn()
            torch.cuda.synchronize()
            t[name] = t.get(name, 0.0) + (time.perf_counter() - t0)
            if rc:
                raise RuntimeError(f"reference {name} returned {rc}")
        sl = lambda: lib.ref_get_slices(ptr(model), s, ptr(slices), ptr(rot), ptr(x), ptr(y),
                                        ptr(z), 0, chunk)
        timed("get_slices", sl)
        timed("update_scaling_full", lambda: lib.ref_update_scaling_full(
            ptr(images), ptr(slices), ptr(mask), ptr(scaling), n2, N, 0, chunk, 1))
        timed("get_slices", sl)
        timed("calculate_responsabilities", lambda: lib.ref_calculate_responsabilities(
            ptr(slices), ptr(images), ptr(mask), sigma, ptr(scaling), ptr(respons), ptr(w), n2, N,
            0, chunk, 1))
        timed("max_vector", lambda: lib.ref_max_vector(ptr(respons), N, chunk, ptr(maxr)))
        timed("respons_max_expf", lambda: lib.ref_respons_max_expf(ptr(respons), ptr(maxr), N,
                                                                   chunk, ptr(sums)))
        timed("norm_respons_sumexpf", lambda: lib.ref_norm_respons_sumexpf(
            ptr(respons), ptr(sums), ptr(maxr), N, chunk))
        timed("get_slices", sl)
        timed("update_slices", lambda: lib.ref_update_slices(
            ptr(images), ptr(slices), ptr(mask), ptr(respons), ptr(scaling), ptr(active), N, 0,
            chunk, n2, s, ptr(new_model), ptr(x), ptr(y), ptr(z), ptr(rot), ptr(weight)))
        return t

    one()  # warm-up (module load, first launches)
    steps.append(one())
    per = {k: statistics.mean(st[k] for st in steps) for k in steps[0]}
    total = sum(per.values())
    pairs = float(chunk) * N
    return {"kind": "the reference's CUDA kernels, built unchanged for sm_103a",
            "sample": f"{chunk} rotations x {N} patterns of the workload, one pass of main.cpp's "
                      "per-chunk sequence, host clock around each synchronising call",
            "pairs_per_s": pairs / total, "ms_per_chunk": total * 1e3,
            "ms_per_call": {k: v * 1e3 for k, v in per.items()},
            "full_iteration_ms_implied": R * N / (pairs / total) * 1e3}


# (side, patterns, rotation level) of the eight batched reconstructions
BATCHED = [(48, 500, 3), (64, 1000, 4), (80, 2500, 5), (96, 5000, 6), (112, 10000, 7),
           (128, 15000, 8), (144, 20000, 8), (160, 30000, 8)]


def run_batched(args):
    """Eight uneven reconstructions (48^3..160^3, 500..30,000 patterns, levels
    3..8; synthetic as the small configuration -- 400 atoms, ~1,000 photons,
    scale U(0.5, 1.5) -- with the particle radius and beamstop scaled by
    side/64; seeds 0..7), mixed precision.  Times one iteration of all eight
    as one graph launch (concurrent) against the same eight graphs launched
    one after another, and reports aggregate pairs/s."""
    import numpy as np
    import torch

    import emc_gb300 as E
    from emc_gb300 import synthetic as S
    dev = torch.device("cuda:0")
    T = lambda a, dt=torch.float32: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    ctxs, plans, models, weights, keep, pairs, rasters = [], [], [], [], [], [], []
    for k, (side, n, lvl) in enumerate(BATCHED):
        f = side / 64.0
        cfg = S.Config(f"batched{k}", side, 400, 1.5, 12 * f, n, 1000, (0.5, 1.5), 4 * f, lvl, 1,
                       seed=k)
        prob = S.make_problem(cfg, device="cuda")
        c = E.Context(0)
        R = prob.quats.shape[0]
        plan = E.Plan(c, side, n, R, precision=E.PREC_MIXED)
        inputs = (T(prob.images), T(prob.mask, torch.int32), T(prob.x), T(prob.y), T(prob.z),
                  T(prob.quats), T(prob.weights))
        plan.bind(*inputs)
        m = T(prob.init_model)
        c.normalize_model(side, m)
        rasters.append(plan.autotune(m, 0.4)[0] if not args.raster else args.raster)
        plan.set_option(E.Plan.OPT_ESTEP_RASTER, rasters[-1])
        w = torch.empty_like(m)
        ctxs.append(c)
        plans.append(plan)
        models.append(m)
        weights.append(w)
        keep.append(inputs)
        pairs.append(R * n)
        del prob
    batch = E.Batch(plans, models, weights)
    sig = [E.sigma_schedule(0, 0.4, 0.12, 25)] * len(plans)
    for _ in range(args.warmup):
        batch.run(sig)
        batch.wait()
    clocks = ClockSampler(0)
    clocks.start()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        batch.run(sig)
    batch.wait()
    t_conc = (time.perf_counter() - t0) / args.steps
    # the same captured iterations, one problem after another
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for plan, s in zip(plans, sig):
            plan.replay(s)
            plan.wait(stats=False)
    t_seq = (time.perf_counter() - t0) / args.steps
    ck = clocks.stop()
    total = float(sum(pairs))
    line = {"metric": METRIC, "value": total / t_conc, "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_conc * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f16/f32",
            "data": "synthetic (seeded; eight uneven problems)",
            "config": {"workload": "batched: 8 reconstructions 48^3..160^3, 500..30,000 "
                                   "patterns, rotation levels 3..8, one iteration each",
                       "problems": [{"side": s, "n_images": n, "rot_n": l, "pairs": p,
                                     "estep_raster": r}
                                    for (s, n, l), p, r in zip(BATCHED, pairs, rasters)],
                       "total_pairs": total, "precision": "mixed",
                       "timing": "host clock around graph launches + synchronise"},
            "sequential": {"ms_per_step": t_seq * 1e3, "pairs_per_s": total / t_seq},
            "speedup_vs_sequential": t_seq / t_conc, "clocks": ck}
    print(json.dumps(line), flush=True)
    batch.close()
    for plan, c in zip(plans, ctxs):
        plan.close()
        c.close()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.config == "batched":
        run_batched(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
