"""The `emc` host driver (the counterpart of main.cpp) end to end: emc.conf in,
the reference's output files out, results equal to the library driven from
Python (fused path, deterministic insertion: bit-identical) and to the oracle's
reference-semantics iteration (drop-in path)."""
import json
import os
import subprocess

import numpy as np
import pytest
import torch

import emc_gb300 as E
from emc_gb300 import synthetic as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu
EXE = os.path.join(os.path.dirname(E.__file__), "_build", "emc")


@pytest.fixture(scope="module")
def prob():
    return S.make_problem(S.tiny(side=24, n_images=60, rot_n=2, photons=2000))


def run_driver(conf, out, *args):
    os.makedirs(out, exist_ok=True)
    r = subprocess.run([EXE, conf, "--out", str(out), *args], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    return [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]


def test_fused_driver_matches_library(ctx, cuda, prob, tmp_path):
    conf = S.write_problem(prob, tmp_path / "in", iterations=2)
    logs = run_driver(conf, tmp_path / "out", "--deterministic")
    assert [l["iteration"] for l in logs] == [0, 1]
    s, R, N = prob.cfg.side, prob.quats.shape[0], prob.images.shape[0]
    # the same two iterations through the Python binding
    T = lambda a, dt=torch.float32: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=cuda)
    plan = E.Plan(ctx, s, N, R, insert_mode=E.INSERT_DETERMINISTIC)
    plan.bind(T(prob.images), T(prob.mask, torch.int32), T(prob.x), T(prob.y), T(prob.z),
              T(prob.quats), T(prob.weights))
    m = T(prob.init_model)
    ctx.normalize_model(s, m)  # main.cpp:180
    w = torch.empty_like(m)
    for it in range(2):
        st = plan.iterate(m, w, E.sigma_schedule(it, 0.4, 0.12, 25))
        assert st.total_loglik == logs[it]["total_loglik"]
    mm, ww = m.cpu().numpy(), w.cpu().numpy()
    out = tmp_path / "out"
    model = np.fromfile(out / "output" / "model_0001.bin", np.float32)
    mask = np.fromfile(out / "output" / "model_0001.mask.bin", np.uint8)
    weight = np.fromfile(out / "output" / "weight_0001.bin", np.float32)
    ok = (ww > 0) & (mm > 0)  # file_helper.cpp:50-65
    assert np.array_equal(mask, ok.astype(np.uint8))
    assert np.array_equal(model, np.where(ok, mm, 0).astype(np.float32))
    assert np.array_equal(weight, ww)
    resp = np.fromfile(out / "debug" / "respons_0001.data", np.float32)
    assert resp.size == R * N and abs(resp.reshape(R, N).sum(0) - 1).max() < 1e-4
    assert len(open(out / "ExeTime.data").read().splitlines()) == 3
    q = np.loadtxt(out / "debug_samples.data")
    assert q.shape == (R, 4) and np.allclose(q, prob.quats, atol=1e-5)


def test_dropin_driver_matches_reference_oracle(prob, tmp_path):
    conf = S.write_problem(prob, tmp_path / "in", iterations=1)
    run_driver(conf, tmp_path / "out", "--dropin")
    s = prob.cfg.side
    m0 = prob.init_model.copy()
    O.normalize_model(m0)
    want = O.ref_iteration(m0, prob.images, prob.mask, prob.x, prob.y, prob.z, prob.quats,
                           prob.weights, O.sigma_at(0), s)
    got_w = np.fromfile(tmp_path / "out" / "output" / "weight_0000.bin", np.float32)
    np.testing.assert_allclose(got_w, want["weight"], rtol=1e-5, atol=1e-6 * want["weight"].max())
    got_m = np.fromfile(tmp_path / "out" / "output" / "model_0000.bin", np.float32)
    ok = (want["weight"] > 0) & (want["model"] > 0)
    np.testing.assert_allclose(got_m, np.where(ok, want["model"], 0), rtol=2e-5, atol=1e-6)


def test_driver_bins_raw_frames(prob, tmp_path):
    """Frames whose 2x2 blocks repeat each pattern value bin back to the
    patterns exactly (sum 4k / mask sum 4), so the run equals the one from the
    binned patterns bit for bit."""
    frames = np.repeat(np.repeat(prob.images.reshape(-1, prob.cfg.side, prob.cfg.side), 2, 1), 2, 2)
    fmasks = np.ones(frames.shape, np.int32)
    a = run_driver(S.write_problem(prob, tmp_path / "a", iterations=1), tmp_path / "oa",
                   "--deterministic")
    b = run_driver(S.write_problem(prob, tmp_path / "b", iterations=1, raw=(frames, fmasks),
                                   read_stride=2), tmp_path / "ob", "--deterministic")
    assert a[0]["total_loglik"] == b[0]["total_loglik"]
    for name in ("model_0000.bin", "weight_0000.bin"):
        assert np.array_equal(np.fromfile(tmp_path / "oa" / "output" / name, np.float32),
                              np.fromfile(tmp_path / "ob" / "output" / name, np.float32))


@pytest.mark.parametrize("model_input", [1, 3])
@pytest.mark.parametrize("dropin", [False, True])
def test_driver_model_init_modes(prob, tmp_path, model_input, dropin):
    conf = S.write_problem(prob, tmp_path / "in", iterations=1, model_input=model_input,
                           normalize_images=True)
    logs = run_driver(conf, tmp_path / "out", *(["--dropin"] if dropin else []))
    assert len(logs) == 1 and np.isfinite(logs[0]["total_loglik"])
    m = np.fromfile(tmp_path / "out" / "output" / "model_0000.bin", np.float32)
    assert np.all(np.isfinite(m)) and m.max() > 0


def test_driver_graph_replay_matches_direct(prob, tmp_path):
    """--graph replays one captured iteration: the same files as direct calls."""
    conf = S.write_problem(prob, tmp_path / "in", iterations=2)
    a = run_driver(conf, tmp_path / "a", "--deterministic")
    b = run_driver(conf, tmp_path / "b", "--deterministic", "--graph")
    assert [x["total_loglik"] for x in a] == [x["total_loglik"] for x in b]
    for name in ("model_0001.bin", "weight_0001.bin"):
        assert np.array_equal(np.fromfile(tmp_path / "a" / "output" / name, np.float32),
                              np.fromfile(tmp_path / "b" / "output" / name, np.float32))


def test_driver_prune_writes_input_order(prob, tmp_path):
    """--prune keeps the plan's rotations and patterns in its own order; the
    debug responsibilities come back in the input order (here every iteration
    is a full scan: the first always is, and at sigma 0.4 this likelihood is
    too broad to prune)."""
    conf = S.write_problem(prob, tmp_path / "in", iterations=2)
    a = run_driver(conf, tmp_path / "a", "--precision", "mixed", "--deterministic")
    b = run_driver(conf, tmp_path / "b", "--precision", "mixed", "--deterministic", "--prune")
    R, N = prob.quats.shape[0], prob.images.shape[0]
    for it in range(2):
        assert abs(a[it]["total_loglik"] - b[it]["total_loglik"]) <= 1e-5 * abs(a[it]["total_loglik"])
        ra = np.fromfile(tmp_path / "a" / "debug" / f"respons_{it:04d}.data", np.float32)
        rb = np.fromfile(tmp_path / "b" / "debug" / f"respons_{it:04d}.data", np.float32)
        assert np.abs(ra.reshape(R, N) - rb.reshape(R, N)).max() < 1e-4
