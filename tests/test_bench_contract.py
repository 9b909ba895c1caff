"""bench.py's output contract, on the CPU.

* The reference arm (`--impl reference`) times the oracle's restatement of the
  reference iteration on the host cores. Run here on a short sample of the
  small configuration, it prints
  one JSON line with the keys the contract names. Its end-to-end figure has no
  host-device copies, and its cpu_baseline describes the same run.
* The default arguments keep the timing rules: at least 3 warm-up steps, N = 1,
  and the mid workload with the reference likelihood."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line(built):
    # the small configuration keeps the synthetic data quick to draw on the CPU
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--config",
           "small", "--steps", "1", "--warmup", "1", "--ref-seconds", "3", "--ref-gpu-chunk", "0"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["value"] > 0 and d["ms_per_step"] > 0 and d["higher_is_better"] is True
    assert d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] == 1
    assert "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_default_arguments_keep_the_timing_rules(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setattr(sys, "argv", ["bench.py"])
    a = bench.parse()
    assert a.gpus == 1 and a.impl == "ours" and a.config == "mid"
    assert a.warmup >= 3 and a.steps >= 1
    assert a.diff == "poisson" and a.insert == "atomic"
    assert a.e2e_steps >= 4
    monkeypatch.setattr(sys, "argv", ["bench.py", "--steps", "20", "--warmup", "5"])
    a = bench.parse()
    assert a.steps == 20 and a.warmup == 5 and a.e2e_steps == 10
