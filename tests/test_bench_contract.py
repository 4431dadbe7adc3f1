"""The benchmark's JSON line: every key the report contract names, on small
workloads (the reference arm on CPU, our arm on the GPU)."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_bench(*args, timeout=600):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT,
                         capture_output=True, text=True, timeout=timeout)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, out.stdout[-2000:]
    return json.loads(lines[0])


def check_common(d):
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config", "e2e",
              "cpu_baseline"):
        assert k in d, k
    assert d["metric"] == "fwd+adjoint particle-steps/s"
    assert d["unit"] == "particle-steps/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert "workload" in d["config"]
    for k in ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step"):
        assert k in d["e2e"], k
    for k in ("value", "unit", "cores", "kind", "sample"):
        assert k in d["cpu_baseline"], k
    assert d["cpu_baseline"]["kind"] in ("port", "reference")


def test_reference_arm_line():
    d = run_bench("--impl", "reference", "--side", "24", "--nsteps", "8", "--steps", "1",
                  "--warmup", "1", "--ref-step-seconds", "0.3")
    check_common(d)
    assert d["impl"] == "reference"
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["e2e"]["value"] == d["value"] == d["cpu_baseline"]["value"]


def test_reference_arm_under_torchrun_prints_one_line_from_rank_0():
    # launched like the scaling runs: rank 0 times the CPU path, the other
    # rank exits 0 without work
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
                          "--nproc-per-node", "2", "--master-addr", "127.0.0.1",
                          "--master-port", str(port), os.path.join(ROOT, "bench.py"),
                          "--impl", "reference", "--gpus", "2", "--side", "24", "--nsteps", "8",
                          "--steps", "1", "--warmup", "1", "--ref-step-seconds", "0.3"],
                         cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0


@pytest.mark.gpu
def test_gpu_arm_line():
    d = run_bench("--side", "48", "--nsteps", "16", "--snapshots", "4", "--steps", "1",
                  "--warmup", "3", "--cpu-seconds", "1", "--e2e-steps", "1", "--autotune", "0")
    check_common(d)
    assert d["dtype"] == "f32" and d["n_gpus"] == 1
    r = d["roofline"]
    for k in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
        assert k in r, k
    assert r["bound"] == "hbm" and r["unit"] == "GB/s" and r["achieved"] > 0
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-9
    s = d["solve_roofline"]
    assert s["forward_steps"] == 16 + d["recomputed_forward_steps_per_solve"]
    assert s["bytes_per_solve"] > 0 and s["achieved"] > 0
    assert d["gpu_launches"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] > 0 and d["e2e"]["d2h_bytes_per_step"] > 0
    # nvidia-smi samples every 200 ms: a timed region this short may see none
    assert "clocks" in d
    if d["clocks"] is not None:
        assert "sm_mhz" in d["clocks"] and "reasons" in d["clocks"]
