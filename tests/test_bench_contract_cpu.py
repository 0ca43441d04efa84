"""The benchmark's command-line contract, on the CPU.

bench.py prints one JSON line per run. Its reference arm times the CPU
restatement of the reference's algorithm (one full shot per step) and runs
without a GPU; under torchrun only rank 0 runs it and prints, the other
ranks exit 0 without work. The GPU arm refuses to run without a GPU instead
of falling back to anything on the CPU. Each reference-arm run here times
one full C2 shot on the host cores (tens of seconds on a small machine).
"""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _env():
    env = dict(os.environ)
    env["CUDA_VISIBLE_DEVICES"] = ""  # no device, even where one exists
    return env


def _json_lines(text):
    return [json.loads(l) for l in text.splitlines() if l.startswith("{")]


def _check_reference_line(d, n_gpus):
    assert d["impl"] == "reference"
    assert d["unit"] == "shots/s" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["n_gpus"] == n_gpus and d["steps"] == 1 and d["warmup"] == 0
    assert d["config"]["grid"] == [681, 141] and d["config"]["shots"] == 16 and d["config"]["nt"] == 4000
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert d["vs_baseline"] is None and d["dtype"] == "f32"


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"],
                       cwd=ROOT, env=_env(), capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1
    _check_reference_line(lines[0], 1)
    # without a device the reference kernels' GPU leg says why it did not run
    assert "unavailable" in lines[0]["reference_gpu"]


def test_reference_arm_under_two_ranks_prints_once():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port),
           "bench.py", "--gpus", "2", "--impl", "reference", "--steps", "1", "--warmup", "0", "--no-ref-gpu"]
    r = subprocess.run(cmd, cwd=ROOT, env=_env(), capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1  # rank 0 alone
    _check_reference_line(lines[0], 2)
    assert "reference_gpu" not in lines[0]


def test_gpu_arm_fails_loudly_without_a_gpu():
    r = subprocess.run([sys.executable, "bench.py", "--steps", "1", "--warmup", "0"], cwd=ROOT, env=_env(),
                       capture_output=True, text=True, timeout=300)
    assert r.returncode != 0
    assert _json_lines(r.stdout) == []
    assert "no CUDA device" in r.stderr
