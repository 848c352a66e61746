"""bench.py's reference arm on the CPU: the FP64 oracle timed on a bounded
sample of the benchmark workload, one JSON line with the benchmark's keys.

Under torchrun with two ranks (gloo, 127.0.0.1) rank 0 alone runs and
prints; the other rank exits 0 without work.
"""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ARGS = ["--impl", "reference", "--steps", "1", "--warmup", "0", "--cpu-sample", "8"]


def _json_lines(out):
    return [json.loads(s) for s in out.splitlines() if s.startswith("{")]


def _check_line(line, n_gpus):
    assert line["impl"] == "reference"
    assert line["unit"] == "voxels/s" and line["value"] > 0
    assert line["n_gpus"] == n_gpus and line["steps"] == 1 and line["warmup"] == 0
    assert line["higher_is_better"] is True and line["vs_baseline"] is None
    # the same config as the library's headline line (bench.headline_config)
    sys.path.insert(0, ROOT)
    import bench
    assert line["config"] == bench.headline_config(bench.NVOX, n_gpus)
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert cb["sample"].startswith("8 voxels") and "plugin" in cb
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_one_process(built):
    r = subprocess.run([sys.executable, "bench.py", *ARGS], cwd=ROOT, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1, r.stdout
    _check_line(lines[0], 1)


def test_reference_arm_two_ranks(built):
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
                        "--nproc-per-node", "2", "--master-addr", "127.0.0.1",
                        "--master-port", str(port), "bench.py", "--gpus", "2", *ARGS],
                       cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1, r.stdout
    _check_line(lines[0], 2)
