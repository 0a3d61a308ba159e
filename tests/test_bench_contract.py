"""The bench's JSON contract on the CPU: the reference arm's line (the CPU
restatement on the host cores) and the roofline's byte model for the
64-frame workload."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    """`bench.py --impl reference` prints one JSON line with the contract's
    keys, the reference marker, a CPU baseline describing the run and an e2e
    record without device copies."""
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"],
                       cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    if "unavailable" in d:
        pytest.skip(d["unavailable"])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["steps"] == 1 and d["warmup"] == 0 and d["n_gpus"] == 1
    assert d["unit"] == "frames/s" and d["higher_is_better"] is True and d["value"] > 0
    assert abs(d["value"] - 64 * 1e3 / d["ms_per_step"]) < 1e-6 * d["value"]
    assert "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_roofline_bytes_of_the_workload():
    """The path's byte model over the seeded 64-frame workload: the level
    terms (resize / blur / FAST) are 312.0 MB per step, about 9.3 W H per
    frame."""
    sys.path.insert(0, ROOT)
    import bench
    frames = bench.workload()
    stage, whole = bench.extraction_roofline_bytes(frames, [0] * len(frames))
    assert stage == whole == 311996778
    px = sum(img.shape[0] * img.shape[1] for img, _ in frames)
    assert 9.2 * px < stage < 9.4 * px
    _, whole = bench.extraction_roofline_bytes(frames, [1000] * len(frames))
    assert whole == stage + 60 * 64000


def test_reference_arm_under_torchrun_prints_once():
    """Launched as the driver launches N > 1 (torchrun, one process per
    rank), the reference arm runs on rank 0 alone: one JSON line in all, and
    every rank exits 0."""
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
                        "--gpus", "2", "--steps", "1", "--warmup", "0"],
                       cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d.get("impl") == "reference"
