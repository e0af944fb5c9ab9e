"""bench.py's reference arm on the CPU: one JSON line with the keys the measurement
contract names (impl, metric, value, unit, the step counts, cpu_baseline with its kind,
cores and sample, and an e2e object that moves no bytes), on the smallest configured
workload so that it runs in seconds."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "bcc16k", "--steps", "1",
                          "--warmup", "0", "--no-mc"], cwd=ROOT, check=True, capture_output=True, text=True,
                         timeout=600).stdout
    lines = [ln for ln in out.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "LLG atom-steps/s" and d["unit"] == "atom-steps/s"
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["n_gpus"] == 1 and d["steps"] == 1
    assert d["warmup"] >= 3  # at least three warm-up steps whatever was asked
    assert d["higher_is_better"] is True and d["scaling"] in ("weak", "strong")
    assert d["config"]["workload"] == "bcc16k"
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_under_torchrun_prints_once():
    """Launched as the multi-GPU runs are (torchrun, two ranks on 127.0.0.1), rank 0
    alone runs the reference arm and prints its line; the other rank exits 0."""
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    out = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                          "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
                          "--gpus", "2", "--workload", "bcc16k", "--steps", "1", "--warmup", "0", "--no-mc"],
                         cwd=ROOT, check=True, capture_output=True, text=True, timeout=600).stdout
    lines = [ln for ln in out.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    assert json.loads(lines[0])["impl"] == "reference"
