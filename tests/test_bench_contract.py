"""The benchmark's output contract, checked on the CPU through its reference
arm (`bench.py --impl reference`, which times the CPU restatement of the
probe update on the host cores and needs no GPU): one JSON line with the
metric, unit, configuration, the CPU-baseline record and an end-to-end
record; under torchrun with two ranks only rank 0 prints, the other exits
without work."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ARGS = ["--impl", "reference", "--steps", "1", "--warmup", "0", "--ref-probes", "16"]


def _lines(out):
    return [json.loads(s) for s in out.splitlines() if s.startswith("{")]


def _check_line(d, gpus):
    assert d["impl"] == "reference"
    assert d["metric"] and d["unit"] == "Grays/s"
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["n_gpus"] == gpus and d["steps"] == 1 and d["warmup"] == 0
    assert d["config"]["workload"] == "terrain_32x16x32_r256"
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, "bench.py"] + ARGS, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = _lines(r.stdout)
    assert len(lines) == 1, r.stdout[-2000:]
    _check_line(lines[0], 1)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_reference_arm_two_ranks_rank0_only():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--gpus", "2"] + ARGS
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = _lines(r.stdout)
    assert len(lines) == 1, r.stdout[-2000:]
    _check_line(lines[0], 2)


RANKS_SCRIPT = """
import os, sys
sys.path.insert(0, {root!r})
import torch.distributed as dist
import bench
dist.init_process_group("gloo")
r = dist.get_rank()
with open(os.path.join({out!r}, "rank%d.txt" % r), "w") as f:  # one file per rank: no interleaved output
    f.write("rank %d max %.3f single %.3f" % (r, bench.max_over_ranks(1.5 + r, "cpu"), 1.5 + r))
dist.destroy_process_group()
"""


def test_max_over_ranks_two_gloo_ranks(tmp_path):
    """The replicas' timing reduction (the slowest rank's time) over two
    gloo ranks on the CPU; without a process group it is the identity."""
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(3.25, "cpu") == 3.25
    script = tmp_path / "ranks.py"
    script.write_text(RANKS_SCRIPT.format(root=ROOT, out=str(tmp_path)))
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(_free_port()), str(script)]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]
    got = [(tmp_path / ("rank%d.txt" % k)).read_text() for k in range(2)]
    assert got == ["rank 0 max 2.500 single 1.500", "rank 1 max 2.500 single 2.500"], r.stdout
