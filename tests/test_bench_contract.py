"""The benchmark's reporting contract, checked on the CPU: the reference arm
prints one JSON line with the required keys, the roofline's DRAM traffic is
read from the committed ncu summary, and every committed ncu command leaves
the GPU clocks alone."""

import json
import re
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload", "dcsbm_4096",
                          "--steps", "1", "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "dtype", "config", "impl", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["warmup"] >= 3
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["e2e"]["value"] == d["value"]


def test_roofline_traffic_from_committed_summary():
    sys.path.insert(0, str(ROOT))
    import bench
    traffic = bench.profiled_traffic("score", "rmat24", "ranker")
    text = (ROOT / "profiles" / "ScoreKernel_rmat24_ranker_dram.md").read_text()
    m = re.search(r"traffic_bytes_per_launch:\s*(\d+)", text)
    assert m and traffic == float(m.group(1)) and traffic > 0


def test_ncu_commands_keep_clocks():
    for p in sorted((ROOT / "profiles").glob("*.md")):
        cmds = [l for l in p.read_text().splitlines() if l.startswith("ncu ")]
        assert cmds, p.name
        for c in cmds:
            assert "--clock-control none" in c, (p.name, c)


def test_plain_form_is_bounded():
    """The plain form runs in a child process bounded by the bench's time
    budget: with no budget left it is not started, and a child that cannot
    finish (here: no GPU in the process, or a GPU run) is reported with
    `complete` set accordingly, never as a 20-iteration time it did not
    measure."""
    import types
    sys.path.insert(0, str(ROOT))
    import bench
    args = types.SimpleNamespace(workload="dcsbm_4096")
    r = bench.plain_form(args, 0, 30.0)
    assert r["complete"] is False and r["wall_s_20iter"] is None and "time budget" in r["note"]
    r = bench.plain_form(args, 0, 300.0)
    if r["complete"]:
        assert r["wall_s_20iter"] > 0 and r["partition_hash"]
    else:
        assert r["wall_s_20iter"] is None and r["note"]


def test_cpu_baseline_is_bounded():
    import types
    sys.path.insert(0, str(ROOT))
    import bench
    args = types.SimpleNamespace(workload="dcsbm_4096", cpu_sample_seconds=0.5)
    r = bench.cpu_baseline(args, timeout_s=0.01)
    assert r["value"] is None and "stopped after" in r["sample"]
