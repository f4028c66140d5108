"""The drop-in CLI end to end on the GPU: beam_gb300/bin/beam with the
reference's flags (--scoring-backend cuda) on fixtures made by the reference
program prints the same metric lines (partition hash, costs, every work
counter) and writes byte-identical G.txt / P.txt / Cp.txt / Cm.txt."""

import subprocess
from pathlib import Path

import pytest

from conftest import file_hashes, golden_cases

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
CLI = ROOT / "beam_gb300" / "bin" / "beam"
NAMES = ["clique7", "gnm_sparse_s3", "rmat12", "rmat12_batchea", "dcsbm_4096", "rmat12_nothreshold"]


def write_graph(case, path):
    from beam_gb300 import Graph
    if "spec" in case:
        Graph.generate(case["spec"]).write_text(str(path))
    else:
        path.write_text("".join(f"{u} {v}\n" for u, v in case["edges"]))


@pytest.mark.parametrize("case", [c for c in golden_cases() if c["name"] in NAMES], ids=lambda c: c["name"])
def test_cli_matches_reference(case, tmp_path):
    graph = tmp_path / "graph.txt"
    write_graph(case, graph)
    flags = list(case["flags"])
    flags[flags.index("--scoring-backend") + 1] = "cuda"
    out = tmp_path / "out"
    r = subprocess.run([str(CLI), "--input", str(graph), *flags, "--write-output", "--out", str(out)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    got = {}
    for line in r.stdout.splitlines():
        if line.startswith("metric."):
            k, v = line[len("metric."):].split("=", 1)
            got[k] = v
    want = case["metrics"]
    timing = {"runtime_run_ms"}
    diffs = {k: (want[k], got.get(k)) for k in want if k not in timing and want[k] != got.get(k)}
    assert not diffs, diffs
    assert file_hashes(out) == case["files_sha256"]
