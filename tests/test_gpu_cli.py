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


def test_cli_csv_outputs_and_quotient_validation(tmp_path):
    """--results-csv and --profiling rounds --profile-csv append rows with the
    reference's schemas (src/main.cpp:1061-1178, 1197-1487); a second run
    appends under the same header; --validate-quotient checks the state after
    every iteration and changes no result."""
    import csv
    case = next(c for c in golden_cases() if c["name"] == "rmat12")
    graph = tmp_path / "data" / "graph.txt"
    graph.parent.mkdir()
    write_graph(case, graph)
    flags = list(case["flags"])
    flags[flags.index("--scoring-backend") + 1] = "cuda"
    flags[flags.index("--profiling") + 1] = "rounds"
    results, profile = tmp_path / "results.csv", tmp_path / "profile.csv"
    for _ in range(2):
        r = subprocess.run([str(CLI), "--input", str(graph), *flags, "--validate-quotient", "--results-csv",
                            str(results), "--profile-csv", str(profile)], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
        assert f"metric.partition_hash={case['metrics']['partition_hash']}" in r.stdout
        assert "metric.validate_quotient=true" in r.stdout
    rows = list(csv.DictReader(results.open()))
    assert len(rows) == 2 and len(rows[0]) == 146
    assert rows[0]["partition_hash"] == case["metrics"]["partition_hash"]
    assert rows[0]["accepted_merges_after_validation"] == case["metrics"]["accepted_merges_after_validation"]
    prof = list(csv.DictReader(profile.open()))
    assert len(prof) == 40 and len(prof[0]) == 70
    assert [int(p["iteration"]) for p in prof[:20]] == list(range(1, 21))
    assert prof[0]["dataset"] == "data"
    merges = sum(int(p["actual_merge_count"]) for p in prof[:20])
    assert merges == int(case["metrics"]["accepted_merges_after_validation"])
    assert sum(int(p["exact_gain_calls"]) for p in prof[:20]) == int(case["metrics"]["merge_exact_gain_calls"])
    # a file with another header is refused, as the reference refuses it
    bad = tmp_path / "bad.csv"
    bad.write_text("n,something_else\n")
    r = subprocess.run([str(CLI), "--input", str(graph), *flags, "--results-csv", str(bad)], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 1 and "header does not match" in r.stdout
