"""Generates tests/golden/golden.json by running the reference program itself.

The reference (githubofzby/beam) is compiled from its own sources into
oracle/_ref/beam_ref by `make -C oracle ref` (needs the sources under
the directory named by BEAM_REFERENCE_DIR, present only where the fixtures
are made). Each case is a
graph (a generator spec of beam_gb300's seeded generators, or an explicit
edge list) plus reference flags; the fixture keeps the reference's metric
lines that the GB300 path must reproduce, the SHA-256 of its G.txt, P.txt,
Cp.txt and Cm.txt, and a checksum of the input edge list so a generator that
drifts across machines is caught.

Usage: python tests/golden/make_golden.py [--only NAME ...]
"""

from __future__ import annotations

import argparse
import hashlib
import json
import os
import subprocess
import sys
import tempfile
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from beam_gb300 import REFERENCE_FLAGS, WORKLOADS, Graph  # noqa: E402

REF_BIN = ROOT / "oracle" / "_ref" / "beam_ref"
OUT = Path(__file__).resolve().parent / "golden.json"

KEEP_METRICS = [
    "n", "input_edges_raw", "graph_arcs", "partition_hash", "exact_partition_cost", "supernode_count", "P", "Cp",
    "Cm", "num_superedges_loop", "num_superedges_nonloop", "encoding_cost_mags_x2", "cost_ratio_mags_compatible",
    "divide_max_group_size", "divide_fallback_splits", "merge_group_count", "merge_group_max_size",
    "merge_raw_pair_count", "merge_candidate_pairs_after_prune", "merge_exact_gain_calls",
    "merge_positive_gain_pairs", "merge_rejected_by_threshold", "merge_rejected_by_overlap",
    "merge_candidate_pairs", "merge_selected_pairs", "merge_total_local_gain", "isolated_gain_sum",
    "selected_merges_for_validation", "accepted_merges_after_validation", "rejected_nonpositive",
    "validation_exact_calls", "validation_exact_row_entry_work", "update_touched_quotient_entries",
    "quotient_nnz_final", "exact_raw_entries_a", "exact_raw_entries_b", "exact_union_neighbors",
    "exact_overlap_neighbors", "candidate_proxy_pairs_examined", "exact_gain_input_nnz", "runtime_run_ms",
]

HAND = {
    "two_triangles_bridge": [(0, 1), (1, 2), (2, 0), (3, 4), (4, 5), (5, 3), (2, 3), (5, 6)],
    "star9": [(0, i) for i in range(1, 10)],
    "path12": [(i, i + 1) for i in range(11)],
    "clique7": [(i, j) for i in range(7) for j in range(i + 1, 7)],
    "two_cliques_bridge": [(i, j) for i in range(6) for j in range(i + 1, 6)]
    + [(i, j) for i in range(6, 12) for j in range(i + 1, 12)] + [(5, 6)],
    "k4_4": [(i, j) for i in range(4) for j in range(4, 8)],
    "single_edge": [(0, 1)],
    "isolated_ids": [(0, 5), (5, 9), (9, 2), (2, 0)],
    "twins_and_hub": [(0, j) for j in range(10, 20)] + [(1, j) for j in range(10, 20)]
    + [(2, j) for j in range(10, 19)] + [(3, j) for j in range(12, 20)] + [(4, 5), (5, 6), (6, 4)],
}

ERROR_CASES = {
    # the reference aborts with this message (thrown inside an OpenMP region)
    "duplicate_edge": ([(0, 1), (0, 1), (1, 2), (2, 0)], "edge count exceeds block capacity"),
}


def flags_with(**over) -> list[str]:
    # --profiling summary fills the work counters (exact_raw_entries_*, ...);
    # it does not change any decision
    f = list(REFERENCE_FLAGS) + ["--profiling", "summary"]
    drop = {k for k, v in over.items() if v is None}
    out = []
    i = 0
    while i < len(f):
        key = f[i].lstrip("-").replace("-", "_")
        takes_value = i + 1 < len(f) and not f[i + 1].startswith("--")
        if key in over:
            if key not in drop:
                out.append(f[i])
                if takes_value:
                    out.append(str(over[key]))
            i += 2 if takes_value else 1
            continue
        out.append(f[i])
        if takes_value:
            out.append(f[i + 1])
        i += 2 if takes_value else 1
    return out


CASES = []
for name, edges in HAND.items():
    CASES.append({"name": name, "edges": edges, "flags": flags_with()})
for seed in range(1, 7):
    CASES.append({"name": f"gnm_sparse_s{seed}", "spec": f"gnm:n=80,m=220,seed={seed}", "flags": flags_with()})
for seed in range(1, 4):
    CASES.append({"name": f"gnm_dense_s{seed}", "spec": f"gnm:n=40,m=520,seed={seed}", "flags": flags_with()})
CASES += [
    {"name": "grid40", "spec": "grid:side=40,del=0.1,diag=0.02,seed=2", "flags": flags_with()},
    {"name": "rmat12", "spec": "rmat:scale=12,ef=4,a=0.57,b=0.19,c=0.19,seed=3", "flags": flags_with()},
    {"name": "rmat14", "spec": "rmat:scale=14,ef=2,a=0.57,b=0.19,c=0.19,seed=5", "flags": flags_with()},
    {"name": "chunglu_twins_20k", "spec": "chunglu:n=20000,gamma=2.3,deg=8,twins=1500,seed=5",
     "flags": flags_with()},
    {"name": "dcsbm_4096", "spec": WORKLOADS["dcsbm_4096"], "flags": flags_with()},
    {"name": "rmat12_topk4", "spec": "rmat:scale=12,ef=4,a=0.57,b=0.19,c=0.19,seed=3",
     "flags": flags_with(top_k=4)},
    {"name": "rmat12_batch1", "spec": "rmat:scale=12,ef=4,a=0.57,b=0.19,c=0.19,seed=3",
     "flags": flags_with(group_batch_size=1)},
    {"name": "rmat12_batch7", "spec": "rmat:scale=12,ef=4,a=0.57,b=0.19,c=0.19,seed=3",
     "flags": flags_with(group_batch_size=7)},
    {"name": "rmat12_maxgroup8", "spec": "rmat:scale=12,ef=4,a=0.57,b=0.19,c=0.19,seed=3",
     "flags": flags_with() + ["--divide-max-group", "8"]},
    {"name": "rmat12_fallback", "spec": "rmat:scale=12,ef=4,a=0.57,b=0.19,c=0.19,seed=3",
     "flags": flags_with() + ["--divide-hash-dims", "2", "--divide-max-group", "16"]},
    {"name": "rmat12_nothreshold", "spec": "rmat:scale=12,ef=4,a=0.57,b=0.19,c=0.19,seed=3",
     "flags": flags_with(ea_use_threshold=None)},
    {"name": "rmat12_seed42_it5", "spec": "rmat:scale=12,ef=4,a=0.57,b=0.19,c=0.19,seed=3",
     "flags": flags_with(seed=42, iterations=5)},
    {"name": "dcsbm_topk32_maxgroup1024", "spec": WORKLOADS["dcsbm_4096"],
     "flags": flags_with(top_k=32) + ["--divide-max-group", "1024"]},
    # the non-blocked batch-ea mode (group by group)
    {"name": "rmat12_batchea", "spec": "rmat:scale=12,ef=4,a=0.57,b=0.19,c=0.19,seed=3",
     "flags": flags_with(merge_mode="batch-ea")},
    {"name": "gnm_sparse_s2_batchea", "spec": "gnm:n=80,m=220,seed=2", "flags": flags_with(merge_mode="batch-ea")},
    {"name": "rmat19", "spec": WORKLOADS["rmat19"], "flags": flags_with(), "large": True},
    # the batched form: one block holding every group of an iteration
    {"name": "rmat19_batched", "spec": WORKLOADS["rmat19"], "flags": flags_with(group_batch_size=1 << 30),
     "large": True},
    {"name": "union_batched", "spec": WORKLOADS["grid_chunglu_union"], "flags": flags_with(group_batch_size=1 << 30),
     "large": True, "huge": True},
    # the plain form (64-group blocks) of the grid + Chung-Lu union
    {"name": "union_plain", "spec": WORKLOADS["grid_chunglu_union"], "flags": flags_with(), "large": True,
     "huge": True},
    # the 4M-node Chung-Lu graph with 200k planted twin groups, first 5 iterations
    {"name": "chunglu4m_twins_it5", "spec": WORKLOADS["chunglu4m_twins"], "flags": flags_with(iterations=5),
     "large": True, "huge": True},
    # R-MAT scale 24, edge factor 16: the large single-GPU run, plain form
    {"name": "rmat24", "spec": WORKLOADS["rmat24"], "flags": flags_with(), "large": True, "huge": True},
]


def edge_text(edges) -> str:
    return "".join(f"{u} {v}\n" for u, v in edges)


def file_checksum(path: Path) -> str:
    h = hashlib.sha256()
    with open(path, "rb") as f:
        for block in iter(lambda: f.read(1 << 24), b""):
            h.update(block)
    return h.hexdigest()


def run_reference(graph: Path, flags: list[str], tmp: Path, threads: int) -> tuple[dict, dict, str]:
    out = tmp / "out"
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    proc = subprocess.run([str(REF_BIN), "--input", str(graph), *flags, "--write-output", "--out", str(out)],
                          capture_output=True, text=True, env=env)
    metrics = {}
    for line in proc.stdout.splitlines():
        if line.startswith("metric."):
            k, v = line[len("metric."):].split("=", 1)
            if k in KEEP_METRICS:
                metrics[k] = v
    hashes = {}
    if proc.returncode == 0:
        for f in ("G.txt", "P.txt", "Cp.txt", "Cm.txt"):
            hashes[f] = file_checksum(out / f)
    return metrics, hashes, proc.stdout + proc.stderr


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", nargs="*")
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1, help="OpenMP threads of the reference")
    args = ap.parse_args()
    if not REF_BIN.exists():
        subprocess.run(["make", "-C", str(ROOT / "oracle"), "ref"], check=True)
    old = json.loads(OUT.read_text()) if OUT.exists() else {"cases": [], "errors": []}
    keep = {c["name"]: c for c in old.get("cases", [])}
    for case in CASES:
        if args.only and case["name"] not in args.only:
            continue
        with tempfile.TemporaryDirectory() as td:
            graph = Path(td) / "graph.txt"
            if "spec" in case:
                # the library's writer prints the generated edge list as "u v" lines
                Graph.generate(case["spec"]).write_text(graph)
            else:
                graph.write_text(edge_text(case["edges"]))
            checksum = file_checksum(graph)
            metrics, hashes, log = run_reference(graph, case["flags"], Path(td), args.threads)
        if not hashes:
            raise RuntimeError(f"reference failed on {case['name']}:\n{log}")
        entry = {k: case[k] for k in ("name", "flags") }
        if "spec" in case:
            entry["spec"] = case["spec"]
        else:
            entry["edges"] = case["edges"]
        entry["large"] = bool(case.get("large"))
        entry["huge"] = bool(case.get("huge"))  # too slow for the CPU oracle in the CPU suite
        entry["graph_sha256"] = checksum
        entry["metrics"] = metrics
        entry["files_sha256"] = hashes
        keep[case["name"]] = entry
        print(f"{case['name']}: hash={metrics.get('partition_hash')} run_ms={metrics.get('runtime_run_ms')}")
    errors = []
    for name, (edges, message) in ERROR_CASES.items():
        with tempfile.TemporaryDirectory() as td:
            graph = Path(td) / "graph.txt"
            graph.write_text(edge_text(edges))
            metrics, hashes, log = run_reference(graph, flags_with(), Path(td), args.threads)
        assert not hashes and message in log, log
        errors.append({"name": name, "edges": edges, "message": message})
    order = [c["name"] for c in CASES]
    cases = sorted(keep.values(), key=lambda c: order.index(c["name"]) if c["name"] in order else 1 << 30)
    OUT.write_text(json.dumps({
        "generator": "tests/golden/make_golden.py",
        "reference": "githubofzby/beam, compiled from its sources by `make -C oracle ref`",
        "cases": cases, "errors": errors}, indent=1) + "\n")


if __name__ == "__main__":
    main()
