"""Pins the oracle (the C restatement) to the reference program's own outputs
recorded in tests/golden/golden.json: partition hash, every recorded counter
and the SHA-256 of G.txt / P.txt / Cp.txt / Cm.txt must match exactly."""

import pytest

from conftest import file_hashes, golden_cases, graph_for, iterations_from_flags, options_from_flags
from oracle import Oracle

EXACT = ["n", "partition_hash", "exact_partition_cost", "supernode_count", "P", "Cp", "Cm", "num_superedges_loop",
         "num_superedges_nonloop", "encoding_cost_mags_x2", "cost_ratio_mags_compatible", "divide_max_group_size",
         "divide_fallback_splits", "merge_group_count", "merge_group_max_size", "merge_raw_pair_count",
         "merge_candidate_pairs_after_prune", "merge_exact_gain_calls", "merge_positive_gain_pairs",
         "merge_rejected_by_threshold", "merge_rejected_by_overlap", "merge_candidate_pairs",
         "merge_selected_pairs", "merge_total_local_gain", "isolated_gain_sum", "selected_merges_for_validation",
         "accepted_merges_after_validation", "rejected_nonpositive", "validation_exact_calls",
         "validation_exact_row_entry_work", "update_touched_quotient_entries", "quotient_nnz_final",
         "exact_raw_entries_a", "exact_raw_entries_b", "exact_union_neighbors", "exact_overlap_neighbors",
         "candidate_proxy_pairs_examined", "exact_gain_input_nnz"]


def oracle_metrics(o, enc):
    st = o.stats()
    m = {k: st[k] for k in st if k in EXACT}
    m.update(partition_hash=o.partition_hash(), exact_partition_cost=o.exact_partition_cost(),
             supernode_count=enc["n_supernodes"], P=enc["p"], Cp=enc["cp"], Cm=enc["cm"],
             num_superedges_loop=enc["num_superedges_loop"], num_superedges_nonloop=enc["num_superedges_nonloop"],
             encoding_cost_mags_x2=enc["encoding_cost_mags_x2"],
             cost_ratio_mags_compatible=f"{enc['cost_ratio_mags_compatible']:.6f}", n=o.n)
    return {k: str(v) for k, v in m.items()}


@pytest.mark.parametrize("case", golden_cases(include_huge=False), ids=lambda c: c["name"])
def test_oracle_matches_reference(case, tmp_path):
    g = graph_for(case)
    o = Oracle.from_graph(g, **options_from_flags(case["flags"]))
    o.run(iterations_from_flags(case["flags"]))
    enc = o.encode(tmp_path)
    got = oracle_metrics(o, enc)
    want = case["metrics"]
    diffs = {k: (want[k], got[k]) for k in EXACT if k in want and k in got and want[k] != got[k]}
    assert not diffs, diffs
    assert file_hashes(tmp_path) == case["files_sha256"]


def test_oracle_rejects_duplicate_edges(golden):
    from beam_gb300 import Graph
    case = golden["errors"][0]
    u, v = zip(*case["edges"])
    g = Graph.from_edges(list(u), list(v))
    o = Oracle.from_graph(g)
    with pytest.raises(RuntimeError):
        o.run(20)
