"""The library's host-side Encode / metrics (beam_encode,
beam_exact_partition_cost, beam_partition_hash) on partitions produced by the
oracle: byte-identical G.txt / P.txt / Cp.txt / Cm.txt and the same metrics
as the reference recorded in tests/golden/golden.json. No GPU needed."""

import pytest

from conftest import file_hashes, golden_cases, graph_for, iterations_from_flags, options_from_flags
from oracle import Oracle


@pytest.mark.parametrize("case", golden_cases(include_large=False), ids=lambda c: c["name"])
def test_host_encode_matches_reference(case, tmp_path):
    from beam_gb300 import partition_hash
    g = graph_for(case)
    o = Oracle.from_graph(g, **options_from_flags(case["flags"]))
    o.run(iterations_from_flags(case["flags"]))
    head, nxt = o.member_lists()
    labels = o.labels()
    enc = g.encode(head, nxt, tmp_path)
    m = case["metrics"]
    assert str(partition_hash(labels)) == m["partition_hash"]
    assert str(g.exact_partition_cost(labels)) == m["exact_partition_cost"]
    assert str(enc["supernodes"]) == m["supernode_count"]
    assert (str(enc["p"]), str(enc["cp"]), str(enc["cm"])) == (m["P"], m["Cp"], m["Cm"])
    assert str(enc["encoding_cost_mags_x2"]) == m["encoding_cost_mags_x2"]
    assert f"{enc['cost_ratio_mags_compatible']:.6f}" == m["cost_ratio_mags_compatible"]
    assert file_hashes(tmp_path) == case["files_sha256"]
