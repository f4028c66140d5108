"""Properties the reference's missing tests checked (experiments.md C1/C2),
re-created on the oracle with independent Python restatements:
  - the local integer merge gain equals the change of the global exact cost
    for every legal merge on random small graphs and partitions
  - the incrementally maintained quotient rows equal a full rebuild from the
    partition after random merge sequences
  - the summary (G, P, Cp, Cm) reconstructs the input graph losslessly
"""

from collections import Counter
from pathlib import Path

import numpy as np
import pytest

from conftest import golden_cases, graph_for, options_from_flags
from oracle import Oracle


def block_cost(sa, sb, e, internal):
    cap = sa * (sa - 1) // 2 if internal else sa * sb
    assert 0 <= e <= cap
    return min(e, 1 + cap - e)


def partition_cost(edges, labels):
    sizes = Counter(labels)
    pairs = Counter()
    for u, v in edges:
        a, b = labels[u], labels[v]
        pairs[(min(a, b), max(a, b))] += 1
    return sum(block_cost(sizes[a], sizes[b], e, a == b) for (a, b), e in pairs.items())


def random_graph(seed, n=36, m=110):
    from beam_gb300 import Graph
    return Graph.generate(f"gnm:n={n},m={m},seed={seed}")


@pytest.mark.parametrize("seed", range(1, 26))
def test_local_gain_equals_global_cost_change(seed):
    g = random_graph(seed)
    u, v = g.edge_list()
    edges = list(zip(u.tolist(), v.tolist()))
    o = Oracle.from_graph(g)
    rng = np.random.default_rng(seed)
    for _ in range(8):  # a random partition through random merges
        act = np.unique(o.labels())
        a, b = rng.choice(act, 2, replace=False)
        o.merge_pair(int(a), int(b))
    labels = o.labels().tolist()
    base = partition_cost(edges, labels)
    assert base == o.exact_partition_cost()
    act = sorted(set(labels))
    for a in act:
        for b in act:
            if a >= b:
                continue
            gain, before = o.exact_gain(a, b)
            merged = [a if x == b else x for x in labels]
            assert gain == base - partition_cost(edges, merged), (a, b)
            assert before > 0


@pytest.mark.parametrize("seed", range(1, 11))
def test_incremental_rows_equal_rebuild(seed):
    g = random_graph(seed, n=60, m=240)
    u, v = g.edge_list()
    o = Oracle.from_graph(g)
    rng = np.random.default_rng(100 + seed)
    for step in range(40):
        act = np.unique(o.labels())
        if len(act) < 2:
            break
        a, b = rng.choice(act, 2, replace=False)
        o.merge_pair(int(a), int(b))
        labels = o.labels()
        rows = {}
        internal = Counter()
        for x, y in zip(u.tolist(), v.tolist()):
            la, lb = int(labels[x]), int(labels[y])
            if la == lb:
                internal[la] += 1
            else:
                rows.setdefault(la, Counter())[lb] += 1
                rows.setdefault(lb, Counter())[la] += 1
        for rep in np.unique(labels).tolist():
            nb, cnt = o.row(rep)
            want = sorted(rows.get(rep, {}).items())
            assert list(zip(nb.tolist(), cnt.tolist())) == want, (step, rep)
            assert o.internal(rep) == internal[rep]
            assert o.size(rep) == int((labels == rep).sum())


def reconstruct(out_dir: Path):
    """Edge set encoded by G.txt / P.txt / Cp.txt / Cm.txt (mags-compatible:
    each undirected edge once, internal pairs u < v)."""
    members = {}
    for line in (out_dir / "G.txt").read_text().splitlines():
        parts = [int(x) for x in line.split("\t")]
        members[parts[0]] = parts[1:]
    edges = set()
    for line in (out_dir / "P.txt").read_text().splitlines():
        a, b = (int(x) for x in line.split("\t"))
        for x in members[a]:
            for y in members[b]:
                if a == b and x >= y:
                    continue
                edges.add((min(x, y), max(x, y)))
    for line in (out_dir / "Cm.txt").read_text().splitlines():
        x, y = (int(t) for t in line.split("\t"))
        edges.remove((min(x, y), max(x, y)))
    for line in (out_dir / "Cp.txt").read_text().splitlines():
        x, y = (int(t) for t in line.split("\t"))
        key = (min(x, y), max(x, y))
        assert key not in edges
        edges.add(key)
    return edges


@pytest.mark.parametrize("case", [c for c in golden_cases(include_large=False)
                                  if c["name"] in ("two_triangles_bridge", "clique7", "two_cliques_bridge", "k4_4",
                                                   "twins_and_hub", "gnm_dense_s1", "gnm_dense_s2", "grid40",
                                                   "rmat12", "dcsbm_4096")], ids=lambda c: c["name"])
def test_summary_is_lossless(case, tmp_path):
    g = graph_for(case)
    o = Oracle.from_graph(g, **options_from_flags(case["flags"]))
    o.run(20)
    o.encode(tmp_path)
    u, v = g.edge_list()
    want = {(min(a, b), max(a, b)) for a, b in zip(u.tolist(), v.tolist())}
    assert reconstruct(tmp_path) == want


def test_merge_blocks_resume_at_block_boundaries():
    """The bounded timing sample (Merge's blocks from a block boundary, until a
    time budget runs out) ends at a block boundary, and samples that resume
    where the last one ended give the whole Merge."""
    from beam_gb300 import Graph
    g = Graph.generate("rmat:scale=12,ef=4,a=0.57,b=0.19,c=0.19,seed=3")
    full = Oracle.from_graph(g, threads=2, group_batch_size=8)
    part = Oracle.from_graph(g, threads=2, group_batch_size=8)
    full.divide(1)
    full.merge(1)
    part.divide(1)
    ngroups = len(part.groups()[1])
    at, steps = 0, 0
    while at < ngroups:
        nxt = part.merge_blocks(1, at, 1e-9)  # the budget is spent after one block
        assert nxt == min(at + 8, ngroups)
        at, steps = nxt, steps + 1
    assert steps == (ngroups + 7) // 8
    assert part.partition_hash() == full.partition_hash()
    assert part.stats()["accepted_merges_after_validation"] == full.stats()["accepted_merges_after_validation"]
    with pytest.raises(RuntimeError, match="block boundary"):
        part.merge_blocks(1, 3, 0.0)
    for o in (full, part):
        o.close()
