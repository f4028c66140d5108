"""Stage-by-stage parity of the GPU kernels with the oracle on the same state:
Divide groups, EA-proxy candidates, exact merge gains and quotient-graph
maintenance after merge batches. Integer work: bit-exact."""

import numpy as np
import pytest

from oracle import Oracle

pytestmark = pytest.mark.gpu

SPECS = {
    "dcsbm": "dcsbm:n=4096,blocks=32,ratio=40,gamma=2.5,deg=43,seed=1",
    "rmat12": "rmat:scale=12,ef=4,a=0.57,b=0.19,c=0.19,seed=3",
    "chunglu_twins": "chunglu:n=20000,gamma=2.3,deg=8,twins=1500,seed=5",
}


def pair(spec, **kw):
    from beam_gb300 import Engine, Graph
    g = Graph.generate(spec)
    return g, Engine(g, **kw), Oracle.from_graph(g, **kw)


@pytest.mark.parametrize("name,kw", [("dcsbm", {}), ("rmat12", {}), ("rmat12", {"divide_max_group": 8}),
                                     ("rmat12", {"divide_hash_dims": 2, "divide_max_group": 16}),
                                     ("chunglu_twins", {})])
def test_divide_matches_oracle(name, kw):
    g, e, o = pair(SPECS[name], **kw)
    for it in range(1, 5):
        e.divide(it)
        o.divide(it)
        go, gs, gl = e.groups()
        oo, os_, ol = o.groups()
        assert np.array_equal(go, oo), f"group order differs at iteration {it}"
        assert np.array_equal(gs, os_) and np.array_equal(gl, ol)
        e.merge(it)
        o.merge(it)
    e.close()


@pytest.mark.parametrize("name", ["dcsbm", "rmat12", "chunglu_twins"])
def test_score_pairs_match_oracle(name):
    g, e, o = pair(SPECS[name])
    for it in (1, 2):
        e.divide(it)
        o.divide(it)
        e.merge(it)
        o.merge(it)
    labels = o.labels()
    active = np.unique(labels)
    rng = np.random.default_rng(7)
    a = rng.choice(active, 3000)
    b = rng.choice(active, 3000)
    keep = a != b
    a, b = a[keep], b[keep]
    # add adjacent pairs (shared neighbours and e(a,b) > 0)
    for rep in active[:300]:
        nb, _ = o.row(int(rep))
        if len(nb):
            a = np.append(a, rep)
            b = np.append(b, nb[0])
    gain, before = e.score_pairs(a, b)
    for i in range(len(a)):
        want = o.exact_gain(int(a[i]), int(b[i]))
        assert (int(gain[i]), int(before[i])) == want, (int(a[i]), int(b[i]))
    e.close()


@pytest.mark.parametrize("name", ["dcsbm", "rmat12", "chunglu_twins"])
def test_prepare_candidates_match_oracle(name):
    g, e, o = pair(SPECS[name])
    e.divide(1)
    o.divide(1)
    e.merge(1)
    o.merge(1)
    o.divide(2)
    order, starts, lengths = o.groups()
    checked = 0
    for s, ln in zip(starts, lengths):
        if ln < 2:
            continue
        q = order[s:s + ln]
        assert np.array_equal(e.prepare_group(q), o.prepare_group(q)), f"group at {s} of size {ln}"
        checked += 1
        if checked >= 400:
            break
    assert checked > 0
    e.close()


def compare_state(e, o, n):
    labels, head, nxt = e.partition()
    assert np.array_equal(labels, o.labels())
    oh, on = o.member_lists()
    assert np.array_equal(head, oh)
    act = head >= 0
    assert np.array_equal(nxt[act], on[act]) or np.array_equal(nxt, on)
    for rep in range(n):
        nb, cnt, size, internal = e.row(rep)
        if not o.active(rep):
            assert size == 0
            continue
        onb, ocnt = o.row(rep)
        assert size == o.size(rep) and internal == o.internal(rep), rep
        assert np.array_equal(nb, onb) and np.array_equal(cnt, ocnt), rep


@pytest.mark.parametrize("name", ["rmat12", "dcsbm"])
def test_merge_batches_match_oracle(name):
    g, e, o = pair(SPECS[name])
    rng = np.random.default_rng(3)
    for _ in range(6):
        active = np.unique(o.labels())
        rng.shuffle(active)
        k = len(active) // 5
        keep, rem = active[:k], active[k:2 * k]
        e.merge_pairs(keep, rem)
        for a, b in zip(keep, rem):
            o.merge_pair(int(a), int(b))
    compare_state(e, o, g.n)
    e.close()


def test_run_state_matches_oracle_each_iteration():
    g, e, o = pair(SPECS["rmat12"])
    for it in range(1, 6):
        e.divide(it)
        o.divide(it)
        e.merge(it)
        o.merge(it)
        compare_state(e, o, g.n)
    e.close()


def test_hub_rows_and_large_groups():
    """A hub adjacent to thousands of near-twins: rows longer than the
    shared-memory staging and groups whose bucket tables spill to scratch."""
    from beam_gb300 import Engine, Graph
    rng = np.random.default_rng(5)
    u, v = [], []
    hub_nb = np.arange(1, 6001)
    u += [0] * len(hub_nb)
    v += hub_nb.tolist()
    for t in range(6001, 6401):  # 400 nodes sharing most of 40 hub neighbours
        nbrs = rng.choice(np.arange(1, 41), 36, replace=False)
        u += [t] * len(nbrs)
        v += nbrs.tolist()
    for _ in range(6000):
        a, b = rng.integers(1, 6401, 2)
        if a != b:
            u.append(int(min(a, b)))
            v.append(int(max(a, b)))
    pairs = sorted({(min(a, b), max(a, b)) for a, b in zip(u, v)})  # each undirected edge once
    g = Graph.from_edges([p[0] for p in pairs], [p[1] for p in pairs])
    e = Engine(g)
    o = Oracle.from_graph(g)
    for it in range(1, 8):
        e.divide(it)
        o.divide(it)
        assert np.array_equal(e.groups()[0], o.groups()[0])
        e.merge(it)
        o.merge(it)
    compare_state(e, o, g.n)
    assert e.stats()["accepted_merges_after_validation"] == o.stats()["accepted_merges_after_validation"]
    e.close()


@pytest.mark.parametrize("name", ["rmat12", "dcsbm", "chunglu_twins"])
def test_batched_form_matches_oracle(name):
    """The batched form (one block of all groups per iteration) is the same
    algorithm with a larger block; the oracle with the same block size gives
    the same partition and counters."""
    from beam_gb300 import partition_hash
    batch = 1 << 30
    g, e, o = pair(SPECS[name], group_batch_size=batch)
    e.run(20)
    o.run(20)
    assert partition_hash(e.partition()[0]) == o.partition_hash()
    st, ost = e.stats(), o.stats()
    for k in ("accepted_merges_after_validation", "merge_exact_gain_calls", "candidate_proxy_pairs_examined",
              "update_touched_quotient_entries", "blocks"):
        if k in ost:
            assert st[k] == ost[k], k
    assert 1 <= st["blocks"] <= 20
    e.close()


@pytest.mark.parametrize("name,batch", [("chunglu_twins", 300), ("chunglu_twins", 1000), ("rmat12", 257)])
def test_multi_block_batched_form_matches_oracle(name, batch):
    """Blocks of a few hundred to a thousand groups (several per iteration, each
    scored from its own block-start row sums) against the oracle with the same
    block size: the same partition and counters."""
    from beam_gb300 import partition_hash
    g, e, o = pair(SPECS[name], group_batch_size=batch)
    e.run(20)
    o.run(20)
    assert partition_hash(e.partition()[0]) == o.partition_hash()
    st, ost = e.stats(), o.stats()
    for k in ("accepted_merges_after_validation", "merge_exact_gain_calls", "candidate_proxy_pairs_examined",
              "update_touched_quotient_entries", "exact_union_neighbors", "exact_overlap_neighbors"):
        assert st[k] == ost[k], k
    assert st["blocks"] > 20
    e.close()


@pytest.mark.parametrize("batch", [64, 1 << 30])
def test_validate_quotient_after_every_iteration(batch):
    """--validate-quotient: after every Merge the resident quotient graph equals
    a full rebuild from the labels (QuotientGraph::ValidateAgainstOriginalGraph,
    src/quotient_graph.cpp:867-886), in the plain and the batched forms."""
    from beam_gb300 import Engine, Graph
    for spec in ("rmat:scale=12,ef=4,a=0.57,b=0.19,c=0.19,seed=3", "dcsbm:n=4096,blocks=32,ratio=40,gamma=2.5,deg=43,seed=1"):
        g = Graph.generate(spec)
        with Engine(g, group_batch_size=batch) as e:
            e.validate_quotient()
            for it in range(1, 8):
                e.divide(it)
                e.merge(it, 20)
                e.validate_quotient()


def test_block_size_tuner_picks_a_size_within_the_bound():
    """beam_gb300.tune: the chosen block size keeps the cost ratio within the
    bound of the plain form's, and is the fastest such size of the ladder."""
    from beam_gb300 import Graph
    from beam_gb300.tune import tune_block_size
    g = Graph.generate(SPECS["chunglu_twins"])
    r = tune_block_size(g, bound=0.001, ladder=(1 << 30, 1024, 256))
    assert len(r["table"]) == 3
    assert abs(r["delta_vs_plain"]) <= 0.001
    ok = [t for t in r["table"] if t["within_bound"]]
    if ok:
        assert r["wall_s"] == min(t["wall_s"] for t in ok)
