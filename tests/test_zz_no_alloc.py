"""The allocation-free prepare entry point (beam_prepare_flat_noalloc) against
the engine's own prepare entry point (beam_engine_prepare_group) on the same
groups, through the C ABI: identical candidate pairs (integer work, exact),
on consecutive calls that reuse the same static scratch array.

It serves callers that cannot allocate device memory; the test owns every
device buffer it passes (allocated here with torch) and the library
allocates nothing for the call.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def engine_rows(engine):
    """(neighbours, counts, size, internal) of a rep from the engine state."""
    return engine.row


def oracle_rows(oracle):
    """(neighbours, counts, size, internal) of a rep from the oracle state."""
    def row(rep):
        nb, cnt = oracle.row(rep)
        return nb, cnt, oracle.size(rep), oracle.internal(rep)
    return row


def flat_group(row_of, q):
    """The reference's flat per-group CSR (Sweg::FlatAggCSR) for members q."""
    sizes = {}

    def size_of(rep):
        if rep not in sizes:
            sizes[rep] = row_of(int(rep))[2]
        return sizes[rep]

    offsets, nbs, wts, nbsz, rsz, rint = [0], [], [], [], [], []
    for rep in q:
        nb, cnt, size, internal = row_of(int(rep))
        nbs += nb.tolist()
        wts += cnt.tolist()
        nbsz += [size_of(t) for t in nb.tolist()]
        rsz.append(size)
        rint.append(internal)
        offsets.append(len(nbs))
    return {
        "offsets": np.array(offsets, np.int32), "reps": np.array(q, np.int32), "nb": np.array(nbs, np.int32),
        "wt": np.array(wts, np.int64), "nbsz": np.array(nbsz, np.int64), "rsz": np.array(rsz, np.int64),
        "rint": np.array(rint, np.int64),
    }


def call_raw(f, top_k=16):
    """One call through the C ABI: (status, pairs, *out_count, error text)."""
    import torch

    from beam_gb300 import _native as N
    dev = {k: torch.from_numpy(v.copy()).cuda() if len(v) else torch.zeros(1, dtype=torch.from_numpy(v).dtype,
                                                                             device="cuda")
           for k, v in f.items()}
    g = len(f["reps"])
    cap = max(1, min(g * (g - 1) // 2, g * top_k))
    out_a = torch.full((cap,), -7, dtype=torch.int32, device="cuda")
    out_b = torch.full((cap,), -7, dtype=torch.int32, device="cuda")
    out_n = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = N.lib().beam_prepare_flat_noalloc(
        dev["offsets"].data_ptr(), dev["reps"].data_ptr(), dev["nb"].data_ptr(), dev["wt"].data_ptr(),
        dev["nbsz"].data_ptr(), dev["rsz"].data_ptr(), dev["rint"].data_ptr(), g, len(f["nb"]), top_k,
        out_a.data_ptr(), out_b.data_ptr(), cap, out_n.data_ptr(), C.c_void_p(stream))
    n = int(out_n.cpu().item())
    msg = N.lib().beam_prepare_flat_noalloc_last_error().decode() if rc != 0 else ""
    pairs = np.stack([out_a[:max(n, 0)].cpu().numpy(), out_b[:max(n, 0)].cpu().numpy()], axis=1)
    return rc, pairs, n, msg


def call_noalloc(f, top_k=16):
    from beam_gb300 import _native as N
    rc, pairs, _, msg = call_raw(f, top_k)
    if rc != 0:
        raise N.BeamError(msg)
    return pairs


def pick_groups(engine, want=3):
    order, starts, lengths = engine.groups()
    picked = []
    for s, ln in sorted(zip(starts.tolist(), lengths.tolist()), key=lambda x: -x[1]):
        if 2 <= ln <= 256:
            picked.append(order[s:s + ln].copy())
        if len(picked) == want:
            break
    return picked


def test_noalloc_prepare_matches_engine_prepare():
    from beam_gb300 import Engine, Graph
    g = Graph.generate("dcsbm:n=4096,blocks=32,ratio=40,gamma=2.5,deg=43,seed=1")
    with Engine(g) as e:
        e.divide(1)
        e.merge(1)
        e.divide(2)
        groups = pick_groups(e)
        assert len(groups) >= 2
        flats = [flat_group(engine_rows(e), q) for q in groups]
        # two calls in a row on different groups, then the first group again
        for q, f in list(zip(groups, flats)) + [(groups[0], flats[0])]:
            want = e.prepare_group(q)
            got = call_noalloc(f)
            assert len(want) > 0
            assert np.array_equal(got, want)


def test_noalloc_rejects_sizes_beyond_its_limits():
    from beam_gb300 import _native as N
    lib = N.lib()
    rc = lib.beam_prepare_flat_noalloc(None, None, None, None, None, None, None, 257, 0, 16, None, None, 0,
                                       None, None)
    assert rc != 0
    assert "exceeds the no-allocation limit of 256" in lib.beam_prepare_flat_noalloc_last_error().decode()
    rc = lib.beam_prepare_flat_noalloc(None, None, None, None, None, None, None, 4, 70000, 16, None, None, 0,
                                       None, None)
    assert rc != 0
    assert "row entries" in lib.beam_prepare_flat_noalloc_last_error().decode()
    rc = lib.beam_prepare_flat_noalloc(None, None, None, None, None, None, None, 4, 10, 64, None, None, 0,
                                       None, None)
    assert rc != 0
    assert "top_k" in lib.beam_prepare_flat_noalloc_last_error().decode()
    rc = lib.beam_prepare_flat_noalloc(None, None, None, None, None, None, None, 4, 10, 0, None, None, 0,
                                       None, None)
    assert rc != 0
    assert "top_k=0 must be at least 1" in lib.beam_prepare_flat_noalloc_last_error().decode()


def oracle_after_first_merge(top_k=16):
    """The oracle after Divide(1), Merge(1), Divide(2) of the SBM graph."""
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
    from oracle import Oracle  # checker only

    from beam_gb300 import Graph
    g = Graph.generate("dcsbm:n=4096,blocks=32,ratio=40,gamma=2.5,deg=43,seed=1")
    o = Oracle.from_graph(g, top_k=top_k)
    o.divide(1)
    o.merge(1)
    o.divide(2)
    return g, o


def test_noalloc_prepare_matches_oracle():
    """Against the oracle's prepare step directly: the largest Divide groups,
    and a small group whose size is at most top_k + 1 (every partner kept)."""
    _, o = oracle_after_first_merge()
    order, starts, lengths = o.groups()
    by_size = sorted(zip(starts.tolist(), lengths.tolist()), key=lambda x: -x[1])
    big = [order[s:s + ln].copy() for s, ln in by_size if 2 <= ln <= 256][:2]
    small = [order[s:s + ln].copy() for s, ln in by_size if 3 <= ln <= 8][:1]
    assert len(big) == 2 and len(small) == 1
    for q in big + small + big[:1]:
        want = o.prepare_group(q)
        got = call_noalloc(flat_group(oracle_rows(o), q))
        assert len(want) > 0
        assert np.array_equal(got, want)
    o.close()


@pytest.mark.parametrize("top_k", [16, 32])
def test_noalloc_group_at_the_size_limits(top_k):
    """256 members whose rows hold exactly 65,536 entries (both limits), against
    the oracle, on two calls in a row."""
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
    from oracle import Oracle  # checker only

    from beam_gb300 import Graph
    g = Graph.generate("rmat:scale=13,ef=16,seed=9")
    deg = np.diff(g.row_ptr)
    q, total = [], 0
    for v in np.argsort(-deg, kind="stable").tolist():
        if len(q) == 256:
            break
        if total + deg[v] <= 65536:
            q.append(v)
            total += int(deg[v])
    assert len(q) == 256 and total == 65536
    o = Oracle.from_graph(g, top_k=top_k)
    f = flat_group(oracle_rows(o), np.array(q, np.int32))
    assert len(f["nb"]) == total
    want = o.prepare_group(np.array(q, np.int32))
    for _ in range(2):
        got = call_noalloc(f, top_k=top_k)
        assert len(want) > 0
        assert np.array_equal(got, want)
    o.close()


def test_noalloc_reports_bad_inputs():
    """Bad offsets, repeated reps and weights outside [0, 2^32) fail with a
    message and *out_count = -1; a good call right after still succeeds."""
    _, o = oracle_after_first_merge()
    order, starts, lengths = o.groups()
    s, ln = max(zip(starts.tolist(), lengths.tolist()), key=lambda x: x[1])
    q = order[s:s + min(ln, 64)].copy()
    good = flat_group(oracle_rows(o), q)
    want = o.prepare_group(q) if len(q) == ln else None

    bad = {k: v.copy() for k, v in good.items()}
    bad["offsets"][1], bad["offsets"][2] = bad["offsets"][2], bad["offsets"][1] - 1
    rc, _, n, msg = call_raw(bad)
    assert rc != 0 and n == -1 and "offsets must rise" in msg

    bad = {k: v.copy() for k, v in good.items()}
    bad["reps"][1] = bad["reps"][0]
    rc, _, n, msg = call_raw(bad)
    assert rc != 0 and n == -1 and "row_rep_ids must be distinct" in msg

    for w in (1 << 32, -1):
        bad = {k: v.copy() for k, v in good.items()}
        bad["wt"][len(bad["wt"]) // 2] = w
        rc, _, n, msg = call_raw(bad)
        assert rc != 0 and n == -1 and "weights must lie in [0, 2^32)" in msg

    got = call_noalloc(good)
    assert len(got) > 0
    if want is not None:
        assert np.array_equal(got, want)
    o.close()


def test_noalloc_refuses_stream_capture():
    """On a capturing stream the call fails with a message and enqueues
    nothing (it reads its status back and waits for its stream); the capture
    stays valid, and a call after it succeeds."""
    import torch
    from beam_gb300 import _native as N
    _, o = oracle_after_first_merge()
    order, starts, lengths = o.groups()
    s, ln = max(zip(starts.tolist(), lengths.tolist()), key=lambda x: x[1])
    q = order[s:s + min(ln, 64)].copy()
    f = flat_group(oracle_rows(o), q)
    dev = {k: torch.from_numpy(v.copy()).cuda() for k, v in f.items()}
    g = len(f["reps"])
    cap = min(g * (g - 1) // 2, g * 16)
    out_a = torch.zeros(cap, dtype=torch.int32, device="cuda")
    out_b = torch.zeros(cap, dtype=torch.int32, device="cuda")
    out_n = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    stream = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        rc = N.lib().beam_prepare_flat_noalloc(
            dev["offsets"].data_ptr(), dev["reps"].data_ptr(), dev["nb"].data_ptr(), dev["wt"].data_ptr(),
            dev["nbsz"].data_ptr(), dev["rsz"].data_ptr(), dev["rint"].data_ptr(), g, len(f["nb"]), 16,
            out_a.data_ptr(), out_b.data_ptr(), cap, out_n.data_ptr(), C.c_void_p(stream.cuda_stream))
        out_n.fill_(5)
    msg = N.lib().beam_prepare_flat_noalloc_last_error().decode()
    assert rc != 0 and "cannot be captured" in msg
    graph.replay()
    torch.cuda.synchronize()
    assert int(out_n.item()) == 5
    rc, pairs, n, msg = call_raw(f)
    assert rc == 0 and n == len(pairs) and n > 0
    o.close()
