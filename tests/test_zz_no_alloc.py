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


def flat_group(engine, q):
    """The reference's flat per-group CSR for members q, from the engine state."""
    sizes = {}

    def size_of(rep):
        if rep not in sizes:
            sizes[rep] = engine.row(int(rep))[2]
        return sizes[rep]

    offsets, nbs, wts, nbsz, rsz, rint = [0], [], [], [], [], []
    for rep in q:
        nb, cnt, size, internal = engine.row(int(rep))
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


def call_noalloc(f, top_k=16):
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
    if rc != 0:
        raise N.BeamError(N.lib().beam_prepare_flat_noalloc_last_error().decode())
    n = int(out_n.cpu().item())
    return np.stack([out_a[:n].cpu().numpy(), out_b[:n].cpu().numpy()], axis=1)


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
        flats = [flat_group(e, q) for q in groups]
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
