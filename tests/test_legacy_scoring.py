"""Legacy-objective pair scoring over a flat per-block CSR (scope row f4: the
reference's Sweg::ScoreCandidatesCuda with --cost-objective legacy,
src/cuda_scoring.cu:714-885). Integer work: every {gain, before_cost} must be
exact.

Golden vectors (tests/golden/legacy_gain.json) come from the reference's own
host-side check of that backend (ComputeLocalGainHostFromFlat,
src/cuda_scoring.cu:146-252), compiled from its sources by
tests/golden/make_legacy_golden.py.
"""

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "oracle"))
from oracle import legacy_flat_gains  # noqa: E402  (checker only)

GOLDEN = json.loads((ROOT / "tests" / "golden" / "legacy_gain.json").read_text())["blocks"]


def test_oracle_matches_reference_golden_vectors():
    for b in GOLDEN:
        gain, before = legacy_flat_gains(b, b["pairs"])
        assert gain.tolist() == b["gain"]
        assert before.tolist() == b["before"]


def big_block(seed: int, rows: int = 400, hub_every: int = 50) -> dict:
    """A flat block with hub rows (thousands of entries) beside short rows,
    own-representative entries with self-loops and direct edges."""
    rng = np.random.default_rng(seed)
    reps = rng.choice(200000, size=rows, replace=False)
    pool = np.concatenate([reps, rng.choice(np.arange(200000, 400000), size=20000, replace=False)])
    size_of = {int(x): int(rng.integers(1, 50)) for x in pool.tolist()}
    offsets, nb, wt, nsz, rsz, self_loops = [0], [], [], [], [], []
    for i, r in enumerate(reps.tolist()):
        deg = 3000 if i % hub_every == 0 else int(rng.integers(0, 40))
        picks = set(rng.choice(pool, size=deg, replace=False).tolist())
        if i % 3 == 0:
            picks.add(r)
        sl = 0
        for x in sorted(picks):
            s, sx = size_of[r], size_of[x]
            cap = s * (s - 1) // 2 if x == r else s * sx
            if x == r:
                sl = int(rng.integers(0, cap // 3 + 1))
                e = int(rng.integers(0, cap + sl + 1))
            else:
                e = int(rng.integers(1, cap + 1))
            nb.append(x)
            wt.append(e)
            nsz.append(sx)
        rsz.append(size_of[r])
        self_loops.append(sl)
        offsets.append(len(nb))
    return {"offsets": offsets, "reps": reps.tolist(), "rsz": rsz, "self": self_loops, "nb": nb, "wt": wt,
            "nsz": nsz}


@pytest.mark.gpu
def test_gpu_matches_reference_golden_vectors():
    from beam_gb300 import FlatScorer
    with FlatScorer() as s:
        for b in GOLDEN:
            gain, before = s.score(b, b["pairs"])
            assert gain.tolist() == b["gain"]
            assert before.tolist() == b["before"]
        st = s.stats()
        assert st["calls"] == len(GOLDEN) and st["pairs"] == sum(len(b["pairs"]) for b in GOLDEN)


@pytest.mark.gpu
def test_gpu_matches_oracle_on_hub_blocks():
    """Hub rows of 3,000 entries against short and empty rows; two blocks in a
    row through one scorer (its buffers are reused and grown)."""
    from beam_gb300 import FlatScorer
    rng = np.random.default_rng(7)
    with FlatScorer() as s:
        for seed in (1, 2):
            b = big_block(seed)
            rows = len(b["reps"])
            pairs = rng.integers(0, rows, size=(20000, 2)).astype(np.int32)
            pairs = pairs[pairs[:, 0] != pairs[:, 1]]
            want_gain, want_before = legacy_flat_gains(b, pairs)
            gain, before = s.score(b, pairs)
            assert np.array_equal(gain, want_gain)
            assert np.array_equal(before, want_before)


@pytest.mark.gpu
def test_gpu_scorer_rejects_bad_layouts():
    from beam_gb300 import FlatScorer
    from beam_gb300._native import BeamError
    b = GOLDEN[2]
    with FlatScorer() as s:
        bad = dict(b, nb=list(b["nb"]))
        row = next(i for i in range(len(b["reps"])) if b["offsets"][i + 1] - b["offsets"][i] >= 2)
        k = b["offsets"][row]
        bad["nb"][k], bad["nb"][k + 1] = bad["nb"][k + 1], bad["nb"][k]
        with pytest.raises(BeamError, match="not sorted by neighbour"):
            s.score(bad, b["pairs"])
        with pytest.raises(BeamError, match="outside"):
            s.score(b, [[0, len(b["reps"])]])
        bad = dict(b, offsets=list(b["offsets"]))
        bad["offsets"][-1] += 1
        with pytest.raises(BeamError, match="offsets must rise"):
            s.score(bad, b["pairs"])
        gain, _ = s.score(b, b["pairs"])
        assert gain.tolist() == b["gain"]
