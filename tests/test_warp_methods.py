"""Warp-level search and reorder methods of the kernels, restated lane by
lane in Python and checked against plain results on the CPU:

- WarpLastLE (beam_gb300/csrc/merge.cu): the last index of a non-decreasing
  array at or below a value, found by the whole warp probing 32 points of the
  remaining span per round (the member pass finds each member's group with
  it); checked against bisect on random arrays, with the round count.
- SortMixedRunsKernel (beam_gb300/csrc/divide.cu): a run of keys sharing
  their high word reordered stably by the full key, one warp per run (a warp
  reduction picks the next smallest low word, a ballot compaction moves its
  items in order); checked against a stable sort, including low words of all
  ones.

The GPU tests run the kernels themselves (every golden fixture's groups and
partition hashes); these pin the methods' arguments on the CPU."""

import bisect
import random


def warp_last_le(a, lo, hi, x):
    rounds = 0
    while hi - lo > 1:
        probes = [lo + 1 + (((hi - lo - 1) * lane) >> 5) for lane in range(32)]
        assert all(lo < p <= hi - 1 for p in probes)
        k = sum(1 for p in probes if a[p] <= x)
        assert all((a[p] <= x) == (i < k) for i, p in enumerate(probes))  # lanes 0..k-1 hold
        p_lo, p_hi = probes[k - 1 if k > 0 else 0], probes[k if k < 32 else 31]
        if k > 0:
            lo = p_lo
        if k < 32:
            hi = p_hi
        rounds += 1
    return lo, rounds


def test_warp_last_le_matches_bisect():
    rng = random.Random(1)
    worst = 0
    for trial in range(1500):
        n = rng.randint(1, 40000 if trial % 10 == 0 else 2000)
        a = sorted(rng.randint(0, 10 * n) for _ in range(n))
        lo = rng.randint(0, n - 1)
        hi = rng.randint(lo + 1, n)
        x = rng.randint(a[lo], a[hi - 1] + 5)
        got, rounds = warp_last_le(a, lo, hi, x)
        assert got == bisect.bisect_right(a, x, lo, hi) - 1
        worst = max(worst, rounds)
    assert worst <= 4  # log32 of spans up to 40,000


def reorder_run(keys, vals, r0, end):
    """One warp's work on the run starting at r0 (items before end)."""
    hi = keys[r0] >> 32
    r1 = r0 + 1
    while True:
        inside = [r1 + lane < end and (keys[r1 + lane] >> 32) == hi for lane in range(32)]
        if not all(inside):
            r1 += inside.index(False)
            break
        r1 += 32
    tk, tv = {}, {}
    w, last, moved = r0, 0, False
    while w < r1:
        cands = [k & 0xffffffff for k in keys[r0:r1] if not moved or (k & 0xffffffff) > last]
        if not cands:
            break
        mn = min(cands)  # the warp reduction
        for i0 in range(r0, r1, 32):  # ballot compaction, 32 items at a time
            for i in range(i0, min(i0 + 32, r1)):
                if (keys[i] & 0xffffffff) == mn:
                    tk[w], tv[w] = keys[i], vals[i]
                    w += 1
        last, moved = mn, True
    for i in range(r0, r1):
        keys[i], vals[i] = tk[i], tv[i]
    return r1


def test_mixed_run_reorder_is_a_stable_sort():
    rng = random.Random(3)
    for _ in range(1500):
        length = rng.randint(2, 300)
        hi = rng.randint(0, 5)
        lows = [rng.choice([0, 5, 0xffffffff, 7, 123456]) for _ in range(length)]
        before = [((hi + 1) << 32) | 9] * rng.randint(0, 3)
        run = [(hi << 32) | lo for lo in lows]
        after = [(hi + 2) << 32] * rng.randint(0, 40)
        keys = before + run + after
        vals = list(range(len(keys)))
        r0 = len(before)
        end = len(keys) - rng.randint(0, len(after))
        want = sorted(zip(run, range(r0, r0 + length)), key=lambda kv: kv[0])
        assert reorder_run(keys, vals, r0, end) == r0 + length
        assert list(zip(keys[r0:r0 + length], vals[r0:r0 + length])) == want
