"""Generates tests/golden/legacy_gain.json: golden vectors of the reference's
legacy-objective pair scoring over a flat per-block CSR (Sweg::FlatAggCSR).

The values come from the reference's own host-side check of its CUDA scoring
backend (ComputeLocalGainHostFromFlat, src/cuda_scoring.cu:146-252), compiled
from the reference's sources into oracle/_ref/libref_legacy.so by
`make -C oracle ref-legacy` (needs the reference checkout, BEAM_REFERENCE_DIR).

Blocks are seeded random flat CSRs that exercise every branch of the
objective: rows listing their own representative (self-loop counts
subtracted), rows listing the other row's representative (the merged
internal block), rows listing neither, empty rows, dense blocks whose
complement is cheaper, and sizes large enough for 40-bit capacities.

Usage: python tests/golden/make_legacy_golden.py
"""

from __future__ import annotations

import ctypes as C
import json
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
LIB = ROOT / "oracle" / "_ref" / "libref_legacy.so"
OUT = Path(__file__).resolve().parent / "legacy_gain.json"


def random_block(rng: np.random.Generator, rows: int, max_deg: int, max_size: int, dense: bool,
                 twins: bool = False) -> dict:
    pool = rng.choice(5000, size=rows + 3 * max_deg, replace=False).astype(np.int64)
    reps = pool[:rows]
    shared = rng.choice(pool[rows:], size=max_deg, replace=False).tolist()
    size_of = {int(r): int(rng.integers(1, max_size + 1)) for r in pool}
    offsets, nb, wt, nsz = [0], [], [], []
    rsz = [size_of[int(r)] for r in reps]
    self_loops = []
    for i, r in enumerate(reps.tolist()):
        deg = int(rng.integers(0, max_deg + 1)) if i % 7 else 0  # every 7th row is empty
        if twins:  # near-twin rows: 90% of one shared neighbour set each
            picks = {x for x in shared if rng.random() < 0.9}
        else:
            picks = set(rng.choice(pool, size=min(deg, len(pool)), replace=False).tolist())
        if rng.random() < 0.4:
            picks.add(r)  # the row lists its own representative
        if rng.random() < 0.5 and rows > 1:
            picks.add(int(reps[(i + 1) % rows]))  # a direct edge to another row
        sl = 0
        for x in sorted(picks):
            s, sx = size_of[r], size_of[x]
            cap = s * (s - 1) // 2 if x == r else s * sx
            if x == r:
                sl = int(rng.integers(0, max(1, cap // 4) + 1))
                e = int(rng.integers(0, cap + sl + 1))  # self-loop counts ride on top
            elif dense and cap > 0:
                e = int(rng.integers(max(1, cap // 2), cap + 1))
            elif twins:
                e = sx * s if rng.random() < 0.7 else int(rng.integers(1, cap + 1))
            else:
                e = int(rng.integers(1, max(1, min(cap, 40)) + 1)) if cap > 0 else 0
            nb.append(x)
            wt.append(e)
            nsz.append(sx)
        self_loops.append(sl)
        offsets.append(len(nb))
    return {"offsets": offsets, "reps": reps.tolist(), "rsz": rsz, "self": self_loops, "nb": nb, "wt": wt,
            "nsz": nsz}


def reference_gains(lib, block: dict, pairs: np.ndarray) -> tuple[list[int], list[int]]:
    f = {k: np.ascontiguousarray(v, np.int64 if k in ("rsz", "self", "wt", "nsz") else np.int32)
         for k, v in block.items()}
    pairs = np.ascontiguousarray(pairs, np.int32)
    gain = np.zeros(len(pairs), np.int64)
    before = np.zeros(len(pairs), np.int64)

    def p(a, t):
        return a.ctypes.data_as(C.POINTER(t))

    rc = lib.ref_legacy_flat_gains(p(f["offsets"], C.c_int32), p(f["reps"], C.c_int32), p(f["rsz"], C.c_int64),
                                   p(f["self"], C.c_int64), C.c_int32(len(f["reps"])), p(f["nb"], C.c_int32),
                                   p(f["wt"], C.c_int64), p(f["nsz"], C.c_int64), C.c_int64(len(f["nb"])),
                                   p(pairs, C.c_int32), C.c_int64(len(pairs)), p(gain, C.c_int64),
                                   p(before, C.c_int64))
    assert rc == 0
    return gain.tolist(), before.tolist()


def main() -> None:
    if not LIB.exists():
        subprocess.run(["make", "-C", str(ROOT / "oracle"), "ref-legacy"], check=True)
    lib = C.CDLL(str(LIB))
    lib.ref_legacy_flat_gains.restype = C.c_int
    rng = np.random.default_rng(20261204)
    # (rows, max degree, max size, kind: True = dense blocks, "twins" = near-twin rows)
    settings = [
        (2, 6, 3, False), (5, 10, 4, False), (12, 20, 8, False), (12, 20, 8, True), (30, 40, 30, False),
        (24, 60, 1000, True), (40, 8, 1, False), (16, 30, 200000, True), (20, 12, 5, "twins"),
        (32, 40, 1, "twins"),
    ]
    blocks = []
    for rows, deg, size, kind in settings:
        block = random_block(rng, rows, deg, size, kind is True, twins=kind == "twins")
        all_pairs = [(a, b) for a in range(rows) for b in range(rows) if a != b]
        take = rng.choice(len(all_pairs), size=min(len(all_pairs), 300), replace=False)
        pairs = np.array([all_pairs[i] for i in sorted(take.tolist())], np.int32).reshape(-1, 2)
        gain, before = reference_gains(lib, block, pairs)
        blocks.append({**block, "pairs": pairs.tolist(), "gain": gain, "before": before})
    OUT.write_text(json.dumps({
        "generator": "tests/golden/make_legacy_golden.py",
        "reference": "githubofzby/beam ComputeLocalGainHostFromFlat (src/cuda_scoring.cu:146-252), compiled by "
                     "`make -C oracle ref-legacy`",
        "blocks": blocks}) + "\n")
    print(f"{len(blocks)} blocks, {sum(len(b['pairs']) for b in blocks)} pairs -> {OUT}")


if __name__ == "__main__":
    main()
