"""Block-size tuner for the batched form.

The batched form scores and commits every group of a block against the
block-start state, so larger blocks run faster (fewer, wider launches) and see
staler states (a cost ratio further from the plain form's). The tuner times
the plain form once (the reference's 64-group blocks, bit-exact with the
reference), then the batched form at a ladder of block sizes from the largest
down, and picks the fastest block size whose 20-iteration cost ratio stays
within `bound` (absolute) of the plain form's.

    from beam_gb300 import Graph
    from beam_gb300.tune import tune_block_size
    best = tune_block_size(Graph.generate("..."))
    best["group_batch_size"], best["table"]
"""

from __future__ import annotations

import time

from .engine import Engine, Graph

# the ladder of block sizes in groups, largest first (1 << 30: one block of
# every group of an iteration)
LADDER = (1 << 30, 1 << 18, 1 << 16, 1 << 14, 1 << 12, 1 << 10, 1 << 8)


def _timed_run(g: Graph, iterations: int, device: int, **kw) -> dict:
    with Engine(g, device=device, ea_use_threshold=True, **kw) as e:
        e.run(iterations)  # warm-up: buffers sized, code paths loaded
        e.reset()
        e.step_timer_start()
        e.run(iterations)
        ms = e.step_timer_stop()
        enc = e.encode()
        merges = e.stats()["accepted_merges_after_validation"]
    return {"wall_s": ms / 1000.0, "cost_ratio": enc["cost_ratio_mags_compatible"], "merges": merges}


def tune_block_size(g: Graph, bound: float = 0.001, ladder=LADDER, iterations: int = 20, device: int = 0,
                    plain: dict | None = None) -> dict:
    """The fastest group_batch_size of `ladder` whose cost ratio is within
    `bound` of the plain form's. `plain` ({"wall_s", "cost_ratio"}) skips the
    plain run when it is already known. Returns the choice and the table of
    every size timed."""
    if plain is None:
        with Engine(g, device=device, ea_use_threshold=True, group_batch_size=64) as e:
            t = time.perf_counter()
            e.run(iterations)
            e.synchronize()
            wall = time.perf_counter() - t
            plain = {"wall_s": wall, "cost_ratio": e.encode()["cost_ratio_mags_compatible"]}
    table = []
    best = None
    for size in ladder:
        r = _timed_run(g, iterations, device, group_batch_size=size)
        r["group_batch_size"] = size
        r["delta_vs_plain"] = r["cost_ratio"] - plain["cost_ratio"]
        r["within_bound"] = abs(r["delta_vs_plain"]) <= bound
        table.append(r)
        if r["within_bound"] and (best is None or r["wall_s"] < best["wall_s"]):
            best = r
    if best is None:
        best = {"group_batch_size": 64, "wall_s": plain["wall_s"], "cost_ratio": plain["cost_ratio"],
                "delta_vs_plain": 0.0, "within_bound": True}
    return {"group_batch_size": best["group_batch_size"], "wall_s": best["wall_s"],
            "cost_ratio": best["cost_ratio"], "delta_vs_plain": best["delta_vs_plain"], "bound": bound,
            "plain": plain, "table": table}
