#!/usr/bin/env python
"""Benchmark of the GB300 merge loop on R-MAT scale 24, edge factor 16 (the
large single-GPU configuration: n = 16.8M, m = 260M, 521M CSR arcs).

A step is one full 20-iteration run of the merge loop (Divide + Merge, the
reference's runtime_run_ms span) over the resident graph. The quotient graph
is reset to singletons and L2 is flushed (256 MB write) before every timed
step; both stay outside the timed span, which is measured with CUDA events on
the engine's stream. value = accepted merges of all ranks / slowest rank's
time for the headline form (--form); the other forms (batched: one block of
all groups per iteration; ranker: batched + the learned candidate ranker;
plain: the reference's 64-group blocks, bit-exact with the reference) are
timed beside it for the speed-ups and the cost-ratio comparison. e2e runs the
public C ABI from pinned host buffers every step (create from the host CSR =
H2D copies, 20 iterations, partition download = D2H).

The whole run keeps to a wall budget (--time-budget-s, 23 minutes by
default). The plain form runs last, in a child process stopped when the
budget is spent: at this scale one plain run is about 9 minutes of
latency-bound 64-group blocks, and a form that cannot finish is reported
as incomplete instead of holding the GPU past the budget. The CPU baseline's
child is bounded the same way.

The CPU side (cpu_baseline, and --impl reference) times the C oracle, a
restatement of the reference path pinned to the reference's outputs, with
OpenMP on all host cores (OMP_PROC_BIND=close, OMP_PLACES=cores), on bounded
samples of the same workload: 64-group blocks of Merge spread evenly over
iteration 1, each charged its groups' share of the iteration's Divide time. A
full 20-iteration CPU run of this graph takes hours.

Multi-GPU (torchrun): replicas only - every rank runs the same workload on
its own GPU with no collective on the data path.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "20-iter wall s & merges/s: batched+ranker vs plain GPU at equal cost ratio"
UNIT = "merges/s"
ITERATIONS = 20
WORKLOAD_DESC = {
    "rmat24": "R-MAT scale 24, edge factor 16 (a=0.57, b=0.19, c=0.19), seed 11, deduplicated, loop-free",
    "rmat19": "R-MAT scale 19, edge factor 2 (a=0.57, b=0.19, c=0.19), seed 7, deduplicated, loop-free",
    "rmat20_ef16": "R-MAT scale 20, edge factor 16 (a=0.57, b=0.19, c=0.19), seed 11, deduplicated, loop-free",
    "chunglu4m_twins": "Chung-Lu n=4M, power-law 2.3, mean degree 17, + 200k planted near-twin groups, seed 4",
    "grid_chunglu_union": "1400x1400 grid (10% deleted, 2% diagonals) + Chung-Lu n=1.1M, power-law 2.1, seed 3",
    "dcsbm_4096": "degree-corrected SBM n=4096, 32 blocks, p_in/p_out=40, power-law 2.5, mean degree 43, seed 1",
}
FALLBACK_HBM_GBS = 6800.0
KERNEL_CLASSES = {"score": 1, "prepare": 2, "update": 3, "divide": 4}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ------------------------------------------------------------------ dist


class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch
            import torch.distributed as dist
            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local_rank)
            dist.init_process_group(backend)
            self.pg = dist
            self.device = torch.device("cuda", self.local_rank) if backend == "nccl" else torch.device("cpu")

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def reduce(self, value: float, op: str) -> float:
        if not self.pg:
            return value
        import torch
        t = torch.tensor([value], dtype=torch.float64, device=self.device)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX if op == "max" else self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# --------------------------------------------------------------- clocks


class ClockSampler:
    """nvidia-smi samples every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int, log_path: Path | None):
        self.device = device
        self.rows = []
        self.proc = None
        self.log_path = log_path

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=5)
            self.thread.join(timeout=5)
        if self.log_path and self.rows:
            self.log_path.write_text("\n".join(",".join(r) for r in self.rows) + "\n")

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for name, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------- misc


def measured_peak() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except (KeyError, ValueError):
            pass
    return FALLBACK_HBM_GBS, "fallback"


# the kernel that each timed class stands for (its largest kernel)
KERNEL_OF_CLASS = {"score": "ScoreKernel", "prepare": "PrepareKernel", "update": "CommitKernel",
                   "divide": "MinHashKernel"}


def union_roofline(t: dict, peak: float) -> dict:
    """The scoring roofline with the reference's work counters: 8 B per row
    entry of both rows, 4 B per union neighbour and 24 B per pair
    (8 exact_gain_input_nnz + 4 exact_union_neighbors + 24 merge_exact_gain_calls)."""
    u = t["union"]
    nbytes = 8 * u["exact_gain_input_nnz"] + 4 * u["exact_union_neighbors"] + 24 * u["merge_exact_gain_calls"]
    secs = t["kernel_ms"] / 1000.0
    gbs = nbytes / secs / 1e9 if secs > 0 else 0.0
    return {"algorithmic_bytes_per_launch": round(nbytes / max(1, t["kernel_launches"]), 1),
            "achieved": round(gbs, 2), "frac": round(gbs / peak, 5) if peak else None}


def profiled_traffic(kernel_class: str, workload: str, form: str) -> float | None:
    """Mean DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum)
    from the committed ncu summary of this kernel on this workload and form."""
    f = ROOT / "profiles" / f"{KERNEL_OF_CLASS[kernel_class]}_{workload}_{form}_dram.md"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.strip().startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


def golden_hash(workload: str) -> str | None:
    g = json.loads((ROOT / "tests" / "golden" / "golden.json").read_text())
    for c in g["cases"]:
        if c["name"] == workload:
            return c["metrics"]["partition_hash"]
    return None


# ------------------------------------------------------------ GPU arm


FORMS = {
    # one block per iteration: every group of an iteration is prepared, scored,
    # selected and committed by one launch of each kernel
    "batched": {"group_batch_size": 1 << 30},
    # the batched form with the learned candidate ranker (trained on the exact
    # gains of iterations 1-5, prunes candidates before exact scoring later)
    "ranker": {"group_batch_size": 1 << 30, "ranker": True},
    # the reference's 64-group blocks: bit-exact with the reference CPU path
    "plain": {"group_batch_size": 64},
}


def form_engine(g, device: int, form: str):
    from beam_gb300 import Engine

    return Engine(g, device=device, ea_use_threshold=True, **FORMS[form])


def kernel_breakdown(e, peak: float) -> dict:
    """Device time per kernel class over one untimed 20-iteration run each,
    with the class's algorithmic bytes (counted by its kernels) and the
    roofline fraction they give against the HBM peak."""
    out = {}
    for name, kind in KERNEL_CLASSES.items():
        e.reset()
        b0 = e.stats()[f"{name}_bytes"]
        e.set_timed_kernel(kind)
        e.run(ITERATIONS)
        ms, launches = e.timed_kernel()
        nbytes = e.stats()[f"{name}_bytes"] - b0
        gbs = nbytes / (ms / 1000.0) / 1e9 if ms > 0 else 0.0
        out[name] = {"ms": round(ms, 3), "launches": launches, "algorithmic_bytes": nbytes,
                     "achieved_gbs": round(gbs, 1), "frac": round(gbs / peak, 5) if peak else None}
    e.set_timed_kernel(0)
    return out


def timed_steps(e, steps: int, dominant: str | None) -> dict:
    """steps x (reset, L2 flush, timed 20-iteration run); CUDA events on the
    engine stream around each run, the dominant kernel class timed inside."""
    step_ms, merges, kernel_ms, kernel_launches, kernel_bytes, step_launches = [], 0, 0.0, 0, 0, 0
    union = {"exact_gain_input_nnz": 0, "exact_union_neighbors": 0, "merge_exact_gain_calls": 0}
    for _ in range(steps):
        e.reset()
        e.flush_l2()
        st0 = e.stats()
        if dominant:
            e.set_timed_kernel(KERNEL_CLASSES[dominant])
        launches0 = e.launch_count()
        e.step_timer_start()
        e.run(ITERATIONS)
        step_ms.append(e.step_timer_stop())
        step_launches += e.launch_count() - launches0
        st1 = e.stats()
        if dominant:
            ms, launches = e.timed_kernel()
            kernel_ms += ms
            kernel_launches += launches
            kernel_bytes += st1[f"{dominant}_bytes"] - st0[f"{dominant}_bytes"]
            for k in ("exact_gain_input_nnz", "exact_union_neighbors", "merge_exact_gain_calls"):
                union[k] += st1[k] - st0[k]
        merges += st1["accepted_merges_after_validation"] - st0["accepted_merges_after_validation"]
    e.synchronize()
    e.set_timed_kernel(0)
    return {"step_ms": step_ms, "merges": merges, "kernel_ms": kernel_ms, "kernel_launches": kernel_launches,
            "kernel_bytes": kernel_bytes, "launches": step_launches, "union": union}


class PinnedGraph:
    """The graph's CSR copied into page-locked host memory (the e2e input)."""

    def __init__(self, g, row_ptr, col_idx, keep):
        self.n, self.arcs, self.row_ptr, self.col_idx, self._keep = g.n, g.arcs, row_ptr, col_idx, keep


def pinned_graph(g):
    try:
        import torch

        rp = torch.empty(len(g.row_ptr), dtype=torch.int64, pin_memory=True)
        ci = torch.empty(len(g.col_idx), dtype=torch.int32, pin_memory=True)
        rp.numpy()[:] = g.row_ptr
        ci.numpy()[:] = g.col_idx
        return PinnedGraph(g, rp.numpy(), ci.numpy(), (rp, ci))
    except (ImportError, RuntimeError):
        return g  # no CUDA-enabled torch: pageable host memory


def final_metrics(e) -> tuple[float, str]:
    """Cost ratio (device Encode) and partition hash of the engine's current
    partition."""
    from beam_gb300 import partition_hash

    enc = e.encode()
    labels, _, _ = e.partition()
    return enc["cost_ratio_mags_compatible"], str(partition_hash(labels))


def hbm_residency(e, g) -> dict:
    """Device bytes of the resident state, by part (the engine's own buffers)."""
    n, arcs = g.n, g.arcs
    pool = 2 * 8 * (3 * arcs + 2 * n + 4096)
    return {"csr_bytes": 8 * (n + 1) + 8 * arcs, "quotient_pool_bytes": pool,
            "quotient_row_meta_bytes": 8 * n + 4 * n * 3 + 8 * n,
            "candidate_bytes_per_slot": 40, "device_used_bytes": device_used_bytes()}


def device_used_bytes() -> int | None:
    try:
        import torch

        free, total = torch.cuda.mem_get_info()
        return int(total - free)
    except Exception:  # noqa: BLE001 - reporting only
        return None


def run_ours(args, dist: Dist) -> dict | None:
    from beam_gb300 import WORKLOADS, Graph

    t_start = time.perf_counter()

    def remaining() -> float:
        """Seconds left of the whole run's time budget (--time-budget-s)."""
        return args.time_budget_s - (time.perf_counter() - t_start)

    spec = WORKLOADS[args.workload]
    t0 = time.perf_counter()
    g = Graph.generate(spec)
    log(f"[bench] graph {args.workload}: n={g.n} m={g.edges} ({time.perf_counter() - t0:.1f}s)")
    device = dist.local_rank
    head_form = args.form
    # the in-process comparison forms; the plain form (thousands of dependent
    # 64-group blocks, minutes per run) runs last, in a child process bounded
    # by what is left of the time budget
    others = [] if args.no_other_form else [f for f in FORMS if f not in (head_form, "plain")]
    run_plain = not args.no_other_form and head_form != "plain"
    want = golden_hash(args.workload)

    # headline form: warm-up, kernel breakdown, timed region
    e = form_engine(g, device, head_form)
    for _ in range(args.warmup):
        e.reset()
        e.run(ITERATIONS)
    peak, peak_kind = measured_peak()
    breakdown = kernel_breakdown(e, peak)
    residency = hbm_residency(e, g)
    # the roofline kernel: ScoreKernel, the scoring kernel of the path
    dominant = args.timed_kernel or "score"
    dist.barrier()
    e.synchronize()
    # the raw nvidia-smi samples of the timed region, when a path is given
    clock_log = Path(os.environ["BEAM_BENCH_CLOCKS_CSV"]) if os.environ.get("BEAM_BENCH_CLOCKS_CSV") else None
    wall0 = time.perf_counter()
    with ClockSampler(device, clock_log) as clocks:
        t = timed_steps(e, args.steps, dominant)
    dist.barrier()
    wall_s = time.perf_counter() - wall0
    total_ms = sum(t["step_ms"])
    max_ms = dist.reduce(total_ms, "max")
    all_merges = dist.reduce(float(t["merges"]), "sum")
    value = all_merges / (max_ms / 1000.0)
    ms_per_step = max_ms / args.steps
    head_ratio, head_hash = final_metrics(e)
    info = e.ranker_info() if FORMS[head_form].get("ranker") else None
    e.close()
    log(f"[bench] {head_form}: {args.steps} timed steps, {ms_per_step:.1f} ms per step "
        f"({time.perf_counter() - t_start:.0f} s into the run)")
    forms = {head_form: {"wall_s_20iter": round(ms_per_step / 1000.0, 4),
                         "merges_per_s": round(value / dist.world, 1),
                         "merges_per_step": t["merges"] // max(1, args.steps),
                         "cost_ratio_mags_compatible": round(head_ratio, 6),
                         "partition_hash": head_hash, "steps": args.steps, **FORMS[head_form]}}
    if info:
        forms[head_form]["ranker"] = {k: info[k] for k in ("samples", "train_steps", "ranked", "pruned", "train_ms",
                                                           "final_loss")}

    # the other forms, for the speed-ups and the cost-ratio comparison
    for other_form in others:
        eo = form_engine(g, device, other_form)
        eo.reset()
        eo.run(ITERATIONS)
        o_steps = max(1, min(args.steps, 3))
        to = timed_steps(eo, o_steps, None)
        o_ms = sum(to["step_ms"]) / o_steps
        o_ratio, o_hash = final_metrics(eo)  # the partition of the last timed run
        info = eo.ranker_info() if FORMS[other_form].get("ranker") else None
        eo.close()
        forms[other_form] = {"wall_s_20iter": round(o_ms / 1000.0, 4),
                             "merges_per_s": round(to["merges"] / (sum(to["step_ms"]) / 1000.0), 1),
                             "merges_per_step": to["merges"] // o_steps,
                             "cost_ratio_mags_compatible": round(o_ratio, 6),
                             "partition_hash": o_hash, "steps": o_steps, **FORMS[other_form]}
        if info:
            forms[other_form]["ranker"] = {k: info[k] for k in ("samples", "train_steps", "ranked", "pruned",
                                                                "train_ms", "final_loss")}
        log(f"[bench] {other_form}: {o_steps} timed steps, {o_ms:.1f} ms per step "
            f"({time.perf_counter() - t_start:.0f} s into the run)")

    # e2e through the C ABI from host buffers: create from the host CSR
    # held in pinned memory (H2D), 20 iterations, partition download (D2H)
    hg = pinned_graph(g)
    e2e_steps = max(1, min(args.steps, args.e2e_steps))
    e2e_ms, e2e_merges = [], 0
    for i in range(1 + e2e_steps):
        if i >= 2 and remaining() < 240:
            e2e_steps = i - 1  # keep the rest of the budget for the CPU baseline and the plain form
            break
        t1 = time.perf_counter()
        with form_engine(hg, device, head_form) as ee:
            ee.run(ITERATIONS)
            ee.partition()
            m = ee.stats()["accepted_merges_after_validation"]
        if i >= 1:
            e2e_ms.append((time.perf_counter() - t1) * 1000.0)
            e2e_merges += m
    e2e_max = dist.reduce(sum(e2e_ms), "max")
    e2e_all = dist.reduce(float(e2e_merges), "sum")
    log(f"[bench] e2e: {e2e_steps} timed steps ({time.perf_counter() - t_start:.0f} s into the run)")

    # the CPU baseline (rank 0, one GPU), then the plain form, both bounded
    cpu_base = None
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        cpu_base = cpu_baseline(args, timeout_s=max(60.0, min(300.0, remaining() - 120.0)))
        log(f"[bench] cpu baseline ({time.perf_counter() - t_start:.0f} s into the run)")
    if run_plain:
        forms["plain"] = plain_form(args, device, timeout_s=remaining() - 30.0)
        log(f"[bench] plain: {forms['plain'].get('wall_s_20iter')} s per 20-iteration run "
            f"({time.perf_counter() - t_start:.0f} s into the run)")
        if forms["plain"].get("complete"):
            forms["plain"]["bit_exact_vs_reference"] = (None if want is None
                                                        else forms["plain"]["partition_hash"] == want)
    comparison = {}
    if forms.get("plain", {}).get("complete"):
        for f in forms:
            if f == "plain":
                continue
            comparison[f"speedup_{f}_vs_plain"] = round(forms["plain"]["wall_s_20iter"] / forms[f]["wall_s_20iter"], 3)
            comparison[f"cost_ratio_delta_abs_{f}_vs_plain"] = round(
                forms[f]["cost_ratio_mags_compatible"] - forms["plain"]["cost_ratio_mags_compatible"], 6)

    kernel_ms, kernel_launches = t["kernel_ms"], t["kernel_launches"]
    achieved = t["kernel_bytes"] / (kernel_ms / 1000.0) / 1e9 if kernel_ms > 0 else 0.0
    traffic = profiled_traffic(dominant, args.workload, head_form)
    result = {
        "metric": METRIC,
        "value": round(value, 1),
        "unit": UNIT,
        "n_gpus": dist.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_per_step, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int64",
        "data": "synthetic (seeded generator)",
        "config": {
            "workload": f"{args.workload}: {WORKLOAD_DESC.get(args.workload, spec)}; n={g.n}, m={g.edges}",
            "form": head_form,
            "path": {"batched": "batched GPU form: one block of all groups per iteration",
                     "ranker": "batched GPU form + learned candidate ranker",
                     "plain": "plain GPU form: 64-group blocks, bit-exact with the reference"}[head_form],
            "flags": "batch-ea-blocked, mags-compatible, persistent, incremental, legacy index, certification off, "
                     "g0, top-k 16, reciprocal threshold, 20 iterations, seed 1",
            "wall_s_20iter": round(ms_per_step / 1000.0, 4),
            "l2": "flushed by a 256 MB write before every timed step (outside the timed span); the quotient graph "
                  "(tens of GB) is far larger than L2",
            "parallelism": f"replicas x{dist.world}",
            "hbm_residency": residency,
        },
        "forms": forms,
        "comparison": comparison,
        "e2e": {
            "value": round(e2e_all / (e2e_max / 1000.0), 1) if e2e_max > 0 else None,
            "unit": UNIT,
            "h2d_bytes_per_step": 8 * (g.n + 1) + 4 * g.arcs,
            "host_buffers": "pinned" if isinstance(hg, PinnedGraph) else "pageable",
            "d2h_bytes_per_step": 12 * g.n,
            "ms_per_step": round(e2e_max / e2e_steps, 3),
            "steps": e2e_steps,
        },
        "gpu_launches": t["launches"],
        "roofline": {
            "kernel": KERNEL_OF_CLASS[dominant],
            "bound": "hbm",
            "achieved": round(achieved, 2),
            "peak": peak,
            "unit": "GB/s",
            "frac": round(achieved / peak, 5) if peak else None,
            "peak_source": peak_kind,
            "traffic": traffic,
            "algorithmic_bytes_per_launch": round(t["kernel_bytes"] / max(1, kernel_launches), 1),
            "bytes_counted": "8 B per row entry read, 4 B per shared-neighbour size, 36 B of row sums and 24 B "
                             "per scored pair (the kernel's own reads)",
            "union_count": union_roofline(t, peak),
            "avg_launch_us": round(1000.0 * kernel_ms / max(1, kernel_launches), 3),
            "launches": kernel_launches,
        },
        "breakdown_ms_per_run": breakdown,
        "clocks": clocks.summary(),
        "wall_s_timed_region": round(wall_s, 3),
        "wall_s_run": round(time.perf_counter() - t_start, 1),
    }
    if cpu_base is not None:
        result["cpu_baseline"] = cpu_base
    return result


# ------------------------------------------------------------ CPU side

OMP_ENV = {"OMP_PROC_BIND": "close", "OMP_PLACES": "cores"}


def host_cpu() -> dict:
    """Host cores and model (lscpu), for the CPU baseline's description."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    return {"cores": os.cpu_count() or 1, "model": model}


def cpu_sample(g, steps: int, warmup: int, step_budget_s: float, threads: int) -> dict:
    """The oracle on bounded samples of the workload: 64-group blocks of Merge
    spread evenly over iteration 1 (every stride-th block from a few probe
    blocks' timing, so that all steps end near the middle of the iteration
    rather than all in its first groups), each block charged its groups' share
    of the iteration's Divide time. A step is the blocks that start before
    step_budget_s has run out. Blocks are sequentially dependent, so skipping
    the ones between changes the state a little; the sample measures the cost
    and the merges of representative blocks, not one exact run."""
    sys.path.insert(0, str(ROOT / "oracle"))
    from oracle import Oracle

    t0 = time.perf_counter()
    o = Oracle.from_graph(g, ea_use_threshold=True, threads=threads)
    setup_s = time.perf_counter() - t0
    t1 = time.perf_counter()
    o.divide(1)
    divide_s = time.perf_counter() - t1
    ngroups = o.group_count()
    bs = 64
    nblocks = max(1, (ngroups + bs - 1) // bs)
    accepted = lambda: o.stats()["accepted_merges_after_validation"]  # noqa: E731

    def run_block(b: int) -> tuple[float, int, int]:
        m0 = accepted()
        t = time.perf_counter()
        nxt = o.merge_blocks(1, b * bs, 1e-9)  # exactly one block
        return time.perf_counter() - t, accepted() - m0, nxt - b * bs

    # probe: the per-block cost of a few blocks spread over the iteration
    probe = [run_block(b) for b in range(0, nblocks, max(1, nblocks // 16))][:16]
    per_block = max(1e-6, sum(p[0] for p in probe) / len(probe))
    if ITERATIONS * (nblocks * per_block + divide_s) <= 0.5 * (warmup + steps) * step_budget_s:
        # a small graph: whole 20-iteration runs fit the budget, one per step
        o.close()
        timed_merges, timed_s, groups = 0, 0.0, 0
        for step in range(warmup + steps):
            o = Oracle.from_graph(g, ea_use_threshold=True, threads=threads)
            t = time.perf_counter()
            o.run(ITERATIONS)
            dt = time.perf_counter() - t
            if step >= warmup:
                timed_merges += o.stats()["accepted_merges_after_validation"]
                timed_s += dt
            o.close()
        return {"merges": timed_merges, "secs": timed_s, "groups": 0, "iterations": list(range(1, ITERATIONS + 1)),
                "setup_s": setup_s, "stride": 0, "nblocks": nblocks, "full_runs": steps}
    want = max(1, int((warmup + steps) * step_budget_s / per_block))
    stride = max(1, nblocks // want)
    order = list(range(stride // 2, nblocks, stride))
    timed_merges, timed_s, timed_groups, pos = 0, 0.0, 0, 0
    for step in range(warmup + steps):
        merges, secs, groups = 0, 0.0, 0
        while secs < step_budget_s:
            if pos == len(order):
                # a small graph runs out of blocks: the same blocks again, on a
                # fresh partition (setup untimed, Divide timed again)
                o.close()
                o = Oracle.from_graph(g, ea_use_threshold=True, threads=threads)
                t1 = time.perf_counter()
                o.divide(1)
                divide_s = time.perf_counter() - t1
                pos = 0
            dt, m, gcount = run_block(order[pos])
            pos += 1
            secs += dt + divide_s * gcount / max(1, ngroups)
            merges += m
            groups += gcount
        if step >= warmup:
            timed_merges += merges
            timed_s += secs
            timed_groups += groups
    o.close()
    return {"merges": timed_merges, "secs": timed_s, "groups": timed_groups, "iterations": [1],
            "setup_s": setup_s, "stride": stride, "nblocks": nblocks, "full_runs": 0}


def sample_text(workload: str, r: dict) -> str:
    head = f"the C oracle (the reference path restated, pinned to its outputs) on {workload}: "
    if r["full_runs"]:
        return head + f"whole 20-iteration runs ({r['merges']} merges, {r['secs']:.2f} s)"
    return head + (f"every {r['stride']}th of the {r['nblocks']} 64-group blocks of iteration 1, {r['groups']} Divide "
                   f"groups in all ({r['merges']} merges, {r['secs']:.2f} s including their share of Divide; oracle "
                   f"setup {r['setup_s']:.1f} s untimed)")


def reexec_with_omp_env() -> None:
    """OpenMP reads its placement variables when it starts: run this process
    again with them set (once)."""
    if all(os.environ.get(k) == v for k, v in OMP_ENV.items()):
        return
    env = dict(os.environ, **OMP_ENV)
    env.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    os.execve(sys.executable, [sys.executable, *sys.argv], env)


def _text(x) -> str:
    return x.decode(errors="replace") if isinstance(x, bytes) else (x or "")


def cpu_baseline(args, timeout_s: float) -> dict:
    """The oracle on the host cores in a child process (OpenMP placement set
    before it starts), one bounded sample of the workload, stopped after
    timeout_s."""
    cmd = [sys.executable, str(ROOT / "bench.py"), "--cpu-sample", "--workload", args.workload,
           "--sample-seconds", str(args.cpu_sample_seconds)]
    env = dict(os.environ, **OMP_ENV, OMP_NUM_THREADS=str(os.cpu_count() or 1))
    try:
        proc = subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=timeout_s)
        out, err, rc = proc.stdout, proc.stderr, proc.returncode
    except subprocess.TimeoutExpired as ex:
        out, err, rc = _text(ex.stdout), _text(ex.stderr), None
    lines = [l for l in out.splitlines() if l.startswith("{")]
    if rc != 0 or not lines:
        why = f"stopped after {timeout_s:.0f} s" if rc is None else f"failed: {err[-300:]}"
        return {"value": None, "unit": UNIT, "cores": 0, "kind": "port", "sample": f"CPU sample {why}"}
    return json.loads(lines[-1])


def plain_form(args, device: int, timeout_s: float) -> dict:
    """The plain form (the reference's 64-group blocks, bit-exact with the
    reference) timed in a child process (--plain-child): a warm-up of
    iteration 1, then one 20-iteration run, its cost ratio and partition hash.
    The child is stopped when the run's time budget is spent; the form is then
    reported as incomplete, with the last iteration it finished."""
    base = {"group_batch_size": FORMS["plain"]["group_batch_size"], "steps": 1}
    if timeout_s < 60.0:
        return {**base, "complete": False, "wall_s_20iter": None,
                "note": "not run: the bench's time budget (--time-budget-s) was spent"}
    cmd = [sys.executable, str(ROOT / "bench.py"), "--plain-child", "--workload", args.workload,
           "--plain-device", str(device)]
    try:
        proc = subprocess.run(cmd, capture_output=True, text=True, timeout=timeout_s)
        out, err, rc = proc.stdout, proc.stderr, proc.returncode
    except subprocess.TimeoutExpired as ex:
        out, err, rc = _text(ex.stdout), _text(ex.stderr), None
    lines = [l for l in out.splitlines() if l.startswith("{")]
    if rc == 0 and lines:
        return {**json.loads(lines[-1]), **base, "complete": True}
    progress = [l for l in err.splitlines() if l.startswith("[plain]")]
    why = (f"stopped at the bench's time budget after {timeout_s:.0f} s" if rc is None
           else f"child failed (rc {rc}): {err[-300:]}")
    log(f"[bench] plain form incomplete: {why}; last progress: {progress[-1] if progress else 'none'}")
    return {**base, "complete": False, "wall_s_20iter": None, "note": why,
            "progress": progress[-1] if progress else None}


def plain_child(args) -> None:
    """--plain-child: the plain form's measurement (see plain_form), one JSON
    line on stdout, progress per iteration on stderr."""
    from beam_gb300 import WORKLOADS, Graph

    g = Graph.generate(WORKLOADS[args.workload])
    e = form_engine(g, args.plain_device, "plain")
    log("[plain] engine ready, warm-up (iteration 1) started")
    t0 = time.perf_counter()
    e.divide(1)
    e.synchronize()
    log(f"[plain] warm-up Divide: {time.perf_counter() - t0:.1f} s")
    e.merge(1, ITERATIONS)
    e.synchronize()
    warmup_s = time.perf_counter() - t0
    log(f"[plain] warm-up (iteration 1): {warmup_s:.1f} s")
    e.reset()
    e.flush_l2()
    acc = "accepted_merges_after_validation"
    m0 = e.stats()[acc]
    t1 = time.perf_counter()
    e.step_timer_start()
    for it in range(1, ITERATIONS + 1):
        e.divide(it)
        e.merge(it, ITERATIONS)
        log(f"[plain] iteration {it} of {ITERATIONS} done, {time.perf_counter() - t1:.1f} s into the timed run")
    ms = e.step_timer_stop()
    merges = e.stats()[acc] - m0
    ratio, phash = final_metrics(e)
    e.close()
    print(json.dumps({"wall_s_20iter": round(ms / 1000.0, 4), "merges_per_s": round(merges / (ms / 1000.0), 1),
                      "merges_per_step": merges, "cost_ratio_mags_compatible": round(ratio, 6),
                      "partition_hash": phash, "warmup_s": round(warmup_s, 1)}), flush=True)


def cpu_sample_main(args) -> None:
    from beam_gb300 import WORKLOADS, Graph

    g = Graph.generate(WORKLOADS[args.workload])
    cpu = host_cpu()
    r = cpu_sample(g, steps=1, warmup=0, step_budget_s=args.sample_seconds, threads=cpu["cores"])
    value = r["merges"] / r["secs"] if r["secs"] > 0 else 0.0
    print(json.dumps({
        "value": round(value, 1), "unit": UNIT, "cores": cpu["cores"], "kind": "port",
        "affinity": "OMP_PROC_BIND=close, OMP_PLACES=cores", "cpu_model": cpu["model"],
        "sample": sample_text(args.workload, r)}), flush=True)


def run_reference(args, dist: Dist) -> dict | None:
    if dist.rank != 0:
        return None
    from beam_gb300 import WORKLOADS, Graph

    g = Graph.generate(WORKLOADS[args.workload])
    cpu = host_cpu()
    budget = args.reference_step_seconds
    r = cpu_sample(g, steps=args.steps, warmup=args.warmup, step_budget_s=budget, threads=cpu["cores"])
    value = r["merges"] / r["secs"] if r["secs"] > 0 else 0.0
    sample = sample_text(args.workload, r) + f"; {args.warmup} warm-up + {args.steps} timed steps of about {budget:g} s"
    return {
        "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1000.0 * r["secs"] / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int64", "data": "synthetic (seeded generator)",
        "impl": "reference",
        "config": {"workload": f"{args.workload}: {WORKLOAD_DESC.get(args.workload, '')}; n={g.n}, m={g.edges}",
                   "path": "CPU restatement of the reference path (C + OpenMP), pinned bit-exact to its outputs",
                   "affinity": "OMP_PROC_BIND=close, OMP_PLACES=cores", "cpu_model": cpu["model"]},
        "cpu_baseline": {"value": round(value, 1), "unit": UNIT, "cores": cpu["cores"], "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 1), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def profile_run(args) -> None:
    """One 20-iteration run of the workload (the unit ncu captures)."""
    from beam_gb300 import WORKLOADS, Engine, Graph

    g = Graph.generate(WORKLOADS[args.workload])
    batch = FORMS[args.form]["group_batch_size"]
    with Engine(g, ea_use_threshold=True, **FORMS[args.form]) as e:
        t = time.perf_counter()
        e.run(args.profile_iterations)
        e.synchronize()
        st = e.stats()
        log(f"[profile-run] {args.workload} batch={batch}: {time.perf_counter() - t:.3f} s, "
            f"{st['accepted_merges_after_validation']} merges, {e.launch_count()} launches, "
            f"divide {st['runtime_divide_ms']:.1f} ms, merge {st['runtime_merge_ms']:.1f} ms, "
            f"blocks {st['blocks']}, compactions {st['pool_compactions']}")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--profile-run", action="store_true", help="one run only, for ncu")
    ap.add_argument("--profile-iterations", type=int, default=ITERATIONS)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="rmat24")
    ap.add_argument("--timed-kernel", choices=list(KERNEL_CLASSES), default=None)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--form", choices=list(FORMS), default="ranker",
                    help="form whose throughput is the headline value")
    ap.add_argument("--no-other-form", action="store_true", help="skip timing the other forms")
    ap.add_argument("--time-budget-s", type=float, default=1380.0,
                    help="wall budget of the whole run: the CPU baseline and the plain form (run last) are "
                         "stopped when it is spent")
    ap.add_argument("--plain-child", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--plain-device", type=int, default=0, help=argparse.SUPPRESS)
    ap.add_argument("--e2e-steps", type=int, default=5, help="timed e2e runs (at most --steps)")
    ap.add_argument("--batch-groups", type=int, default=None,
                    help="groups per block of the batched and ranker forms (default: all groups of an iteration)")
    ap.add_argument("--cpu-sample", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--sample-seconds", type=float, default=20.0, help=argparse.SUPPRESS)
    ap.add_argument("--cpu-sample-seconds", type=float, default=20.0,
                    help="length of the CPU baseline's bounded sample")
    ap.add_argument("--reference-step-seconds", type=float, default=4.0,
                    help="length of one step of the reference arm's bounded samples")
    args = ap.parse_args()
    if args.batch_groups:
        for f in ("batched", "ranker"):
            FORMS[f]["group_batch_size"] = args.batch_groups
    if args.profile_run:
        profile_run(args)
        return
    if args.cpu_sample:
        cpu_sample_main(args)
        return
    if args.plain_child:
        plain_child(args)
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference" and int(os.environ.get("RANK", "0")) == 0:
        reexec_with_omp_env()
    dist = Dist()
    try:
        result = run_reference(args, dist) if args.impl == "reference" else run_ours(args, dist)
        if result is not None and dist.rank == 0:
            print(json.dumps(result), flush=True)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
