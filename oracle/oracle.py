"""ORACLE — test infrastructure only: ctypes wrapper of oracle/bin/liboracle.so,
the plain-C CPU restatement of the reference merge loop. Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg may use it, and only
as the checker or the timed CPU baseline.
"""

from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "bin" / "liboracle.so"
CLI_PATH = HERE / "bin" / "beam_oracle"
REF_BIN = HERE / "_ref" / "beam_ref"


class OracleConfig(C.Structure):
    _fields_ = [("top_k", C.c_int), ("group_batch_size", C.c_int), ("divide_hash_dims", C.c_int),
                ("divide_max_group", C.c_int), ("ea_use_threshold", C.c_int), ("seed", C.c_uint64),
                ("threads", C.c_int)]


_STATS = ["runtime_run_ms", "runtime_divide_ms", "runtime_merge_ms", "merge_prepare_wall_ms",
          "merge_gain_scoring_ms", "merge_selection_ms", "merge_update_ms"]
_STATS_I = ["divide_max_group_size", "divide_fallback_splits", "merge_group_count", "merge_group_max_size",
            "merge_raw_pair_count", "merge_candidate_pairs_after_prune", "merge_exact_gain_calls",
            "merge_positive_gain_pairs", "merge_rejected_by_threshold", "merge_rejected_by_overlap",
            "merge_candidate_pairs", "merge_selected_pairs", "merge_total_local_gain",
            "selected_merges_for_validation", "accepted_merges_after_validation", "rejected_nonpositive",
            "stale_endpoint", "validation_exact_calls", "validation_exact_row_entry_work",
            "update_touched_quotient_entries", "candidate_proxy_pairs_examined", "exact_gain_input_nnz",
            "exact_raw_entries_a", "exact_raw_entries_b", "exact_union_neighbors", "exact_overlap_neighbors",
            "quotient_nnz_final", "isolated_gain_sum", "groups_last", "active_supernodes_last"]
_SIGNED = {"divide_max_group_size", "divide_fallback_splits", "merge_candidate_pairs", "merge_selected_pairs",
           "merge_total_local_gain", "isolated_gain_sum"}


class OracleStats(C.Structure):
    _fields_ = ([(n, C.c_double) for n in _STATS]
                + [(n, C.c_int64 if n in _SIGNED else C.c_uint64) for n in _STATS_I])


class OracleEncoding(C.Structure):
    _fields_ = [("n_supernodes", C.c_int64), ("p", C.c_int64), ("cp", C.c_int64), ("cm", C.c_int64),
                ("encoding_cost_mags_x2", C.c_int64), ("cost_ratio_mags_compatible", C.c_double),
                ("num_superedges_loop", C.c_int64), ("num_superedges_nonloop", C.c_int64)]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            subprocess.run(["make", "-C", str(HERE), "oracle"], check=True, capture_output=True)
        L = C.CDLL(str(LIB_PATH))
        vp, i32, i64, P32, P64 = C.c_void_p, C.c_int32, C.c_int64, C.POINTER(C.c_int32), C.POINTER(C.c_int64)
        sig = {
            "beam_oracle_default_config": (None, [C.POINTER(OracleConfig)]),
            "beam_oracle_create": (vp, [i32, i64, P64, P32, C.POINTER(OracleConfig)]),
            "beam_oracle_free": (None, [vp]),
            "beam_oracle_last_error": (C.c_char_p, []),
            "beam_oracle_run": (C.c_int, [vp, C.c_int]),
            "beam_oracle_divide": (C.c_int, [vp, C.c_int]),
            "beam_oracle_merge": (C.c_int, [vp, C.c_int, C.c_int]),
            "beam_oracle_merge_blocks": (C.c_int, [vp, C.c_int, i64, C.c_double, P64]),
            "beam_oracle_group_count": (i64, [vp]),
            "beam_oracle_active_count": (i64, [vp]),
            "beam_oracle_groups": (C.c_int, [vp, P32, P32, P32]),
            "beam_oracle_prepare_group": (i64, [vp, P32, i32, P32, P32, i64]),
            "beam_oracle_exact_gain": (C.c_int, [vp, i32, i32, P64, P64]),
            "beam_oracle_merge_pair": (C.c_int, [vp, i32, i32]),
            "beam_oracle_labels": (C.c_int, [vp, P32]),
            "beam_oracle_member_lists": (C.c_int, [vp, P32, P32]),
            "beam_oracle_partition_hash": (C.c_uint64, [vp]),
            "beam_oracle_active": (C.c_int, [vp, i32]),
            "beam_oracle_size": (i64, [vp, i32]),
            "beam_oracle_internal": (i64, [vp, i32]),
            "beam_oracle_row": (i64, [vp, i32, P32, P64, i64]),
            "beam_oracle_exact_partition_cost": (i64, [vp]),
            "beam_oracle_get_stats": (None, [vp, C.POINTER(OracleStats)]),
            "beam_oracle_encode": (C.c_int, [vp, C.c_char_p, C.POINTER(OracleEncoding)]),
            "beam_oracle_legacy_flat_gain": (C.c_int, [P32, P32, P64, P64, P32, P64, P64, i32, i32, P64, P64]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class Oracle:
    """CPU restatement over a CSR (row_ptr int64[n+1], col_idx int32[arcs])."""

    def __init__(self, row_ptr, col_idx, top_k=16, group_batch_size=64, divide_hash_dims=16,
                 divide_max_group=512, ea_use_threshold=True, seed=1, threads=0):
        self.row_ptr = np.ascontiguousarray(row_ptr, np.int64)
        self.col_idx = np.ascontiguousarray(col_idx, np.int32)
        self.n = len(self.row_ptr) - 1
        cfg = OracleConfig()
        lib().beam_oracle_default_config(C.byref(cfg))
        cfg.top_k, cfg.group_batch_size = top_k, group_batch_size
        cfg.divide_hash_dims, cfg.divide_max_group = divide_hash_dims, divide_max_group
        cfg.ea_use_threshold, cfg.seed, cfg.threads = int(ea_use_threshold), seed, threads
        self._h = lib().beam_oracle_create(self.n, int(self.row_ptr[-1]), _p(self.row_ptr, C.c_int64),
                                           _p(self.col_idx, C.c_int32), C.byref(cfg))
        if not self._h:
            raise RuntimeError(lib().beam_oracle_last_error().decode())

    @classmethod
    def from_graph(cls, g, **kw) -> "Oracle":
        return cls(g.row_ptr, g.col_idx, **kw)

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(lib().beam_oracle_last_error().decode())

    def close(self):
        if getattr(self, "_h", None):
            lib().beam_oracle_free(self._h)
            self._h = None

    __del__ = close

    def run(self, iterations=20):
        self._check(lib().beam_oracle_run(self._h, iterations))

    def divide(self, it):
        self._check(lib().beam_oracle_divide(self._h, it))

    def merge(self, it, total=20):
        self._check(lib().beam_oracle_merge(self._h, it, total))

    def merge_blocks(self, it, first_group=0, budget_ms=0.0) -> int:
        """The blocks of Merge(it) from group first_group (a block boundary)
        until budget_ms ran out (<= 0: to the end); returns the first group of
        the next unprocessed block."""
        nxt = C.c_int64()
        self._check(lib().beam_oracle_merge_blocks(self._h, it, int(first_group), float(budget_ms), C.byref(nxt)))
        return int(nxt.value)

    def group_count(self) -> int:
        return int(lib().beam_oracle_group_count(self._h))

    def groups(self):
        na = lib().beam_oracle_active_count(self._h)
        ng = lib().beam_oracle_group_count(self._h)
        order = np.zeros(max(na, 1), np.int32)
        starts = np.zeros(max(ng, 1), np.int32)
        lengths = np.zeros(max(ng, 1), np.int32)
        lib().beam_oracle_groups(self._h, _p(order, C.c_int32), _p(starts, C.c_int32), _p(lengths, C.c_int32))
        return order[:na], starts[:ng], lengths[:ng]

    def prepare_group(self, q):
        q = np.ascontiguousarray(q, np.int32)
        cap = max(1, len(q) * len(q))
        a = np.zeros(cap, np.int32)
        b = np.zeros(cap, np.int32)
        cnt = lib().beam_oracle_prepare_group(self._h, _p(q, C.c_int32), len(q), _p(a, C.c_int32),
                                              _p(b, C.c_int32), cap)
        if cnt < 0:
            raise RuntimeError(lib().beam_oracle_last_error().decode())
        return np.stack([a[:cnt], b[:cnt]], axis=1)

    def exact_gain(self, a, b):
        g, bef = C.c_int64(), C.c_int64()
        self._check(lib().beam_oracle_exact_gain(self._h, int(a), int(b), C.byref(g), C.byref(bef)))
        return int(g.value), int(bef.value)

    def merge_pair(self, keep, remove):
        self._check(lib().beam_oracle_merge_pair(self._h, int(keep), int(remove)))

    def labels(self):
        out = np.zeros(self.n, np.int32)
        self._check(lib().beam_oracle_labels(self._h, _p(out, C.c_int32)))
        return out

    def member_lists(self):
        head = np.zeros(self.n, np.int32)
        nxt = np.zeros(self.n, np.int32)
        lib().beam_oracle_member_lists(self._h, _p(head, C.c_int32), _p(nxt, C.c_int32))
        return head, nxt

    def partition_hash(self):
        return int(lib().beam_oracle_partition_hash(self._h))

    def active(self, rep):
        return bool(lib().beam_oracle_active(self._h, rep))

    def size(self, rep):
        return int(lib().beam_oracle_size(self._h, rep))

    def internal(self, rep):
        return int(lib().beam_oracle_internal(self._h, rep))

    def row(self, rep):
        ln = lib().beam_oracle_row(self._h, rep, None, None, 0)
        nb = np.zeros(max(ln, 1), np.int32)
        cnt = np.zeros(max(ln, 1), np.int64)
        lib().beam_oracle_row(self._h, rep, _p(nb, C.c_int32), _p(cnt, C.c_int64), ln)
        return nb[:ln], cnt[:ln]

    def exact_partition_cost(self):
        return int(lib().beam_oracle_exact_partition_cost(self._h))

    def stats(self) -> dict:
        st = OracleStats()
        lib().beam_oracle_get_stats(self._h, C.byref(st))
        return {n: getattr(st, n) for n, _ in st._fields_}

    def encode(self, out_dir=None) -> dict:
        enc = OracleEncoding()
        self._check(lib().beam_oracle_encode(self._h, None if out_dir is None else str(out_dir).encode(),
                                             C.byref(enc)))
        return {n: getattr(enc, n) for n, _ in enc._fields_}


def legacy_flat_gains(flat: dict, pairs) -> tuple[np.ndarray, np.ndarray]:
    """Legacy-objective {gain, before_cost} of (a_idx, b_idx) row pairs of a flat
    per-block CSR (keys offsets, reps, rsz, self, nb, wt, nsz)."""
    f = {k: np.ascontiguousarray(flat[k], np.int64 if k in ("rsz", "self", "wt", "nsz") else np.int32)
         for k in ("offsets", "reps", "rsz", "self", "nb", "wt", "nsz")}
    pairs = np.asarray(pairs, np.int32).reshape(-1, 2)
    gain = np.zeros(len(pairs), np.int64)
    before = np.zeros(len(pairs), np.int64)
    g, b = C.c_int64(), C.c_int64()
    L = lib()
    for i, (x, y) in enumerate(pairs.tolist()):
        L.beam_oracle_legacy_flat_gain(_p(f["offsets"], C.c_int32), _p(f["reps"], C.c_int32),
                                       _p(f["rsz"], C.c_int64), _p(f["self"], C.c_int64), _p(f["nb"], C.c_int32),
                                       _p(f["wt"], C.c_int64), _p(f["nsz"], C.c_int64), x, y, C.byref(g),
                                       C.byref(b))
        gain[i], before[i] = g.value, b.value
    return gain, before
