"""ctypes bindings to libbeam_gb300.so (the C ABI in include/beam_gb300.h).

Loading fails loudly when the in-tree library is missing: there is no
Python or CPU fallback for any kernel.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libbeam_gb300.so"

i32, i64, u64, f64 = C.c_int32, C.c_int64, C.c_uint64, C.c_double
P_i32 = C.POINTER(C.c_int32)
P_i64 = C.POINTER(C.c_int64)
P_f64 = C.POINTER(C.c_double)
vp = C.c_void_p


class EngineConfig(C.Structure):
    _fields_ = [
        ("top_k", i32),
        ("group_batch_size", i32),
        ("divide_hash_dims", i32),
        ("divide_max_group", i32),
        ("ea_use_threshold", i32),
        ("device", i32),
        ("seed", u64),
        ("verify_cuda_gain", i32),
        ("ranker", i32),
        ("ranker_train_iters", i32),
        ("ranker_recall", C.c_float),
        ("ranker_audit", i32),
        ("ranker_max_samples", i32),
        ("ranker_epochs", i32),
        ("ranker_max_steps", i32),
        ("ranker_lr", C.c_float),
    ]


_STAT_FIELDS = [
    "merge_group_count", "merge_group_max_size", "merge_raw_pair_count",
    "merge_candidate_pairs_after_prune", "candidate_proxy_pairs_examined",
    "merge_exact_gain_calls", "exact_gain_input_nnz",
    "exact_raw_entries_a", "exact_raw_entries_b", "exact_union_neighbors", "exact_overlap_neighbors",
    "merge_positive_gain_pairs", "merge_rejected_by_threshold", "merge_rejected_by_overlap",
    "merge_candidate_pairs", "merge_selected_pairs", "merge_total_local_gain",
    "selected_merges_for_validation", "validation_exact_calls", "validation_exact_row_entry_work",
    "accepted_merges_after_validation", "rejected_nonpositive", "update_touched_quotient_entries",
    "isolated_gain_sum", "divide_max_group_size", "divide_fallback_splits",
    "rows_rewritten", "row_entries_rewritten",
    "score_bytes", "prepare_bytes", "update_bytes", "divide_bytes",
    "blocks", "iterations", "pool_compactions", "active_supernodes", "groups_last",
]


class EngineStats(C.Structure):
    _fields_ = [("runtime_run_ms", f64), ("runtime_divide_ms", f64), ("runtime_merge_ms", f64)] + [
        (name, u64) for name in _STAT_FIELDS
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class RankerInfo(C.Structure):
    _fields_ = [(name, u64) for name in ("samples", "positives", "train_steps", "ranked", "pruned",
                                          "audit_passing", "audit_lost")] + [
        (name, f64) for name in ("train_ms", "first_loss", "final_loss", "cutoff", "calib_recall", "calib_prune")
    ] + [("trained", i32), ("reserved", i32)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_ if name != "reserved"}


class Encoding(C.Structure):
    _fields_ = [
        ("supernodes", i64), ("p", i64), ("cp", i64), ("cm", i64),
        ("superedges_loop", i64), ("superedges_nonloop", i64),
        ("encoding_cost_standard", i64), ("encoding_cost_mags_x2", i64),
        ("cost_ratio_standard", f64), ("cost_ratio_mags_compatible", f64),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class FlatScorerStats(C.Structure):
    _fields_ = [(name, i64) for name in ("calls", "kernel_launches", "pairs", "h2d_bytes", "d2h_bytes",
                                          "max_pairs_per_launch")] + [("kernel_ms", f64)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


TIME_NONE, TIME_SCORE, TIME_PREPARE, TIME_UPDATE, TIME_DIVIDE = 0, 1, 2, 3, 4

# name -> (restype, argtypes); every symbol declared in include/beam_gb300.h
SIGNATURES = {
    "beam_graph_generate": (vp, [C.c_char_p]),
    "beam_graph_load_text": (vp, [C.c_char_p]),
    "beam_graph_load_binary": (vp, [C.c_char_p]),
    "beam_graph_from_edges": (vp, [P_i32, P_i32, i64]),
    "beam_graph_write_text": (C.c_int, [vp, C.c_char_p]),
    "beam_graph_write_binary": (C.c_int, [vp, C.c_char_p]),
    "beam_graph_num_nodes": (i64, [vp]),
    "beam_graph_num_edges": (i64, [vp]),
    "beam_graph_num_arcs": (i64, [vp]),
    "beam_graph_row_ptr": (P_i64, [vp]),
    "beam_graph_col_idx": (P_i32, [vp]),
    "beam_graph_edge_u": (P_i32, [vp]),
    "beam_graph_edge_v": (P_i32, [vp]),
    "beam_graph_free": (None, [vp]),
    "beam_graph_last_error": (C.c_char_p, []),
    "beam_engine_default_config": (None, [C.POINTER(EngineConfig)]),
    "beam_engine_create": (C.c_int, [i32, i64, P_i64, P_i32, C.POINTER(EngineConfig), C.POINTER(vp)]),
    "beam_engine_destroy": (None, [vp]),
    "beam_engine_reset": (C.c_int, [vp]),
    "beam_engine_run": (C.c_int, [vp, i32]),
    "beam_engine_divide": (C.c_int, [vp, i32]),
    "beam_engine_merge": (C.c_int, [vp, i32, i32]),
    "beam_engine_group_counts": (C.c_int, [vp, P_i64, P_i64]),
    "beam_engine_groups": (C.c_int, [vp, P_i32, P_i32, P_i32]),
    "beam_engine_score_pairs": (C.c_int, [vp, P_i32, P_i32, i64, P_i64, P_i64]),
    "beam_engine_prepare_group": (C.c_int, [vp, P_i32, i32, P_i32, P_i32, i64, P_i64]),
    "beam_engine_merge_pairs": (C.c_int, [vp, P_i32, P_i32, i64]),
    "beam_engine_partition": (C.c_int, [vp, P_i32, P_i32, P_i32]),
    "beam_engine_export_row": (C.c_int, [vp, i32, P_i32, P_i64, i64, P_i64, P_i64, P_i64]),
    "beam_engine_get_stats": (C.c_int, [vp, C.POINTER(EngineStats)]),
    "beam_engine_quotient_nnz": (C.c_int, [vp, P_i64]),
    "beam_engine_exact_partition_cost": (C.c_int, [vp, P_i64]),
    "beam_engine_validate_quotient": (C.c_int, [vp]),
    "beam_engine_encode": (C.c_int, [vp, C.c_char_p, C.POINTER(Encoding)]),
    "beam_engine_ranker_info": (C.c_int, [vp, C.POINTER(RankerInfo)]),
    "beam_ranker_grad": (C.c_int, [i32, vp, vp, vp, i64, vp, vp, P_f64, vp]),
    "beam_ranker_last_error": (C.c_char_p, []),
    "beam_engine_set_timed_kernel": (C.c_int, [vp, i32]),
    "beam_engine_timed_kernel": (C.c_int, [vp, P_f64, P_i64]),
    "beam_engine_synchronize": (C.c_int, [vp]),
    "beam_engine_step_timer_start": (C.c_int, [vp]),
    "beam_engine_step_timer_stop": (C.c_int, [vp, P_f64]),
    "beam_engine_flush_l2": (C.c_int, [vp]),
    "beam_engine_launch_count": (C.c_int, [vp, P_i64]),
    "beam_engine_last_error": (C.c_char_p, []),
    "beam_prepare_flat_noalloc": (C.c_int, [vp, vp, vp, vp, vp, vp, vp, i32, i64, i32, vp, vp, i64, vp, vp]),
    "beam_prepare_flat_noalloc_last_error": (C.c_char_p, []),
    "beam_flat_scorer_create": (C.c_int, [i32, C.POINTER(vp)]),
    "beam_flat_scorer_destroy": (None, [vp]),
    "beam_flat_scorer_get_stats": (C.c_int, [vp, C.POINTER(FlatScorerStats)]),
    "beam_flat_scorer_memory_budget": (C.c_int, [vp, P_i64]),
    "beam_flat_scorer_score": (C.c_int, [vp, P_i32, i64, P_i32, P_i32, P_i64, P_i64, i32, P_i32, P_i64, P_i64, i64,
                                         P_i64, P_i64]),
    "beam_flat_scorer_last_error": (C.c_char_p, []),
    "beam_encode": (C.c_int, [i32, i64, P_i64, P_i32, P_i32, P_i32, C.c_char_p, C.POINTER(Encoding)]),
    "beam_exact_partition_cost": (C.c_int, [i32, P_i64, P_i32, P_i32, P_i64]),
    "beam_partition_hash": (u64, [i32, P_i32]),
    "beam_encode_last_error": (C.c_char_p, []),
}

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH} is missing: build the CUDA library first "
                "(python -c 'import __graft_entry__ as g; g.build()')")
        handle = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _lib = handle
    return _lib


class BeamError(RuntimeError):
    """Error reported through a *_last_error() call of the C ABI."""


def check(rc: int, err_fn: str = "beam_engine_last_error") -> None:
    if rc != 0:
        raise BeamError(getattr(lib(), err_fn)().decode())
