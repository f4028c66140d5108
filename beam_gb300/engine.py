"""Python face of the GB300 merge loop, mirroring the reference's Sweg /
QuotientGraph operations (src/sweg.cpp, src/quotient_graph.cpp) over the C ABI.

    g = Graph.generate("rmat:scale=19,ef=2,a=0.57,b=0.19,c=0.19,seed=7")
    e = Engine(g, ea_use_threshold=True)
    e.run(20)                       # Sweg::Run
    labels, head, nxt = e.partition()
    enc = g.encode(head, nxt)       # Sweg::Encode + compression metrics
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native as N

__all__ = ["Graph", "Engine", "EngineOptions"]


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


class Graph:
    """Symmetric CSR graph held by the native library (reference loader rules)."""

    def __init__(self, handle: int):
        if not handle:
            raise N.BeamError(N.lib().beam_graph_last_error().decode())
        self._h = handle
        L = N.lib()
        self.n = int(L.beam_graph_num_nodes(handle))
        self.edges = int(L.beam_graph_num_edges(handle))
        self.arcs = int(L.beam_graph_num_arcs(handle))
        self.row_ptr = np.ctypeslib.as_array(L.beam_graph_row_ptr(handle), shape=(self.n + 1,)).copy()
        self.col_idx = (np.ctypeslib.as_array(L.beam_graph_col_idx(handle), shape=(self.arcs,)).copy()
                        if self.arcs else np.zeros(0, np.int32))

    @classmethod
    def generate(cls, spec: str) -> "Graph":
        return cls(N.lib().beam_graph_generate(spec.encode()))

    @classmethod
    def load_text(cls, path: str) -> "Graph":
        return cls(N.lib().beam_graph_load_text(str(path).encode()))

    @classmethod
    def load_binary(cls, path: str) -> "Graph":
        return cls(N.lib().beam_graph_load_binary(str(path).encode()))

    @classmethod
    def from_edges(cls, u, v) -> "Graph":
        u = np.ascontiguousarray(u, dtype=np.int32)
        v = np.ascontiguousarray(v, dtype=np.int32)
        return cls(N.lib().beam_graph_from_edges(_ptr(u, C.c_int32), _ptr(v, C.c_int32), len(u)))

    def edge_list(self) -> tuple[np.ndarray, np.ndarray]:
        L = N.lib()
        u = np.ctypeslib.as_array(L.beam_graph_edge_u(self._h), shape=(self.edges,)).copy()
        v = np.ctypeslib.as_array(L.beam_graph_edge_v(self._h), shape=(self.edges,)).copy()
        return u, v

    def write_text(self, path: str) -> None:
        N.check(N.lib().beam_graph_write_text(self._h, str(path).encode()), "beam_graph_last_error")

    def write_binary(self, path: str) -> None:
        N.check(N.lib().beam_graph_write_binary(self._h, str(path).encode()), "beam_graph_last_error")

    def encode(self, head: np.ndarray, nxt: np.ndarray, out_dir: str | None = None) -> dict:
        enc = N.Encoding()
        head = np.ascontiguousarray(head, np.int32)
        nxt = np.ascontiguousarray(nxt, np.int32)
        N.check(N.lib().beam_encode(self.n, self.arcs, _ptr(self.row_ptr, C.c_int64), _ptr(self.col_idx, C.c_int32),
                                    _ptr(head, C.c_int32), _ptr(nxt, C.c_int32),
                                    None if out_dir is None else str(out_dir).encode(), C.byref(enc)),
                "beam_encode_last_error")
        return enc.as_dict()

    def exact_partition_cost(self, labels: np.ndarray) -> int:
        labels = np.ascontiguousarray(labels, np.int32)
        out = C.c_int64()
        N.check(N.lib().beam_exact_partition_cost(self.n, _ptr(self.row_ptr, C.c_int64),
                                                  _ptr(self.col_idx, C.c_int32), _ptr(labels, C.c_int32),
                                                  C.byref(out)), "beam_encode_last_error")
        return int(out.value)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            N.lib().beam_graph_free(h)
            self._h = None


def partition_hash(labels: np.ndarray) -> int:
    labels = np.ascontiguousarray(labels, np.int32)
    return int(N.lib().beam_partition_hash(len(labels), _ptr(labels, C.c_int32)))


@dataclass
class EngineOptions:
    top_k: int = 16
    group_batch_size: int = 64
    divide_hash_dims: int = 16
    divide_max_group: int = 512
    ea_use_threshold: bool = True
    seed: int = 1
    device: int = 0
    verify_cuda_gain: bool = False
    # learned candidate ranker (off: the reference's method)
    ranker: bool = False
    ranker_train_iters: int = 5
    ranker_recall: float = 0.99
    ranker_audit: bool = False
    ranker_max_samples: int = 1 << 18
    ranker_epochs: int = 4
    ranker_max_steps: int = 256
    ranker_lr: float = 3e-3


class Engine:
    """Device-resident merge loop for one graph (one GPU)."""

    def __init__(self, graph: Graph, options: EngineOptions | None = None, **kw):
        o = options or EngineOptions(**kw)
        cfg = N.EngineConfig()
        N.lib().beam_engine_default_config(C.byref(cfg))
        cfg.top_k, cfg.group_batch_size = o.top_k, o.group_batch_size
        cfg.divide_hash_dims, cfg.divide_max_group = o.divide_hash_dims, o.divide_max_group
        cfg.ea_use_threshold, cfg.seed, cfg.device = int(o.ea_use_threshold), o.seed, o.device
        cfg.verify_cuda_gain = int(o.verify_cuda_gain)
        cfg.ranker, cfg.ranker_train_iters, cfg.ranker_recall = int(o.ranker), o.ranker_train_iters, o.ranker_recall
        cfg.ranker_audit, cfg.ranker_max_samples = int(o.ranker_audit), o.ranker_max_samples
        cfg.ranker_epochs, cfg.ranker_max_steps, cfg.ranker_lr = o.ranker_epochs, o.ranker_max_steps, o.ranker_lr
        h = C.c_void_p()
        N.check(N.lib().beam_engine_create(graph.n, graph.arcs, _ptr(graph.row_ptr, C.c_int64),
                                           _ptr(graph.col_idx, C.c_int32), C.byref(cfg), C.byref(h)))
        self._h = h
        self.n = graph.n
        self.options = o

    def close(self) -> None:
        if getattr(self, "_h", None):
            N.lib().beam_engine_destroy(self._h)
            self._h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # Sweg::Run / Divide / Merge
    def reset(self) -> None:
        N.check(N.lib().beam_engine_reset(self._h))

    def run(self, iterations: int = 20) -> None:
        N.check(N.lib().beam_engine_run(self._h, iterations))

    def divide(self, iteration: int) -> None:
        N.check(N.lib().beam_engine_divide(self._h, iteration))

    def merge(self, iteration: int, total: int = 20) -> None:
        N.check(N.lib().beam_engine_merge(self._h, iteration, total))

    def groups(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        na, ng = C.c_int64(), C.c_int64()
        N.check(N.lib().beam_engine_group_counts(self._h, C.byref(na), C.byref(ng)))
        order = np.zeros(max(na.value, 1), np.int32)
        starts = np.zeros(max(ng.value, 1), np.int32)
        lengths = np.zeros(max(ng.value, 1), np.int32)
        N.check(N.lib().beam_engine_groups(self._h, _ptr(order, C.c_int32), _ptr(starts, C.c_int32),
                                           _ptr(lengths, C.c_int32)))
        return order[:na.value], starts[:ng.value], lengths[:ng.value]

    def score_pairs(self, a, b) -> tuple[np.ndarray, np.ndarray]:
        a = np.ascontiguousarray(a, np.int32)
        b = np.ascontiguousarray(b, np.int32)
        gain = np.zeros(len(a), np.int64)
        before = np.zeros(len(a), np.int64)
        N.check(N.lib().beam_engine_score_pairs(self._h, _ptr(a, C.c_int32), _ptr(b, C.c_int32), len(a),
                                                _ptr(gain, C.c_int64), _ptr(before, C.c_int64)))
        return gain, before

    def prepare_group(self, q) -> np.ndarray:
        q = np.ascontiguousarray(q, np.int32)
        cap = max(1, len(q) * max(1, self.options.top_k))
        a = np.zeros(cap, np.int32)
        b = np.zeros(cap, np.int32)
        cnt = C.c_int64()
        N.check(N.lib().beam_engine_prepare_group(self._h, _ptr(q, C.c_int32), len(q), _ptr(a, C.c_int32),
                                                  _ptr(b, C.c_int32), cap, C.byref(cnt)))
        return np.stack([a[:cnt.value], b[:cnt.value]], axis=1)

    def merge_pairs(self, keep, remove) -> None:
        keep = np.ascontiguousarray(keep, np.int32)
        remove = np.ascontiguousarray(remove, np.int32)
        N.check(N.lib().beam_engine_merge_pairs(self._h, _ptr(keep, C.c_int32), _ptr(remove, C.c_int32),
                                                len(keep)))

    def encode(self, out_dir: str | None = None) -> dict:
        """Sweg::Encode of the current partition on the device; writes the four
        files into out_dir when given."""
        enc = N.Encoding()
        N.check(N.lib().beam_engine_encode(self._h, None if out_dir is None else str(out_dir).encode(),
                                           C.byref(enc)))
        return enc.as_dict()

    def exact_partition_cost(self) -> int:
        """CostOracle::ExactPartitionCost of the current partition, on the device."""
        out = C.c_int64()
        N.check(N.lib().beam_engine_exact_partition_cost(self._h, C.byref(out)))
        return int(out.value)

    def validate_quotient(self) -> None:
        """QuotientGraph::ValidateAgainstOriginalGraph on the device: raises
        BeamError on the first difference from a full rebuild."""
        N.check(N.lib().beam_engine_validate_quotient(self._h))

    def ranker_info(self) -> dict:
        info = N.RankerInfo()
        N.check(N.lib().beam_engine_ranker_info(self._h, C.byref(info)))
        return info.as_dict()

    def partition(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        labels = np.zeros(self.n, np.int32)
        head = np.zeros(self.n, np.int32)
        nxt = np.zeros(self.n, np.int32)
        N.check(N.lib().beam_engine_partition(self._h, _ptr(labels, C.c_int32), _ptr(head, C.c_int32),
                                              _ptr(nxt, C.c_int32)))
        return labels, head, nxt

    def row(self, rep: int) -> tuple[np.ndarray, np.ndarray, int, int]:
        """(neighbours, counts, size, internal) of one supernode's quotient row."""
        ln, size, internal = C.c_int64(), C.c_int64(), C.c_int64()
        N.check(N.lib().beam_engine_export_row(self._h, rep, None, None, 0, C.byref(ln), C.byref(size),
                                               C.byref(internal)))
        nb = np.zeros(max(ln.value, 1), np.int32)
        cnt = np.zeros(max(ln.value, 1), np.int64)
        N.check(N.lib().beam_engine_export_row(self._h, rep, _ptr(nb, C.c_int32), _ptr(cnt, C.c_int64), ln.value,
                                               C.byref(ln), C.byref(size), C.byref(internal)))
        return nb[:ln.value], cnt[:ln.value], int(size.value), int(internal.value)

    def stats(self) -> dict:
        st = N.EngineStats()
        N.check(N.lib().beam_engine_get_stats(self._h, C.byref(st)))
        return st.as_dict()

    def quotient_nnz(self) -> int:
        out = C.c_int64()
        N.check(N.lib().beam_engine_quotient_nnz(self._h, C.byref(out)))
        return int(out.value)

    def set_timed_kernel(self, which: int) -> None:
        N.check(N.lib().beam_engine_set_timed_kernel(self._h, which))

    def timed_kernel(self) -> tuple[float, int]:
        ms, launches = C.c_double(), C.c_int64()
        N.check(N.lib().beam_engine_timed_kernel(self._h, C.byref(ms), C.byref(launches)))
        return float(ms.value), int(launches.value)

    def synchronize(self) -> None:
        N.check(N.lib().beam_engine_synchronize(self._h))

    def step_timer_start(self) -> None:
        N.check(N.lib().beam_engine_step_timer_start(self._h))

    def step_timer_stop(self) -> float:
        ms = C.c_double()
        N.check(N.lib().beam_engine_step_timer_stop(self._h, C.byref(ms)))
        return float(ms.value)

    def flush_l2(self) -> None:
        N.check(N.lib().beam_engine_flush_l2(self._h))

    def launch_count(self) -> int:
        out = C.c_int64()
        N.check(N.lib().beam_engine_launch_count(self._h, C.byref(out)))
        return int(out.value)


class FlatScorer:
    """Legacy-objective pair scoring over a flat per-block CSR on the GPU: the
    service behind the reference's Sweg::ScoreCandidatesCuda
    (src/cuda_scoring.cu:714-885) with --cost-objective legacy."""

    KEYS = {"offsets": np.int32, "reps": np.int32, "rsz": np.int64, "self": np.int64, "nb": np.int32,
            "wt": np.int64, "nsz": np.int64}

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        N.check(N.lib().beam_flat_scorer_create(device, C.byref(h)), "beam_flat_scorer_last_error")
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            N.lib().beam_flat_scorer_destroy(self._h)
            self._h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def score(self, flat: dict, pairs) -> tuple[np.ndarray, np.ndarray]:
        """{gain, before_cost} per (a_idx, b_idx) row pair, in pair order."""
        f = {k: np.ascontiguousarray(flat[k], t) for k, t in self.KEYS.items()}
        pairs = np.ascontiguousarray(np.asarray(pairs, np.int32).reshape(-1, 2))
        gain = np.zeros(len(pairs), np.int64)
        before = np.zeros(len(pairs), np.int64)
        N.check(N.lib().beam_flat_scorer_score(
            self._h, _ptr(pairs, C.c_int32), len(pairs), _ptr(f["offsets"], C.c_int32), _ptr(f["reps"], C.c_int32),
            _ptr(f["rsz"], C.c_int64), _ptr(f["self"], C.c_int64), len(f["reps"]), _ptr(f["nb"], C.c_int32),
            _ptr(f["wt"], C.c_int64), _ptr(f["nsz"], C.c_int64), len(f["nb"]), _ptr(gain, C.c_int64),
            _ptr(before, C.c_int64)), "beam_flat_scorer_last_error")
        return gain, before

    def stats(self) -> dict:
        st = N.FlatScorerStats()
        N.check(N.lib().beam_flat_scorer_get_stats(self._h, C.byref(st)), "beam_flat_scorer_last_error")
        return st.as_dict()


RANKER_FEATURES = 16
RANKER_PARAMS = 64 * 16 + 64 + 64 + 1


def ranker_grad(x, y, params, w=None, device: int = 0) -> tuple[np.ndarray, float, np.ndarray]:
    """One forward + backward pass of the ranker MLP on the GPU (the
    library's own kernels): gradient of the mean weighted logistic loss with
    respect to the fp32 master parameters, the loss, and the logits."""
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    params = np.ascontiguousarray(params, np.float32)
    n = len(y)
    if x.shape != (n, RANKER_FEATURES) or params.shape != (RANKER_PARAMS,):
        raise ValueError("x must be [n, 16] and params [1153]")
    wp = None
    if w is not None:
        w = np.ascontiguousarray(w, np.float32)
        wp = w.ctypes.data
    grad = np.zeros(RANKER_PARAMS, np.float32)
    logits = np.zeros(n, np.float32)
    loss = C.c_double()
    N.check(N.lib().beam_ranker_grad(device, x.ctypes.data, y.ctypes.data, wp, n, params.ctypes.data,
                                     grad.ctypes.data, C.byref(loss), logits.ctypes.data), "beam_ranker_last_error")
    return grad, float(loss.value), logits

