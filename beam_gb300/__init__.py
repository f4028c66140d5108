"""GB300 (sm_103a) implementation of BEAM's merge loop (githubofzby/beam,
recommended mode) behind the reference's C/C++ interfaces.

The compute path is libbeam_gb300.so (hand-written CUDA kernels + C++
runtime); this package only binds it.
"""

from .engine import Engine, EngineOptions, FlatScorer, Graph, partition_hash, ranker_grad

# Seeded synthetic stand-ins for the five workloads of the benchmark plan.
WORKLOADS = {
    "dcsbm_4096": "dcsbm:n=4096,blocks=32,ratio=40,gamma=2.5,deg=43,seed=1",
    "rmat19": "rmat:scale=19,ef=2,a=0.57,b=0.19,c=0.19,seed=7",
    "grid_chunglu_union": "union:side=1400,del=0.10,diag=0.02,n=1100000,gamma=2.1,deg=5.4,maxdeg=28000,seed=3",
    "chunglu4m_twins": "chunglu:n=4000000,gamma=2.3,deg=17,twins=200000,seed=4",
    "rmat24": "rmat:scale=24,ef=16,a=0.57,b=0.19,c=0.19,seed=11",
    # the same generator at scale 20 (n = 1M, m = 16M): the profiling size of
    # the scale-24 graph, larger than L2 yet a few GB on the device
    "rmat20_ef16": "rmat:scale=20,ef=16,a=0.57,b=0.19,c=0.19,seed=11",
}

# The reference's recommended flags (--ea-use-threshold, reciprocal policy,
# top-k 16, group batch 64, 20 iterations, seed 1).
REFERENCE_FLAGS = [
    "--merge-mode", "batch-ea-blocked", "--scoring-backend", "cpu", "--cost-objective", "mags-compatible",
    "--state-backend", "persistent", "--quotient-update", "incremental", "--candidate-index", "legacy",
    "--certification", "off", "--commit-policy", "g0", "--top-k", "16", "--group-batch-size", "64",
    "--ea-use-threshold", "--threshold-policy", "reciprocal", "--iterations", "20", "--print-offset", "0",
    "--seed", "1", "--error-bound", "0.0",
]

__all__ = ["Engine", "EngineOptions", "FlatScorer", "Graph", "partition_hash", "ranker_grad", "WORKLOADS", "REFERENCE_FLAGS"]
