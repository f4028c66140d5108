/*
 * beam_gb300 C ABI: a GB300 (sm_103a) implementation of BEAM's merge loop in
 * its recommended mode (batch-ea-blocked, mags-compatible objective,
 * persistent quotient graph with incremental update, legacy candidate index,
 * certification off, g0 commit).
 *
 * Plain pointers and sizes only. Every function that can fail returns an int
 * status (0 = success, negative = error) and leaves a message readable with
 * the matching *_last_error() call; the CLI turns it into the reference's
 * "Error: <message>" exit-1 behaviour (src/main.cpp:1489-1492).
 *
 * Reference interfaces replaced (paths inside githubofzby/beam):
 *   beam_graph_*            -> LoadUndirectedEdgeList / CSRGraph
 *                              (src/graph_io/graph_io.cpp:12-106,
 *                               include/graph_io/graph.hpp:8-29)
 *   beam_engine_create      -> Sweg::Sweg with persistent state
 *                              (src/sweg.cpp:102-194) and
 *                              QuotientGraph::Initialize (src/quotient_graph.cpp:72-145)
 *   beam_engine_run         -> Sweg::Run (src/sweg.cpp:651-709)
 *   beam_engine_divide      -> Sweg::Divide (src/sweg.cpp:853-890)
 *   beam_engine_merge       -> Sweg::Merge, blocked mode (src/sweg.cpp:953-1145)
 *   beam_engine_score_pairs -> Sweg::ScoreCandidatesCuda's role behind
 *                              --scoring-backend cuda (include/sweg.hpp:656-658,
 *                              src/cuda_scoring.cu:714-885), computing
 *                              QuotientGraph::ExactMergeGainPersistent
 *                              (src/quotient_graph.cpp:340-470)
 *   beam_engine_merge_pairs -> Sweg::Update_S + QuotientGraph::Merge
 *                              (src/sweg.cpp:2977-3015, src/quotient_graph.cpp:628-742)
 *   beam_engine_partition   -> Sweg::CurrentPartitionLabels / Recover_S
 *                              (src/sweg.cpp:2902-2975)
 *   beam_engine_export_row  -> QuotientGraph::GetRowView (src/quotient_graph.cpp:596-616)
 *   beam_engine_stats       -> RuntimeStats (include/sweg.hpp:221-386)
 *
 * The two C++-linkage functions of include/cuda_scoring.hpp in the reference
 * (CudaScoringBuildMode, CudaScoringCompiled) are exported with their exact
 * mangled signatures as well; see include/cuda_scoring.hpp in this tree.
 */
#ifndef BEAM_GB300_H_
#define BEAM_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- graphs */

typedef struct beam_graph beam_graph;

/* Seeded synthetic graph. spec = "<kind>:k=v,..." with kind one of
 *   rmat    (scale, ef, a, b, c, seed)
 *   dcsbm   (n, blocks, ratio, gamma, deg, seed)
 *   chunglu (n, gamma, deg, maxratio, twins, seed)
 *   union   (side, del, diag, n, gamma, deg, maxdeg, seed)
 *   grid    (side, del, diag, seed)
 *   gnm     (n, m, seed)
 * Every kind also takes relabel=0/1 (default 0: ids kept, n = max id + 1).
 * Edges are deduplicated and loop-free. NULL on error. */
beam_graph* beam_graph_generate(const char* spec);
/* Reference-compatible text edge list (src/graph_io/graph_io.cpp:12-106). */
beam_graph* beam_graph_load_text(const char* path);
/* Binary edge list: int64 E, then E pairs of int32 (u, v). */
beam_graph* beam_graph_load_binary(const char* path);
/* Graph from explicit undirected edges (one entry per edge). */
beam_graph* beam_graph_from_edges(const int32_t* u, const int32_t* v, int64_t edges);
int beam_graph_write_text(const beam_graph* g, const char* path);
int beam_graph_write_binary(const beam_graph* g, const char* path);
int64_t beam_graph_num_nodes(const beam_graph* g);
int64_t beam_graph_num_edges(const beam_graph* g); /* input_edges_raw */
int64_t beam_graph_num_arcs(const beam_graph* g);  /* 2 * edges */
const int64_t* beam_graph_row_ptr(const beam_graph* g); /* n + 1 */
const int32_t* beam_graph_col_idx(const beam_graph* g); /* arcs, sorted per row */
const int32_t* beam_graph_edge_u(const beam_graph* g);
const int32_t* beam_graph_edge_v(const beam_graph* g);
void beam_graph_free(beam_graph* g);
const char* beam_graph_last_error(void);

/* ---------------------------------------------------------------- engine */

typedef struct beam_engine beam_engine;

/* Flags of the recommended mode (src/main.cpp:14-56 defaults in brackets). */
typedef struct {
  int32_t top_k;             /* --top-k [16] */
  int32_t group_batch_size;  /* --group-batch-size [64] */
  int32_t divide_hash_dims;  /* --divide-hash-dims [16] */
  int32_t divide_max_group;  /* --divide-max-group [512], at most 1024 */
  int32_t ea_use_threshold;  /* --ea-use-threshold (reciprocal policy) */
  int32_t device;            /* CUDA device ordinal */
  uint64_t seed;             /* --seed [1] */
  int32_t verify_cuda_gain;  /* --verify-cuda-gain: re-score and check every commit */
  /* Learned candidate ranker (this implementation's own; 0 = the reference's method). */
  int32_t ranker;              /* 1: prune candidates before exact scoring after training */
  int32_t ranker_train_iters;  /* iterations whose exact gains are logged for training [5] */
  float ranker_recall;         /* recall of logged positives kept at the cutoff [0.99] */
  int32_t ranker_audit;        /* 1: also score pruned pairs aside and count the positives lost */
  int32_t ranker_max_samples;  /* training log capacity [262144] */
  int32_t ranker_epochs;       /* passes over the log [4] */
  int32_t ranker_max_steps;    /* Adam steps at most [256] */
  float ranker_lr;             /* Adam learning rate [0.003] */
} beam_engine_config;

/* Counters with the reference's metric names (include/sweg.hpp:221-386). */
typedef struct {
  double runtime_run_ms, runtime_divide_ms, runtime_merge_ms;
  uint64_t merge_group_count, merge_group_max_size, merge_raw_pair_count;
  uint64_t merge_candidate_pairs_after_prune, candidate_proxy_pairs_examined;
  uint64_t merge_exact_gain_calls, exact_gain_input_nnz;
  uint64_t exact_raw_entries_a, exact_raw_entries_b, exact_union_neighbors, exact_overlap_neighbors;
  uint64_t merge_positive_gain_pairs, merge_rejected_by_threshold, merge_rejected_by_overlap;
  uint64_t merge_candidate_pairs, merge_selected_pairs, merge_total_local_gain;
  uint64_t selected_merges_for_validation, validation_exact_calls, validation_exact_row_entry_work;
  uint64_t accepted_merges_after_validation, rejected_nonpositive, update_touched_quotient_entries;
  uint64_t isolated_gain_sum, divide_max_group_size, divide_fallback_splits;
  /* this implementation's own counters */
  uint64_t rows_rewritten, row_entries_rewritten;
  uint64_t score_bytes, prepare_bytes, update_bytes, divide_bytes; /* algorithmic HBM bytes */
  uint64_t blocks, iterations, pool_compactions, active_supernodes, groups_last;
} beam_engine_stats;

/* Kernel classes for beam_engine_set_timed_kernel. */
enum { BEAM_TIME_NONE = 0, BEAM_TIME_SCORE = 1, BEAM_TIME_PREPARE = 2, BEAM_TIME_UPDATE = 3, BEAM_TIME_DIVIDE = 4 };

void beam_engine_default_config(beam_engine_config* cfg);
/* Uploads the HOST CSR (row_ptr[n+1], col_idx[arcs], sorted rows, no loops)
 * to the device and builds the singleton quotient graph. */
int beam_engine_create(int32_t n, int64_t arcs, const int64_t* row_ptr, const int32_t* col_idx,
                       const beam_engine_config* cfg, beam_engine** out);
void beam_engine_destroy(beam_engine* e);
/* Back to the singleton partition, rebuilt from the resident CSR. */
int beam_engine_reset(beam_engine* e);
int beam_engine_run(beam_engine* e, int32_t iterations);
int beam_engine_divide(beam_engine* e, int32_t iter);
int beam_engine_merge(beam_engine* e, int32_t iter, int32_t total_iterations);
/* Divide output: active reps in group order, group starts and lengths. */
int beam_engine_group_counts(beam_engine* e, int64_t* n_active, int64_t* n_groups);
int beam_engine_groups(beam_engine* e, int32_t* order, int32_t* starts, int32_t* lengths);
/* Exact merge gain and before-cost for explicit pairs of active reps. */
int beam_engine_score_pairs(beam_engine* e, const int32_t* rep_a, const int32_t* rep_b, int64_t count,
                            int64_t* gain, int64_t* before);
/* EA-proxy candidates (a_idx < b_idx, sorted) of one explicit group; the
 * Divide output is consumed (call beam_engine_divide again before merging). */
int beam_engine_prepare_group(beam_engine* e, const int32_t* q, int32_t g, int32_t* a_idx, int32_t* b_idx,
                              int64_t cap, int64_t* count);
/* Applies endpoint-disjoint merges (keep, remove) as one batch. */
int beam_engine_merge_pairs(beam_engine* e, const int32_t* keep, const int32_t* remove, int64_t count);
/* node -> rep labels, head[rep] (-1 when inactive) and next[node] member lists. */
int beam_engine_partition(beam_engine* e, int32_t* labels, int32_t* head, int32_t* next);
int beam_engine_export_row(beam_engine* e, int32_t rep, int32_t* nb, int64_t* cnt, int64_t cap, int64_t* len,
                           int64_t* size, int64_t* internal);
int beam_engine_get_stats(beam_engine* e, beam_engine_stats* out);

/* Learned candidate ranker of the current run. */
typedef struct {
  uint64_t samples;        /* logged (features, label) rows */
  uint64_t positives;      /* rows labelled positive: exact gain > 0, gain/before >= 1/(iterations+1) */
  uint64_t train_steps;    /* Adam steps */
  uint64_t ranked;         /* candidate pairs ranked in the ranking iterations */
  uint64_t pruned;         /* of which not scored */
  uint64_t audit_passing;  /* ranker_audit: ranked pairs passing the iteration's threshold filter */
  uint64_t audit_lost;     /* ranker_audit: pruned pairs among them */
  double train_ms;         /* training + calibration, host wall time */
  double first_loss, final_loss;  /* weighted logistic loss of the first and last mini-batch */
  double cutoff;           /* logit cutoff */
  double calib_recall;     /* recall of the logged positives at the cutoff */
  double calib_prune;      /* fraction of the log below the cutoff */
  int32_t trained;
  int32_t reserved;
} beam_ranker_info;
int beam_engine_ranker_info(beam_engine* e, beam_ranker_info* out);

/* One forward + backward pass of the ranker's MLP on `device` over n samples
 * (x[n][16] features used as given, y[n] labels in {0,1}, w[n] sample
 * weights or NULL for 1): params[1153] = W1[64][16] | b1[64] | w2[64] | b2
 * (fp32 master; the forward pass uses the weights rounded to bf16). Writes
 * the gradient of the mean weighted logistic loss w.r.t. params, the loss
 * and (if logits != NULL) the n logits. The gradient check against the CPU
 * oracle runs through this entry. */
int beam_ranker_grad(int32_t device, const float* x, const float* y, const float* w, int64_t n,
                     const float* params, float* grad, double* loss, float* logits);
const char* beam_ranker_last_error(void);
/* CostOracle::ExactPartitionCost (src/cost_oracle.cpp:112-124) of the
 * engine's current partition, computed on the device from the resident input
 * graph (sort of supernode-pair keys + run-length encode); the check of
 * src/main.cpp:560-566 compares it with the encoding payload. */
/* QuotientGraph::ValidateAgainstOriginalGraph (src/quotient_graph.cpp:867-886),
 * --validate-quotient: the resident quotient graph (sizes, internal counts,
 * every row) against a full rebuild from the current labels, and its exact
 * cost against CostOracle::ExactPartitionCost. Fails with the reference's
 * message on the first mismatch. */
int beam_engine_validate_quotient(beam_engine* e);
int beam_engine_exact_partition_cost(beam_engine* e, int64_t* cost);
/* QuotientGraph::Nnz (src/quotient_graph.cpp:259-270). */
int beam_engine_quotient_nnz(beam_engine* e, int64_t* nnz);
/* CUDA-event timing of every launch of one kernel class (BEAM_TIME_*). */
int beam_engine_set_timed_kernel(beam_engine* e, int32_t which);
int beam_engine_timed_kernel(beam_engine* e, double* ms, int64_t* launches);
int beam_engine_synchronize(beam_engine* e);
/* CUDA events on the engine stream around a span of work (benchmarking). */
int beam_engine_step_timer_start(beam_engine* e);
int beam_engine_step_timer_stop(beam_engine* e, double* ms);
/* Overwrites a 256 MB device buffer so the next step starts with a cold L2. */
int beam_engine_flush_l2(beam_engine* e);
/* Kernels of this library launched by the engine since creation. */
int beam_engine_launch_count(beam_engine* e, int64_t* launches);
const char* beam_engine_last_error(void);

/* ------------------------------------------- no-allocation prepare step */

/* EA-proxy candidate pairs of ONE group, for callers that cannot allocate
 * device memory (a host that forbids cudaMalloc, a stream that must not see
 * an allocation's implicit synchronisation, an embedder with a fixed memory
 * budget). No counterpart in the reference: it is this library's own
 * allocation-free form of the prepare step.
 *
 * Every pointer is DEVICE memory owned by the caller. Inputs follow the
 * reference's flat per-group CSR (Sweg::FlatAggCSR): member i has reps
 * row_rep_ids[i], size row_sizes[i], internal edge count row_internal[i] and
 * row entries neighbors / weights / neighbor_sizes [offsets[i], offsets[i+1]);
 * offsets has rows + 1 entries and offsets[rows] == num_entries. Output: the
 * candidate pairs (a_idx < b_idx, ascending) in out_a_idx / out_b_idx and
 * their number in *out_count; out_capacity must be at least
 * min(rows*(rows-1)/2, rows*top_k). stream is a cudaStream_t (NULL = legacy
 * default stream); the call waits for its kernel before returning.
 *
 * Limits: rows <= 256, num_entries <= 65536, 1 <= top_k <= 32; other
 * requests fail with a message and launch nothing. Every weight must lie in
 * [0, 2^32): the kernel stages counts as 32-bit words, and a call with a
 * weight outside that range fails with a message (*out_count = -1), as does
 * one whose offsets do not rise from 0 to num_entries or whose row_rep_ids
 * repeat. The scratch is one static device
 * array of about 3 MB, resident on every GPU that loads the library until the
 * process exits, shared by all calls: its contents stay from the last call
 * (the kernel clears what must start at zero) and calls that overlap on the
 * GPU race. The call reads its status back and waits for its stream, so it
 * cannot be captured in a CUDA graph: on a capturing stream it fails with a
 * message and enqueues nothing. */
int beam_prepare_flat_noalloc(const int32_t* offsets, const int32_t* row_rep_ids, const int32_t* neighbors,
                              const int64_t* weights, const int64_t* neighbor_sizes, const int64_t* row_sizes,
                              const int64_t* row_internal, int32_t rows, int64_t num_entries, int32_t top_k,
                              int32_t* out_a_idx, int32_t* out_b_idx, int64_t out_capacity, int32_t* out_count,
                              void* stream);
const char* beam_prepare_flat_noalloc_last_error(void);

/* ------------------------------------- legacy-objective flat pair scoring */

/* The scoring service of the reference's CUDA mode with --cost-objective
 * legacy: Sweg::ScoreCandidatesCuda(pairs, FlatAggCSR, chunk)
 * (include/sweg.hpp:656-658, src/cuda_scoring.cu:714-885; per-pair
 * arithmetic of ComputeLocalGainKernel, src/cuda_scoring.cu:282-357). A
 * scorer owns a stream and device / pinned staging buffers that grow to the
 * largest call, like the reference's CudaScoringCache
 * (src/cuda_scoring.cu:369-533). */
typedef struct beam_flat_scorer beam_flat_scorer;

typedef struct {
  int64_t calls, kernel_launches, pairs, h2d_bytes, d2h_bytes, max_pairs_per_launch;
  double kernel_ms;
} beam_flat_scorer_stats;

int beam_flat_scorer_create(int32_t device, beam_flat_scorer** out);
void beam_flat_scorer_destroy(beam_flat_scorer* s);
int beam_flat_scorer_get_stats(const beam_flat_scorer* s, beam_flat_scorer_stats* out);
/* Device-memory budget for one call of a 64-group block's slice, replacing
 * Sweg::QueryCudaSliceMemoryBudgetBytes (src/cuda_scoring.cu:684-703): a
 * quarter of the device's free memory, at most 4 GiB. */
int beam_flat_scorer_memory_budget(beam_flat_scorer* s, int64_t* bytes);
/* HOST buffers in and out (the reference's std::vector contents):
 * pairs = count (a_idx, b_idx) row-index pairs; the FlatAggCSR arrays
 * (include/sweg.hpp:395-403) with rows + 1 offsets rising from 0 to entries
 * and each row sorted by neighbour without repeats; gain / before_cost get
 * one value per pair, in pair order (Sweg::LocalGainResult). The layout is
 * checked before anything is launched; a violation fails with a message. */
int beam_flat_scorer_score(beam_flat_scorer* s, const int32_t* pairs, int64_t count, const int32_t* offsets,
                           const int32_t* row_rep_ids, const int64_t* row_sizes, const int64_t* row_self_loops,
                           int32_t rows, const int32_t* neighbors, const int64_t* weights,
                           const int64_t* neighbor_sizes, int64_t entries, int64_t* gain, int64_t* before_cost);
const char* beam_flat_scorer_last_error(void);

/* ------------------------------------------------------- summary output */

typedef struct {
  int64_t supernodes, p, cp, cm, superedges_loop, superedges_nonloop;
  int64_t encoding_cost_standard, encoding_cost_mags_x2;
  double cost_ratio_standard, cost_ratio_mags_compatible;
} beam_encoding;

/* Sweg::Encode (src/sweg.cpp:3017-3163) + WriteOutput (src/sweg.cpp:3255-3287)
 * of the engine's current partition, computed on the device (pair-key radix
 * sort, run-length encode, per-block decision, Cm enumeration); writes
 * G.txt, P.txt, Cp.txt, Cm.txt into out_dir when not NULL. Same files and
 * metrics as beam_encode. */
int beam_engine_encode(beam_engine* e, const char* out_dir, beam_encoding* out);

/* Sweg::Encode (mags-compatible) of the partition given as member lists
 * (head[rep] = -1 for inactive reps, next[node]), plus the compression
 * metrics; writes G.txt, P.txt, Cp.txt, Cm.txt into out_dir when not NULL. */
int beam_encode(int32_t n, int64_t arcs, const int64_t* row_ptr, const int32_t* col_idx, const int32_t* head,
                const int32_t* next, const char* out_dir, beam_encoding* out);
/* CostOracle::ExactPartitionCost of a node -> label partition. */
int beam_exact_partition_cost(int32_t n, const int64_t* row_ptr, const int32_t* col_idx, const int32_t* labels,
                              int64_t* cost);
/* Sweg::PartitionHash: FNV-1a over the node -> rep labels. */
uint64_t beam_partition_hash(int32_t n, const int32_t* labels);
const char* beam_encode_last_error(void);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif  /* BEAM_GB300_H_ */
