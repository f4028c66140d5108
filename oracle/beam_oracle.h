/*
 * ORACLE — test infrastructure only. A plain-C CPU restatement of BEAM's merge
 * loop in its recommended mode (githubofzby/beam: batch-ea-blocked,
 * mags-compatible CostOracle, persistent QuotientGraph, incremental update,
 * legacy candidate index, certification off, g0 commit), used as the checker
 * for the GPU path and as the timed CPU baseline. Nothing in the product
 * library may link or call it.
 *
 * Parity is pinned against the reference program itself (built from its
 * sources by `make -C oracle ref`) on the fixtures in tests/golden/.
 */
#ifndef BEAM_ORACLE_H_
#define BEAM_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct beam_oracle beam_oracle;

typedef struct {
  int top_k;             /* --top-k, default 16 */
  int group_batch_size;  /* --group-batch-size, default 64 */
  int divide_hash_dims;  /* --divide-hash-dims, default 16 */
  int divide_max_group;  /* --divide-max-group, default 512 */
  int ea_use_threshold;  /* --ea-use-threshold */
  uint64_t seed;         /* --seed */
  int threads;           /* OpenMP threads, 0 = runtime default */
} beam_oracle_config;

typedef struct {
  double runtime_run_ms, runtime_divide_ms, runtime_merge_ms;
  double merge_prepare_wall_ms, merge_gain_scoring_ms, merge_selection_ms, merge_update_ms;
  int64_t divide_max_group_size, divide_fallback_splits;
  uint64_t merge_group_count, merge_group_max_size, merge_raw_pair_count;
  uint64_t merge_candidate_pairs_after_prune, merge_exact_gain_calls;
  uint64_t merge_positive_gain_pairs, merge_rejected_by_threshold, merge_rejected_by_overlap;
  int64_t merge_candidate_pairs, merge_selected_pairs, merge_total_local_gain;
  uint64_t selected_merges_for_validation, accepted_merges_after_validation;
  uint64_t rejected_nonpositive, stale_endpoint, validation_exact_calls;
  uint64_t validation_exact_row_entry_work, update_touched_quotient_entries;
  uint64_t candidate_proxy_pairs_examined, exact_gain_input_nnz;
  uint64_t exact_raw_entries_a, exact_raw_entries_b, exact_union_neighbors;
  uint64_t exact_overlap_neighbors, quotient_nnz_final;
  int64_t isolated_gain_sum;
  uint64_t groups_last, active_supernodes_last;
} beam_oracle_stats;

typedef struct {
  int64_t n_supernodes, p, cp, cm;
  int64_t encoding_cost_mags_x2;
  double cost_ratio_mags_compatible;
  int64_t num_superedges_loop, num_superedges_nonloop;
} beam_oracle_encoding;

void beam_oracle_default_config(beam_oracle_config* cfg);
/* CSR is borrowed and must outlive the oracle. NULL on error. */
beam_oracle* beam_oracle_create(int32_t n, int64_t arcs, const int64_t* row_ptr,
                                const int32_t* col_idx, const beam_oracle_config* cfg);
void beam_oracle_free(beam_oracle* o);
const char* beam_oracle_last_error(void);

int beam_oracle_run(beam_oracle* o, int iterations);
int beam_oracle_divide(beam_oracle* o, int iter);
int beam_oracle_merge(beam_oracle* o, int iter, int total_iterations);
/* The blocks of Merge(iter) that start at group first_group (a block
 * boundary), in order, until budget_ms of wall time has run out at a block
 * boundary (budget_ms <= 0: to the end): a bounded sample of an iteration for
 * timing. *next_group = the first group of the next unprocessed block. */
int beam_oracle_merge_blocks(beam_oracle* o, int iter, int64_t first_group, double budget_ms,
                             int64_t* next_group);

/* Divide output: order[] holds the active reps in group order (length =
 * active count), starts[] the group starts (length = group count). */
int64_t beam_oracle_group_count(const beam_oracle* o);
int64_t beam_oracle_active_count(const beam_oracle* o);
int beam_oracle_groups(const beam_oracle* o, int32_t* order, int32_t* starts, int32_t* lengths);

/* EA-proxy candidate pairs of one group q[0..g) against the current state:
 * writes up to cap (a_idx, b_idx) pairs, returns the count or < 0. */
int64_t beam_oracle_prepare_group(beam_oracle* o, const int32_t* q, int32_t g,
                                  int32_t* a_idx, int32_t* b_idx, int64_t cap);
/* QuotientGraph::ExactMergeGainPersistent(a, b). */
int beam_oracle_exact_gain(const beam_oracle* o, int32_t a, int32_t b, int64_t* gain,
                           int64_t* before);
/* Sweg::Update_S(keep, remove) (quotient merge + partition lists). */
int beam_oracle_merge_pair(beam_oracle* o, int32_t keep, int32_t remove);

/* node -> representative labels (n entries). */
int beam_oracle_labels(const beam_oracle* o, int32_t* labels);
/* member lists in linked-list order: head[rep] (-1 if inactive), next[node]. */
int beam_oracle_member_lists(const beam_oracle* o, int32_t* head, int32_t* next);
uint64_t beam_oracle_partition_hash(const beam_oracle* o);
int beam_oracle_active(const beam_oracle* o, int32_t rep);
int64_t beam_oracle_size(const beam_oracle* o, int32_t rep);
int64_t beam_oracle_internal(const beam_oracle* o, int32_t rep);
/* row of rep: writes up to cap entries, returns the row length. */
int64_t beam_oracle_row(const beam_oracle* o, int32_t rep, int32_t* nb, int64_t* cnt, int64_t cap);
int64_t beam_oracle_exact_partition_cost(const beam_oracle* o);
void beam_oracle_get_stats(const beam_oracle* o, beam_oracle_stats* out);

/* Legacy-objective local gain of rows a and b of a flat per-block CSR
 * (Sweg::FlatAggCSR), as the reference's CUDA mode scores pairs
 * (src/cuda_scoring.cu:146-252, 282-357). */
int beam_oracle_legacy_flat_gain(const int32_t* offsets, const int32_t* reps, const int64_t* row_sizes,
                                 const int64_t* self_loops, const int32_t* nb, const int64_t* wt,
                                 const int64_t* nsz, int32_t a, int32_t b, int64_t* gain, int64_t* before);

/* Sweg::Encode + ComputeCompressionMetrics (mags-compatible). When dir is not
 * NULL, writes G.txt / P.txt / Cp.txt / Cm.txt there. */
int beam_oracle_encode(beam_oracle* o, const char* dir, beam_oracle_encoding* out);

#ifdef __cplusplus
}
#endif

#endif /* BEAM_ORACLE_H_ */
