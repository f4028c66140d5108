// Reference-side adapter: compiled INTO the reference program in place of its
// CUDA scoring translation unit (src/cuda_scoring.cu, or
// src/cuda_scoring_stub.cpp when SWEG_ENABLE_CUDA is off; CMakeLists.txt:10,
// 18-31) and linked against libbeam_gb300.so, which also exports the two
// functions of include/cuda_scoring.hpp (CudaScoringBuildMode returns "cuda",
// CudaScoringCompiled returns true).
//
// It defines the Sweg members that translation unit must define
// (include/sweg.hpp:449, 452, 656-658, 684-686):
//   ~Sweg, CudaScoringCache, EnsureCudaScoringCache,
//   QueryCudaSliceMemoryBudgetBytes, GetCudaSliceMemoryBudgetBytes,
//   ScoreCandidatesCuda - legacy-objective scoring of one flat block on the
//                         GPU (beam_flat_scorer_score), the README's CUDA mode
//                         (--scoring-backend cuda --cost-objective legacy).
// Errors are thrown as std::runtime_error, which the reference's main prints as
// "Error: <message>" with exit code 1 (src/main.cpp:1489-1492).
//
// With BEAM_GB300_RUN_HOOK defined it also defines Sweg::RunOnGb300, the whole
// merge loop of the recommended mode (mags-compatible objective) on the GPU.
// That needs three edits on the reference side, listed in INTEGRATION.md: the
// declaration in include/sweg.hpp, a dispatch at the top of Sweg::Run, and the
// removal of the CLI guard that refuses --scoring-backend cuda with
// --cost-objective mags-compatible (src/main.cpp:436-440).

#include <algorithm>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "beam_gb300.h"
#include "cuda_scoring.hpp"
#include "sweg.hpp"

struct Sweg::CudaScoringCache {
  beam_flat_scorer* scorer = nullptr;
  size_t slice_memory_budget_bytes = 0;
  ~CudaScoringCache() { beam_flat_scorer_destroy(scorer); }
};

Sweg::~Sweg() = default;

void Sweg::EnsureCudaScoringCache() {
  if (cuda_cache_) return;
  auto cache = std::make_shared<CudaScoringCache>();
  if (beam_flat_scorer_create(0, &cache->scorer) != 0) {
    throw std::runtime_error(std::string("GB300 scoring backend: ") + beam_flat_scorer_last_error());
  }
  cuda_cache_ = std::move(cache);
}

// The library grows its buffers to each block, so the slice planner's budget
// only bounds how much of a 64-group block goes into one call; the GB300
// library's own rule sets it (a quarter of free device memory, at most 4 GiB).
size_t Sweg::QueryCudaSliceMemoryBudgetBytes() {
  EnsureCudaScoringCache();
  if (cuda_cache_->slice_memory_budget_bytes == 0) {
    int64_t bytes = 0;
    if (beam_flat_scorer_memory_budget(cuda_cache_->scorer, &bytes) != 0) {
      throw std::runtime_error(std::string("GB300 scoring backend: ") + beam_flat_scorer_last_error());
    }
    cuda_cache_->slice_memory_budget_bytes = static_cast<size_t>(bytes);
  }
  return cuda_cache_->slice_memory_budget_bytes;
}

size_t Sweg::GetCudaSliceMemoryBudgetBytes() {
  if (cuda_slice_memory_mb_ > 0) {
    return static_cast<size_t>(cuda_slice_memory_mb_) * 1024ULL * 1024ULL;
  }
  return QueryCudaSliceMemoryBudgetBytes();
}

// One flat block: every candidate pair is scored by one launch (the library's
// warp-per-pair kernel needs no chunking, so candidate_chunk_size only caps
// the pairs of one call). --verify-cuda-gain's host re-check is not run here:
// the library's results are checked against the reference's own host check
// function by its test suite instead.
std::vector<Sweg::LocalGainResult> Sweg::ScoreCandidatesCuda(const std::vector<std::pair<int, int>>& candidate_pairs,
                                                             const FlatAggCSR& flat_agg,
                                                             size_t candidate_chunk_size) {
  if (candidate_pairs.empty()) return {};
  EnsureCudaScoringCache();
  const size_t total = candidate_pairs.size();
  const size_t chunk = candidate_chunk_size == 0 ? total : std::max<size_t>(1, std::min(candidate_chunk_size, total));
  std::vector<int32_t> pairs(2 * total);
  for (size_t i = 0; i < total; ++i) {
    pairs[2 * i] = candidate_pairs[i].first;
    pairs[2 * i + 1] = candidate_pairs[i].second;
  }
  std::vector<int64_t> gain(total), before(total);
  beam_flat_scorer_stats st0{}, st1{};
  beam_flat_scorer_get_stats(cuda_cache_->scorer, &st0);
  stats_.cuda_num_calls += 1;
  for (size_t at = 0; at < total; at += chunk) {
    const size_t count = std::min(chunk, total - at);
    const int rc = beam_flat_scorer_score(
        cuda_cache_->scorer, pairs.data() + 2 * at, static_cast<int64_t>(count), flat_agg.offsets.data(),
        flat_agg.row_rep_ids.data(), flat_agg.row_sizes.data(), flat_agg.row_self_loops.data(),
        static_cast<int32_t>(flat_agg.row_rep_ids.size()), flat_agg.neighbors.data(), flat_agg.weights.data(),
        flat_agg.neighbor_sizes.data(), static_cast<int64_t>(flat_agg.neighbors.size()), gain.data() + at,
        before.data() + at);
    if (rc != 0) throw std::runtime_error(std::string("GB300 scoring backend: ") + beam_flat_scorer_last_error());
  }
  beam_flat_scorer_get_stats(cuda_cache_->scorer, &st1);
  stats_.cuda_kernel_launches += st1.kernel_launches - st0.kernel_launches;
  stats_.cuda_kernel_ms += st1.kernel_ms - st0.kernel_ms;
  stats_.cuda_h2d_bytes += st1.h2d_bytes - st0.h2d_bytes;
  stats_.cuda_d2h_bytes += st1.d2h_bytes - st0.d2h_bytes;
  stats_.cuda_packed_h2d_calls += st1.calls - st0.calls;
  stats_.cuda_packed_d2h_calls += st1.calls - st0.calls;
  stats_.cuda_row_uploads += st1.calls - st0.calls;
  stats_.cuda_max_candidates_per_launch = std::max<int64_t>(stats_.cuda_max_candidates_per_launch,
                                                            st1.max_pairs_per_launch);
  std::vector<LocalGainResult> out(total);
  for (size_t i = 0; i < total; ++i) {
    out[i].gain = gain[i];
    out[i].before_cost = before[i];
  }
  return out;
}

#ifdef BEAM_GB300_RUN_HOOK
// The merge loop of the recommended mode (Sweg::Run, src/sweg.cpp:651-709) on
// the GPU: the CSR goes up once, the iterations run on the device, and the
// partition comes back into S_ / I_ / J_ (labels, head member per rep or -1,
// next member or -1), after which the reference's Encode, metrics and the
// payload == ExactPartitionCost check run unchanged.
void Sweg::RunOnGb300(int iterations) {
  auto check = [](int rc) {
    if (rc != 0) throw std::runtime_error(beam_engine_last_error());
  };
  beam_engine_config cfg;
  beam_engine_default_config(&cfg);
  cfg.top_k = top_k_;
  cfg.group_batch_size = merge_mode_ == MergeMode::kBatchEncodingAware ? 1 : group_batch_size_;
  cfg.divide_hash_dims = divide_hash_dims_;
  cfg.divide_max_group = divide_max_group_;
  cfg.ea_use_threshold = ea_use_threshold_ ? 1 : 0;
  cfg.seed = seed64_;
  cfg.verify_cuda_gain = verify_cuda_gain_ ? 1 : 0;
  beam_engine* e = nullptr;
  check(beam_engine_create(graph_->n, static_cast<int64_t>(graph_->col_idx.size()), graph_->row_ptr.data(),
                           graph_->col_idx.data(), &cfg, &e));
  std::unique_ptr<beam_engine, void (*)(beam_engine*)> owner(e, beam_engine_destroy);
  check(beam_engine_run(e, iterations));
  check(beam_engine_partition(e, S_.data(), I_.data(), J_.data()));
  beam_engine_stats st;
  check(beam_engine_get_stats(e, &st));
  stats_.runtime_run_ms = st.runtime_run_ms;
  stats_.runtime_divide_ms = st.runtime_divide_ms;
  stats_.runtime_merge_ms = st.runtime_merge_ms;
  stats_.merge_group_count = st.merge_group_count;
  stats_.merge_group_max_size = st.merge_group_max_size;
  stats_.merge_raw_pair_count = st.merge_raw_pair_count;
  stats_.merge_candidate_pairs_after_prune = st.merge_candidate_pairs_after_prune;
  stats_.merge_exact_gain_calls = st.merge_exact_gain_calls;
  stats_.merge_positive_gain_pairs = st.merge_positive_gain_pairs;
  stats_.merge_rejected_by_threshold = st.merge_rejected_by_threshold;
  stats_.merge_rejected_by_overlap = st.merge_rejected_by_overlap;
  stats_.merge_candidate_pairs = static_cast<int64_t>(st.merge_candidate_pairs);
  stats_.merge_selected_pairs = static_cast<int64_t>(st.merge_selected_pairs);
  stats_.merge_total_local_gain = static_cast<int64_t>(st.merge_total_local_gain);
  stats_.selected_merges_for_validation = st.selected_merges_for_validation;
  stats_.accepted_merges_after_validation = st.accepted_merges_after_validation;
  stats_.rejected_nonpositive = st.rejected_nonpositive;
  stats_.validation_exact_calls = st.validation_exact_calls;
  stats_.update_touched_quotient_entries = st.update_touched_quotient_entries;
  stats_.quotient_nnz_final = 0;
  for (int v = 0; v < n_; ++v) supernode_sizes_by_rep_[v] = 0;
  for (int v = 0; v < n_; ++v) ++supernode_sizes_by_rep_[S_[v]];
}
#endif
