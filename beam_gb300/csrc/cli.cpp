// `beam` command line for the GB300 merge loop. Flags, banner lines and
// metric.k=v output follow the reference CLI (src/main.cpp:14-110, 327-423,
// 489-740); the mags-compatible / --scoring-backend cuda guard of
// src/main.cpp:436-440 is lifted because this library is that backend. Modes
// outside the recommended one are rejected with an error, as the reference
// rejects unsupported combinations.

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "beam_gb300.h"
#include "cuda_scoring.hpp"

namespace {

struct Options {
  std::string input;
  std::string merge_mode = "batch-ea";
  std::string scoring_backend = "cpu";
  std::string cost_objective = "legacy";
  std::string state_backend = "legacy";
  std::string quotient_update = "incremental";
  std::string candidate_index = "legacy";
  std::string certification = "off";
  std::string commit_policy = "g0";
  std::string threshold_policy = "reciprocal";
  std::string profiling = "off";
  std::string out_dir;
  std::string results_csv;
  std::string profile_csv;
  int candidate_budget = 8;
  int candidate_batch_budget = 0;
  int cuda_slice_memory_mb = 0;
  int overflow_group_gmax = 0;
  int overflow_refine_rounds = 0;
  bool validate_quotient = false;
  bool commit_audit = false;
  int top_k = 16;
  int group_batch_size = 64;
  int iterations = 20;
  int print_offset = 1;
  int divide_hash_dims = 16;
  int divide_max_group = 512;
  bool ea_use_threshold = false;
  bool write_output = false;
  bool verify_cuda_gain = false;
  bool ranker = false;
  bool ranker_audit = false;
  double ranker_recall = 0.99;
  int ranker_train_iters = 5;
  bool show_help = false;
  double error_bound = 0.0;
  uint64_t seed = 1;
  int device = 0;
};

void PrintUsage() {
  std::cout << "Usage:\n"
            << "  beam --input <undirected-single-edge-list> [options]\n\n"
            << "GB300 build of the recommended mode: --merge-mode batch-ea-blocked\n"
            << "--scoring-backend cuda --cost-objective mags-compatible --state-backend persistent\n"
            << "--quotient-update incremental --candidate-index legacy --certification off\n"
            << "--commit-policy g0 --threshold-policy reciprocal [--ea-use-threshold]\n"
            << "(--merge-mode batch-ea: the same with one group per block)\n"
            << "Other options: --top-k --group-batch-size --iterations --print-offset --divide-hash-dims\n"
            << "--divide-max-group --seed --error-bound 0 --write-output --out <dir> --device\n"
            << "--results-csv <path> --profiling off|summary|rounds --profile-csv <path> --validate-quotient\n"
            << "--ranker [--ranker-recall r] [--ranker-train-iters k] [--ranker-audit]: learned candidate ranker\n"
            << "Input: text edge list 'u v' per line, or a binary edge list with a .bin suffix.\n";
}

std::string FormatDouble(double v) {
  std::ostringstream oss;
  oss << std::fixed << std::setprecision(6) << v;
  return oss.str();
}

void Metric(const std::string& k, const std::string& v) { std::cout << "metric." << k << "=" << v << "\n"; }
void Metric(const std::string& k, uint64_t v) { Metric(k, std::to_string(v)); }
void MetricI(const std::string& k, int64_t v) { Metric(k, std::to_string(v)); }

Options ParseArgs(int argc, char** argv) {
  Options o;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    const bool has = i + 1 < argc;
    auto take = [&]() { return std::string(argv[++i]); };
    if (a == "--help" || a == "-h") {
      o.show_help = true;
      return o;
    }
    if (a == "--input" && has) o.input = take();
    else if (a == "--merge-mode" && has) o.merge_mode = take();
    else if (a == "--scoring-backend" && has) o.scoring_backend = take();
    else if (a == "--cost-objective" && has) o.cost_objective = take();
    else if (a == "--state-backend" && has) o.state_backend = take();
    else if (a == "--quotient-update" && has) o.quotient_update = take();
    else if (a == "--candidate-index" && has) o.candidate_index = take();
    else if (a == "--certification" && has) o.certification = take();
    else if (a == "--commit-policy" && has) o.commit_policy = take();
    else if (a == "--threshold-policy" && has) o.threshold_policy = take();
    else if (a == "--profiling" && has) o.profiling = take();
    else if (a == "--top-k" && has) o.top_k = std::stoi(take());
    else if (a == "--group-batch-size" && has) o.group_batch_size = std::stoi(take());
    else if (a == "--iterations" && has) o.iterations = std::stoi(take());
    else if (a == "--print-offset" && has) o.print_offset = std::stoi(take());
    else if (a == "--divide-hash-dims" && has) o.divide_hash_dims = std::stoi(take());
    else if (a == "--divide-max-group" && has) o.divide_max_group = std::stoi(take());
    else if (a == "--error-bound" && has) o.error_bound = std::stod(take());
    else if (a == "--out" && has) o.out_dir = take();
    else if (a == "--seed" && has) o.seed = std::stoull(take());
    else if (a == "--device" && has) o.device = std::stoi(take());
    else if (a == "--ea-use-threshold") o.ea_use_threshold = true;
    else if (a == "--write-output") o.write_output = true;
    else if (a == "--verify-cuda-gain") o.verify_cuda_gain = true;  // re-score and check every commit
    else if (a == "--ranker") o.ranker = true;  // learned candidate ranker (beam-gb300's own)
    else if (a == "--ranker-audit") o.ranker_audit = true;
    else if (a == "--ranker-recall" && has) o.ranker_recall = std::stod(take());
    else if (a == "--ranker-train-iters" && has) o.ranker_train_iters = std::stoi(take());
    else if (a == "--results-csv" && has) o.results_csv = take();
    else if (a == "--profile-csv" && has) o.profile_csv = take();
    else if (a == "--validate-quotient") o.validate_quotient = true;
    else if (a == "--candidate-budget" && has) o.candidate_budget = std::stoi(take());
    else if (a == "--candidate-batch-budget" && has) o.candidate_batch_budget = std::stoi(take());
    else if (a == "--cuda-slice-memory-mb" && has) o.cuda_slice_memory_mb = std::stoi(take());
    else if (a == "--overflow-group-gmax" && has) o.overflow_group_gmax = std::stoi(take());
    else if (a == "--overflow-refine-rounds" && has) o.overflow_refine_rounds = std::stoi(take());
    else if (a == "--commit-audit") o.commit_audit = true;
    else if (a == "--commit-audit-csv" && has) {
      take();
      o.commit_audit = true;
    }
    // parameters of the adaptive / mags-geom threshold policies: unused by the
    // reciprocal policy, accepted as the reference accepts them
    else if ((a == "--threshold-high" || a == "--threshold-low" || a == "--threshold-min-low" ||
              a == "--adaptive-q-high" || a == "--adaptive-q-low" || a == "--acceptance-target") && has) {
      std::stod(take());
    } else if (a == "--adaptive-sample-limit" && has) {
      std::stoi(take());
    }
    else {
      std::cerr << "Unknown or incomplete argument: " << a << "\n";
      o.show_help = true;
      return o;
    }
  }
  return o;
}

// Appends one row to a CSV, writing the header first when the file is new and
// refusing a file whose header differs (the reference's append rule,
// src/main.cpp:275-325).
void AppendCsv(const std::string& path, const std::vector<std::string>& columns,
               const std::vector<std::string>& values) {
  if (columns.size() != values.size()) throw std::runtime_error("CSV row does not match its schema: " + path);
  auto join = [](const std::vector<std::string>& v) {
    std::string line;
    for (size_t i = 0; i < v.size(); ++i) line += (i ? "," : "") + v[i];
    return line;
  };
  const std::string header = join(columns);
  if (std::filesystem::exists(path)) {
    std::ifstream in(path);
    if (!in) throw std::runtime_error("Failed to read existing results CSV: " + path);
    std::string first;
    std::getline(in, first);
    if (!first.empty() && first.back() == '\r') first.pop_back();
    if (first != header) throw std::runtime_error("Existing results CSV header does not match current schema: " + path);
  } else {
    std::ofstream out(path, std::ios::app);
    if (!out) throw std::runtime_error("Failed to open results CSV: " + path);
    out << header << '\n';
  }
  std::ofstream out(path, std::ios::app);
  if (!out) throw std::runtime_error("Failed to open results CSV: " + path);
  out << join(values) << '\n';
}

// The dataset label of a profile row: the input's parent directory, else its
// stem (src/main.cpp:252-256).
std::string DatasetLabel(const std::string& input) {
  const std::filesystem::path path(input);
  const std::string label = path.parent_path().filename().string();
  return label.empty() ? path.stem().string() : label;
}

// One row of --profiling rounds: this iteration's counters (differences of
// the cumulative ones) and times.
struct IterationRow {
  int iteration = 0;
  int64_t active = 0, groups = 0;
  uint64_t proxy_examined = 0, after_topk = 0, exact_calls = 0, positive = 0, above_threshold = 0, selected = 0;
  uint64_t merges = 0, input_nnz = 0, touched = 0, raw_a = 0, raw_b = 0, uni = 0, ovl = 0;
  double divide_ms = 0, merge_ms = 0;
};

IterationRow MakeRow(int iter, int64_t active, int64_t groups, const beam_engine_stats& b, const beam_engine_stats& a,
                     double divide_ms, double merge_ms) {
  IterationRow r;
  r.iteration = iter;
  r.active = active;
  r.groups = groups;
  r.proxy_examined = a.candidate_proxy_pairs_examined - b.candidate_proxy_pairs_examined;
  r.after_topk = a.merge_candidate_pairs_after_prune - b.merge_candidate_pairs_after_prune;
  r.exact_calls = a.merge_exact_gain_calls - b.merge_exact_gain_calls;
  r.positive = a.merge_positive_gain_pairs - b.merge_positive_gain_pairs;
  r.above_threshold = a.merge_candidate_pairs - b.merge_candidate_pairs;
  r.selected = a.merge_selected_pairs - b.merge_selected_pairs;
  r.merges = a.accepted_merges_after_validation - b.accepted_merges_after_validation;
  r.input_nnz = a.exact_gain_input_nnz - b.exact_gain_input_nnz;
  r.touched = a.update_touched_quotient_entries - b.update_touched_quotient_entries;
  r.raw_a = a.exact_raw_entries_a - b.exact_raw_entries_a;
  r.raw_b = a.exact_raw_entries_b - b.exact_raw_entries_b;
  r.uni = a.exact_union_neighbors - b.exact_union_neighbors;
  r.ovl = a.exact_overlap_neighbors - b.exact_overlap_neighbors;
  r.divide_ms = divide_ms;
  r.merge_ms = merge_ms;
  return r;
}

// --profile-csv: the reference's per-iteration schema (src/main.cpp:1061-1178).
// Counters the GB300 path has are filled in; the ones of modes it does not run
// (certification, candidate index, legacy row building) are 0. Per-stage
// times inside Merge are not split per iteration on the device: the whole
// Merge time goes to exact_gain_ms.
void WriteProfileCsv(const Options& o, const std::vector<IterationRow>& rounds) {
  const std::vector<std::string> columns = {
      "dataset", "iteration", "algorithm", "profiling_mode", "active_supernodes", "group_count", "sum_group_sizes",
      "candidate_proxy_pairs_examined", "candidate_pairs_after_topk", "candidate_pairs_submitted_for_scoring",
      "candidate_pairs_scored", "exact_gain_calls", "exact_gain_positive_count", "above_threshold_count",
      "matching_selected_count", "actual_merge_count", "prepare_original_edges_scanned", "prepare_aggregated_nnz",
      "exact_gain_input_nnz", "update_partition_nodes_touched", "update_touched_quotient_entries",
      "prepare_row_entries_copied", "prepare_row_copy_bytes", "prepare_row_views_created",
      "prepare_unique_representatives", "prepare_row_acquisition_requests", "prepare_row_acquisition_hits",
      "prepare_row_acquisition_misses", "prepare_duplicate_acquisitions_avoided", "prepare_row_registry_entries",
      "prepare_row_registry_bytes", "exact_persistent_pairs", "exact_raw_entries_a", "exact_raw_entries_b",
      "exact_union_neighbors", "exact_overlap_neighbors", "exact_single_sided_neighbors",
      "exact_internal_block_terms", "exact_block_cost_evaluations", "exact_capacity_multiplications",
      "certification_candidates_seen", "upper_bound_pruned", "upper_bound_passed", "early_abort_count",
      "exact_full_scan_count", "exact_entries_available", "exact_entries_scanned", "exact_entries_skipped",
      "upper_bound_ms", "early_abort_exact_ms", "candidate_index_build_ms", "candidate_index_refresh_ms",
      "candidate_proposal_ms", "candidate_proposals_raw", "candidate_proposals_unique",
      "candidate_duplicates_removed", "candidate_budget_exhausted_nodes", "candidate_nodes_with_zero_proposals",
      "candidate_direct_neighbor_count", "candidate_shared_neighbor_count", "candidate_exploration_count",
      "quotient_row_lookup_ms", "quotient_row_copy_ms", "quotient_exact_gain_ms", "divide_ms", "prepare_ms",
      "candidate_discovery_task_sum_ms", "exact_gain_ms", "matching_ms", "update_ms"};
  const std::string dataset = DatasetLabel(o.input);
  const std::string z = "0", zf = FormatDouble(0.0);
  for (const IterationRow& r : rounds) {
    auto u = [](uint64_t v) { return std::to_string(v); };
    std::vector<std::string> v = {
        dataset, std::to_string(r.iteration), "beam_cost_oracle_reference", o.profiling, std::to_string(r.active),
        std::to_string(r.groups), std::to_string(r.active), u(r.proxy_examined), u(r.after_topk), u(r.exact_calls),
        u(r.exact_calls), u(r.exact_calls), u(r.positive), u(r.above_threshold), u(r.selected), u(r.merges), z, z,
        u(r.input_nnz), z, u(r.touched), z, z, z, z, z, z, z, z, z, z, u(r.exact_calls), u(r.raw_a), u(r.raw_b),
        u(r.uni), u(r.ovl), u(r.uni - r.ovl), u(4 * r.exact_calls), z, z, z, z, z, z, z, z, z, z, zf, zf, zf, zf,
        zf, z, z, z, z, z, z, z, z, zf, zf, zf, FormatDouble(r.divide_ms), zf, zf, FormatDouble(r.merge_ms), zf,
        zf};
    AppendCsv(o.profile_csv, columns, v);
  }
}

// --results-csv: the reference's result-row schema (src/main.cpp:1197-1487),
// one row per run; counters of modes the GB300 path does not run are 0.
void WriteResultsCsv(const Options& o, int64_t n, int64_t edges, int64_t arcs, uint64_t hash,
                     const beam_encoding& enc, const beam_engine_stats& st, double run_ms, double divide_ms,
                     double merge_ms, double encode_ms) {
  const std::vector<std::string> columns = {
      "n", "input_edges_raw", "graph_arcs", "original_undirected_edges", "original_edges_eval", "iterations", "seed",
      "divide_hash_dims", "divide_max_group", "merge_mode", "scoring_backend", "threshold_policy", "cost_objective",
      "state_backend", "candidate_index", "candidate_budget", "certification", "commit_policy", "validate_quotient",
      "quotient_update", "top_k", "group_batch_size", "candidate_batch_budget", "cuda_slice_memory_mb",
      "overflow_group_gmax", "overflow_refine_rounds", "error_bound", "supernode_count", "P", "Cp", "Cm",
      "encoding_cost", "cost_ratio", "num_superedges_nonloop", "num_superedges_loop", "num_positive_corrections",
      "num_negative_corrections", "encoding_cost_standard", "cost_ratio_standard", "encoding_cost_mags_x2",
      "encoding_cost_mags_compatible", "cost_ratio_mags_compatible", "compression_gain", "compression_java_style",
      "runtime_run_ms", "runtime_divide_ms", "runtime_merge_ms", "divide_max_group_size", "divide_fallback_splits",
      "runtime_encode_ms", "runtime_output_ms", "runtime_algorithm_ms", "runtime_end_to_end_ms",
      "merge_prepare_wall_ms", "merge_prepare_task_sum_ms", "merge_create_w_ms", "merge_scoring_ms",
      "merge_candidate_gen_ms", "merge_gain_scoring_ms", "merge_selection_ms", "merge_update_ms",
      "merge_candidate_pairs", "merge_selected_pairs", "merge_total_local_gain", "merge_avg_local_gain",
      "merge_group_count", "merge_group_max_size", "merge_raw_pair_count", "merge_candidate_pairs_after_prune",
      "merge_exact_gain_calls", "merge_positive_gain_pairs", "merge_rejected_by_overlap",
      "merge_rejected_by_threshold", "merge_exact_gain_calls_per_selected", "merge_positive_gain_ratio",
      "partition_hash", "isolated_gain_sum", "realized_marginal_gain_sum", "actual_batch_cost_reduction",
      "interaction_delta", "selected_merges_for_validation", "accepted_merges_after_validation",
      "rejected_nonpositive", "stale_endpoint", "gain_decreased", "gain_increased", "negative_marginal",
      "candidate_refresh_count", "original_exact_calls", "validation_exact_calls", "validation_exact_row_entry_work",
      "commit_validation_ms", "audit_oracle_ms", "certification_candidates_seen", "upper_bound_pruned",
      "upper_bound_passed", "early_abort_count", "exact_full_scan_count", "exact_entries_available",
      "exact_entries_scanned", "exact_entries_skipped", "upper_bound_ms", "early_abort_exact_ms", "threshold_last",
      "threshold_geom_last", "threshold_adaptive_last", "threshold_acceptance_scale",
      "threshold_acceptance_rate_last", "threshold_sample_count_last", "cuda_init_ms", "cuda_h2d_ms",
      "cuda_row_h2d_ms", "cuda_pair_h2d_ms", "cuda_kernel_ms", "cuda_d2h_ms", "cuda_total_ms", "cuda_packed_h2d_ms",
      "cuda_packed_d2h_ms", "cuda_num_calls", "cuda_row_uploads", "cuda_kernel_launches", "cuda_h2d_bytes",
      "cuda_d2h_bytes", "cuda_max_candidates_per_launch", "cuda_packed_h2d_calls", "cuda_packed_d2h_calls",
      "cuda_packed_input_bytes", "cuda_packed_output_bytes", "cuda_slice_count", "cuda_blocks_single_slice",
      "cuda_blocks_multi_slice", "cuda_max_slice_rows", "cuda_max_slice_nnz", "cuda_max_slice_candidates",
      "cuda_slice_memory_budget_bytes", "overflow_groups_seen", "overflow_refined_subgroups",
      "overflow_forced_chunks", "overflow_max_group_before", "overflow_max_group_after", "overflow_refine_ms",
      "encode_relabel_ms", "encode_count_edges_ms", "encode_decision_ms", "encode_correction_generation_ms",
      "reconstruction_pass"};
  auto u = [](uint64_t v) { return std::to_string(v); };
  auto i = [](int64_t v) { return std::to_string(v); };
  auto f = [](double v) { return FormatDouble(v); };
  const std::string z = "0", zf = FormatDouble(0.0);
  const double gain = 1.0 - enc.cost_ratio_standard;
  const double per_selected = static_cast<double>(st.merge_exact_gain_calls) /
                              static_cast<double>(st.merge_selected_pairs ? st.merge_selected_pairs : 1);
  const double positive_ratio = static_cast<double>(st.merge_positive_gain_pairs) /
                                static_cast<double>(st.merge_exact_gain_calls ? st.merge_exact_gain_calls : 1);
  const double avg_gain = st.merge_selected_pairs ? static_cast<double>(st.merge_total_local_gain) /
                                                        static_cast<double>(st.merge_selected_pairs)
                                                  : 0.0;
  const double threshold_last = o.ea_use_threshold ? 1.0 / static_cast<double>(o.iterations + 1) : 0.0;
  std::vector<std::string> v = {
      i(n), i(edges), i(arcs), i(edges), i(edges), i(o.iterations), u(o.seed), i(o.divide_hash_dims),
      i(o.divide_max_group), o.merge_mode, o.scoring_backend, o.threshold_policy, o.cost_objective, o.state_backend,
      o.candidate_index, i(o.candidate_budget), o.certification, o.commit_policy,
      o.validate_quotient ? "true" : "false", o.quotient_update, i(o.top_k), i(o.group_batch_size),
      i(o.candidate_batch_budget), i(o.cuda_slice_memory_mb), i(o.overflow_group_gmax), i(o.overflow_refine_rounds),
      f(o.error_bound), i(enc.supernodes), i(enc.p), i(enc.cp), i(enc.cm), i(enc.encoding_cost_standard),
      f(enc.cost_ratio_standard), i(enc.superedges_nonloop), i(enc.superedges_loop), i(enc.cp), i(enc.cm),
      i(enc.encoding_cost_standard), f(enc.cost_ratio_standard), i(enc.encoding_cost_mags_x2),
      f(static_cast<double>(enc.encoding_cost_mags_x2) / 2.0), f(enc.cost_ratio_mags_compatible), f(gain), f(gain),
      f(run_ms), f(divide_ms), f(merge_ms), u(st.divide_max_group_size), u(st.divide_fallback_splits), f(encode_ms),
      zf, f(run_ms + encode_ms), f(run_ms + encode_ms), zf, zf, zf, zf, zf, zf, zf, zf,
      u(st.merge_candidate_pairs), u(st.merge_selected_pairs), u(st.merge_total_local_gain), f(avg_gain),
      u(st.merge_group_count), u(st.merge_group_max_size), u(st.merge_raw_pair_count),
      u(st.merge_candidate_pairs_after_prune), u(st.merge_exact_gain_calls), u(st.merge_positive_gain_pairs),
      u(st.merge_rejected_by_overlap), u(st.merge_rejected_by_threshold), f(per_selected), f(positive_ratio),
      u(hash), u(st.isolated_gain_sum), z, z, z, u(st.selected_merges_for_validation),
      u(st.accepted_merges_after_validation), u(st.rejected_nonpositive), z, z, z, z, z, z,
      u(st.validation_exact_calls), u(st.validation_exact_row_entry_work), zf, zf, z, z, z, z, z, z, z, z, zf, zf,
      f(threshold_last), zf, zf, f(1.0), zf, z, zf, zf, zf, zf, zf, zf, zf, zf, zf, z, z, z, z, z, z, z, z, z, z,
      z, z, z, z, z, z, z, z, z, z, z, z, zf, zf, zf, zf, zf, "unknown"};
  AppendCsv(o.results_csv, columns, v);
}

void Require(const std::string& flag, const std::string& got, const std::string& want) {
  if (got != want) {
    throw std::runtime_error(flag + " " + got + " is not provided by the GB300 build; it implements " + flag + " " +
                             want);
  }
}

int Run(int argc, char** argv) {
  Options o = ParseArgs(argc, argv);
  if (o.show_help || o.input.empty()) {
    PrintUsage();
    return o.input.empty() ? 1 : 0;
  }
  if (o.write_output && o.out_dir.empty()) throw std::runtime_error("--write-output requires --out <dir>.");
  Require("--scoring-backend", o.scoring_backend, "cuda");
  // batch-ea (one group at a time, src/sweg.cpp:1147-1161) equals
  // batch-ea-blocked with one group per block; --group-batch-size is then unused
  if (o.merge_mode == "batch-ea") {
    o.group_batch_size = 1;
  } else {
    Require("--merge-mode", o.merge_mode, "batch-ea-blocked");
  }
  Require("--cost-objective", o.cost_objective, "mags-compatible");
  Require("--state-backend", o.state_backend, "persistent");
  Require("--quotient-update", o.quotient_update, "incremental");
  Require("--candidate-index", o.candidate_index, "legacy");
  Require("--certification", o.certification, "off");
  Require("--commit-policy", o.commit_policy, "g0");
  Require("--threshold-policy", o.threshold_policy, "reciprocal");
  if (o.error_bound != 0.0) throw std::runtime_error("--error-bound other than 0 is not provided by the GB300 build");
  if (o.overflow_group_gmax != 0) {
    throw std::runtime_error("--overflow-group-gmax other than 0 is not provided by the GB300 build");
  }
  if (o.commit_audit) throw std::runtime_error("--commit-audit is not provided by the GB300 build (commit policy g0)");
  if (o.profiling != "off" && o.profiling != "summary" && o.profiling != "rounds") {
    throw std::runtime_error("Unknown --profiling value: " + o.profiling);
  }
  if (!o.profile_csv.empty() && o.profiling != "rounds") {
    throw std::runtime_error("--profile-csv requires --profiling rounds so every row has an iteration.");
  }
  if (o.divide_hash_dims <= 0) {
    std::cerr << "Warning: invalid --divide-hash-dims=" << o.divide_hash_dims << ", fallback to 16\n";
    o.divide_hash_dims = 16;
  }
  if (o.divide_max_group <= 0) {
    std::cerr << "Warning: invalid --divide-max-group=" << o.divide_max_group << ", fallback to 512\n";
    o.divide_max_group = 512;
  }

  const bool binary = o.input.size() > 4 && o.input.compare(o.input.size() - 4, 4, ".bin") == 0;
  beam_graph* g = binary ? beam_graph_load_binary(o.input.c_str()) : beam_graph_load_text(o.input.c_str());
  if (!g) throw std::runtime_error(beam_graph_last_error());
  const int64_t n = beam_graph_num_nodes(g);
  const int64_t edges = beam_graph_num_edges(g);
  const int64_t arcs = beam_graph_num_arcs(g);
  if (arcs != 2 * edges) {
    throw std::runtime_error("Input graph invariant violated: graph_arcs must equal 2 * input_edges_raw.");
  }
  std::cout << "Loaded graph: n=" << n << " m=" << arcs << "\n";
  std::cout << "Seed: " << o.seed << "\n";
  std::cout << "Divide hash dims: " << o.divide_hash_dims << "\n";
  std::cout << "Divide max group: " << o.divide_max_group << "\n";
  std::cout << "Merge mode: " << o.merge_mode << "\n";
  std::cout << "Scoring backend: " << o.scoring_backend << "\n";
  std::cout << "Threshold policy: " << o.threshold_policy << "\n";
  std::cout << "Cost objective: " << o.cost_objective << "\n";
  std::cout << "State backend: " << o.state_backend << "\n";
  std::cout << "Quotient update: " << o.quotient_update << "\n";
  std::cout << "CUDA scoring build: " << CudaScoringBuildMode() << "\n";
  if (o.write_output) std::cout << "Output directory: " << o.out_dir << "\n";
  else std::cout << "Output writing: disabled\n";

  beam_engine_config cfg;
  beam_engine_default_config(&cfg);
  cfg.top_k = o.top_k;
  cfg.group_batch_size = o.group_batch_size;
  cfg.divide_hash_dims = o.divide_hash_dims;
  cfg.divide_max_group = o.divide_max_group;
  cfg.ea_use_threshold = o.ea_use_threshold ? 1 : 0;
  cfg.seed = o.seed;
  cfg.device = o.device;
  cfg.verify_cuda_gain = o.verify_cuda_gain ? 1 : 0;
  cfg.ranker = o.ranker ? 1 : 0;
  cfg.ranker_audit = o.ranker_audit ? 1 : 0;
  cfg.ranker_recall = static_cast<float>(o.ranker_recall);
  cfg.ranker_train_iters = o.ranker_train_iters;
  beam_engine* e = nullptr;
  if (beam_engine_create(static_cast<int32_t>(n), arcs, beam_graph_row_ptr(g), beam_graph_col_idx(g), &cfg, &e) != 0) {
    throw std::runtime_error(beam_engine_last_error());
  }
  auto check = [&](int rc) {
    if (rc != 0) throw std::runtime_error(beam_engine_last_error());
  };
  using Clock = std::chrono::steady_clock;
  std::vector<IterationRow> rounds;
  const auto t0 = Clock::now();
  double divide_ms = 0, merge_ms = 0, validate_ms = 0;
  for (int iter = 1; iter <= o.iterations; ++iter) {
    const auto d0 = Clock::now();
    check(beam_engine_divide(e, iter));
    const auto d1 = Clock::now();
    int64_t active = 0, groups = 0;
    check(beam_engine_group_counts(e, &active, &groups));
    beam_engine_stats before;
    check(beam_engine_get_stats(e, &before));
    check(beam_engine_merge(e, iter, o.iterations));
    const auto d2 = Clock::now();
    divide_ms += std::chrono::duration<double, std::milli>(d1 - d0).count();
    merge_ms += std::chrono::duration<double, std::milli>(d2 - d1).count();
    if (o.profiling == "rounds") {
      beam_engine_stats after;
      check(beam_engine_get_stats(e, &after));
      rounds.push_back(MakeRow(iter, active, groups, before, after,
                               std::chrono::duration<double, std::milli>(d1 - d0).count(),
                               std::chrono::duration<double, std::milli>(d2 - d1).count()));
    }
    if (o.validate_quotient) {
      // QuotientGraph::ValidateAgainstOriginalGraph after the iteration's
      // commits (the reference checks after each merge; the GB300 path commits
      // a block's merges as one batch, so the state between them never exists)
      const auto v0 = Clock::now();
      check(beam_engine_validate_quotient(e));
      validate_ms += std::chrono::duration<double, std::milli>(Clock::now() - v0).count();
    }
    if (o.print_offset > 0 && (iter % o.print_offset == 0 || iter == o.iterations)) {
      beam_engine_stats after;
      check(beam_engine_get_stats(e, &after));
      const uint64_t merged = after.accepted_merges_after_validation - before.accepted_merges_after_validation;
      std::cout << "Iter " << iter << ": groups=" << groups << " active_supernodes=" << (active - static_cast<int64_t>(merged))
                << "\n";
    }
  }
  const double run_ms = std::chrono::duration<double, std::milli>(Clock::now() - t0).count() - validate_ms;

  std::vector<int32_t> labels(static_cast<size_t>(n)), head(static_cast<size_t>(n)), next(static_cast<size_t>(n));
  check(beam_engine_partition(e, labels.data(), head.data(), next.data()));
  beam_engine_stats st;
  check(beam_engine_get_stats(e, &st));
  beam_ranker_info rk;
  check(beam_engine_ranker_info(e, &rk));
  int64_t qnnz = 0;
  check(beam_engine_quotient_nnz(e, &qnnz));
  // CostOracle::ExactPartitionCost on the device (src/main.cpp:560)
  int64_t exact = 0;
  check(beam_engine_exact_partition_cost(e, &exact));
  // Sweg::Encode on the device, files written by the host
  const auto enc0 = Clock::now();
  beam_encoding enc;
  if (o.write_output) std::filesystem::create_directories(o.out_dir);
  check(beam_engine_encode(e, o.write_output ? o.out_dir.c_str() : nullptr, &enc));
  const double encode_ms = std::chrono::duration<double, std::milli>(Clock::now() - enc0).count();
  beam_engine_destroy(e);
  if (enc.encoding_cost_standard != exact) {
    throw std::runtime_error("MAGS-compatible payload cost differs from exact partition cost");
  }

  Metric("n", static_cast<uint64_t>(n));
  Metric("input_edges_raw", static_cast<uint64_t>(edges));
  Metric("graph_arcs", static_cast<uint64_t>(arcs));
  Metric("original_undirected_edges", static_cast<uint64_t>(edges));
  Metric("original_edges_eval", static_cast<uint64_t>(edges));
  MetricI("iterations", o.iterations);
  Metric("seed", o.seed);
  MetricI("divide_hash_dims", o.divide_hash_dims);
  MetricI("divide_max_group", o.divide_max_group);
  Metric("merge_mode", o.merge_mode);
  Metric("scoring_backend", o.scoring_backend);
  Metric("threshold_policy", o.threshold_policy);
  Metric("profiling_mode", o.profiling);
  Metric("cost_objective", o.cost_objective);
  Metric("state_backend", o.state_backend);
  Metric("certification", o.certification);
  Metric("commit_policy", o.commit_policy);
  Metric("partition_hash", beam_partition_hash(static_cast<int32_t>(n), labels.data()));
  Metric("validate_quotient", o.validate_quotient ? "true" : "false");
  Metric("quotient_update", o.quotient_update);
  MetricI("exact_partition_cost", exact);
  MetricI("top_k", o.top_k);
  MetricI("group_batch_size", o.group_batch_size);
  Metric("error_bound", FormatDouble(o.error_bound));
  MetricI("supernode_count", enc.supernodes);
  MetricI("P", enc.p);
  MetricI("Cp", enc.cp);
  MetricI("Cm", enc.cm);
  MetricI("encoding_cost", enc.encoding_cost_standard);
  Metric("cost_ratio", FormatDouble(enc.cost_ratio_standard));
  MetricI("num_superedges_nonloop", enc.superedges_nonloop);
  MetricI("num_superedges_loop", enc.superedges_loop);
  MetricI("num_positive_corrections", enc.cp);
  MetricI("num_negative_corrections", enc.cm);
  MetricI("encoding_cost_standard", enc.encoding_cost_standard);
  Metric("cost_ratio_standard", FormatDouble(enc.cost_ratio_standard));
  MetricI("encoding_cost_mags_x2", enc.encoding_cost_mags_x2);
  Metric("encoding_cost_mags_compatible", FormatDouble(static_cast<double>(enc.encoding_cost_mags_x2) / 2.0));
  Metric("cost_ratio_mags_compatible", FormatDouble(enc.cost_ratio_mags_compatible));
  Metric("compression_gain", FormatDouble(1.0 - enc.cost_ratio_standard));
  Metric("runtime_run_ms", FormatDouble(run_ms));
  Metric("runtime_divide_ms", FormatDouble(divide_ms));
  Metric("runtime_merge_ms", FormatDouble(merge_ms));
  Metric("divide_max_group_size", st.divide_max_group_size);
  Metric("divide_fallback_splits", st.divide_fallback_splits);
  Metric("runtime_encode_ms", FormatDouble(encode_ms));
  Metric("runtime_algorithm_ms", FormatDouble(run_ms + encode_ms));
  Metric("merge_candidate_pairs", st.merge_candidate_pairs);
  Metric("merge_selected_pairs", st.merge_selected_pairs);
  Metric("merge_total_local_gain", st.merge_total_local_gain);
  Metric("merge_avg_local_gain",
         FormatDouble(st.merge_selected_pairs ? static_cast<double>(st.merge_total_local_gain) /
                                                    static_cast<double>(st.merge_selected_pairs)
                                              : 0.0));
  Metric("merge_group_count", st.merge_group_count);
  Metric("merge_group_max_size", st.merge_group_max_size);
  Metric("merge_raw_pair_count", st.merge_raw_pair_count);
  Metric("merge_candidate_pairs_after_prune", st.merge_candidate_pairs_after_prune);
  Metric("merge_exact_gain_calls", st.merge_exact_gain_calls);
  Metric("merge_positive_gain_pairs", st.merge_positive_gain_pairs);
  Metric("merge_rejected_by_overlap", st.merge_rejected_by_overlap);
  Metric("merge_rejected_by_threshold", st.merge_rejected_by_threshold);
  Metric("isolated_gain_sum", st.isolated_gain_sum);
  Metric("selected_merges_for_validation", st.selected_merges_for_validation);
  Metric("accepted_merges_after_validation", st.accepted_merges_after_validation);
  Metric("rejected_nonpositive", st.rejected_nonpositive);
  Metric("stale_endpoint", static_cast<uint64_t>(0));
  Metric("validation_exact_calls", st.validation_exact_calls);
  Metric("validation_exact_row_entry_work", st.validation_exact_row_entry_work);
  Metric("update_touched_quotient_entries", st.update_touched_quotient_entries);
  Metric("quotient_nnz_final", static_cast<uint64_t>(qnnz));
  Metric("exact_raw_entries_a", st.exact_raw_entries_a);
  Metric("exact_raw_entries_b", st.exact_raw_entries_b);
  Metric("exact_union_neighbors", st.exact_union_neighbors);
  Metric("exact_overlap_neighbors", st.exact_overlap_neighbors);
  Metric("candidate_proxy_pairs_examined", st.candidate_proxy_pairs_examined);
  Metric("exact_gain_input_nnz", st.exact_gain_input_nnz);
  Metric("merges_per_second", FormatDouble(run_ms > 0 ? 1000.0 * static_cast<double>(st.accepted_merges_after_validation) / run_ms : 0.0));
  if (o.ranker) {
    Metric("ranker_samples", rk.samples);
    Metric("ranker_train_steps", rk.train_steps);
    Metric("ranker_train_ms", FormatDouble(rk.train_ms));
    Metric("ranker_ranked", rk.ranked);
    Metric("ranker_pruned", rk.pruned);
    if (o.ranker_audit) {
      Metric("ranker_audit_passing", rk.audit_passing);
      Metric("ranker_audit_lost", rk.audit_lost);
    }
  }
  if (!o.profile_csv.empty()) WriteProfileCsv(o, rounds);
  if (!o.results_csv.empty()) {
    WriteResultsCsv(o, n, edges, arcs, beam_partition_hash(static_cast<int32_t>(n), labels.data()), enc, st, run_ms,
                    divide_ms, merge_ms, encode_ms);
  }
  beam_graph_free(g);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  try {
    return Run(argc, argv);
  } catch (const std::exception& e) {
    std::cout << "Error: " << e.what() << "\n";
    return 1;
  }
}
