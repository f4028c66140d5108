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
            << "--divide-max-group --seed --error-bound 0 --write-output --out <dir> --profiling --device\n"
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
    else {
      std::cerr << "Unknown or incomplete argument: " << a << "\n";
      o.show_help = true;
      return o;
    }
  }
  return o;
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
  const auto t0 = Clock::now();
  double divide_ms = 0, merge_ms = 0;
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
    if (o.print_offset > 0 && (iter % o.print_offset == 0 || iter == o.iterations)) {
      beam_engine_stats after;
      check(beam_engine_get_stats(e, &after));
      const uint64_t merged = after.accepted_merges_after_validation - before.accepted_merges_after_validation;
      std::cout << "Iter " << iter << ": groups=" << groups << " active_supernodes=" << (active - static_cast<int64_t>(merged))
                << "\n";
    }
  }
  const double run_ms = std::chrono::duration<double, std::milli>(Clock::now() - t0).count();

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
  Metric("validate_quotient", "false");
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
