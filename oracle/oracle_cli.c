/*
 * ORACLE — test infrastructure only. Command-line front end of the C
 * restatement: accepts the reference's flags for the recommended mode
 * (src/main.cpp:327-423), loads a text edge list with the reference loader's
 * rules (src/graph_io/graph_io.cpp:12-106), runs, and prints metric.k=v lines
 * with the reference's names and formatting (src/main.cpp:258-273, 577-740).
 */
#define _POSIX_C_SOURCE 200809L
#include <errno.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

#include "beam_oracle.h"

static int fail(const char* msg) {
  printf("Error: %s\n", msg);
  return 1;
}

typedef struct {
  int64_t n, edges;
  int64_t* row_ptr;
  int32_t* col;
} csr;

static int cmp_i32(const void* x, const void* y) {
  const int32_t a = *(const int32_t*)x, b = *(const int32_t*)y;
  return a < b ? -1 : (a > b ? 1 : 0);
}

static int load_text(const char* path, csr* g, char* err, size_t errlen) {
  FILE* f = fopen(path, "r");
  if (!f) {
    snprintf(err, errlen, "Failed to open file: %s", path);
    return -1;
  }
  int64_t cap = 1 << 20, ne = 0, max_node = -1, line_no = 0;
  int32_t* eu = (int32_t*)malloc(sizeof(int32_t) * (size_t)cap);
  int32_t* ev = (int32_t*)malloc(sizeof(int32_t) * (size_t)cap);
  char* line = NULL;
  size_t lcap = 0;
  while (getline(&line, &lcap, f) >= 0) {
    ++line_no;
    char* p = line;
    while (*p == ' ' || *p == '\t' || *p == '\r') ++p;
    if (*p == '\n' || *p == '\0' || *p == '#') continue;
    char* end = NULL;
    errno = 0;
    const long long a = strtoll(p, &end, 10);
    if (end == p || errno) {
      snprintf(err, errlen, "Malformed edge list line %lld: expected at least two integers 'u v'.", (long long)line_no);
      goto bad;
    }
    p = end;
    const long long b = strtoll(p, &end, 10);
    if (end == p || errno) {
      snprintf(err, errlen, "Malformed edge list line %lld: expected at least two integers 'u v'.", (long long)line_no);
      goto bad;
    }
    if (a < 0 || b < 0) {
      snprintf(err, errlen, "Negative node id at line %lld.", (long long)line_no);
      goto bad;
    }
    if (a > 2147483647LL || b > 2147483647LL) {
      snprintf(err, errlen, "Node id exceeds int range at line %lld.", (long long)line_no);
      goto bad;
    }
    if (a == b) {
      snprintf(err, errlen, "Self-loop is not supported at line %lld.", (long long)line_no);
      goto bad;
    }
    if (ne == cap) {
      cap *= 2;
      eu = (int32_t*)realloc(eu, sizeof(int32_t) * (size_t)cap);
      ev = (int32_t*)realloc(ev, sizeof(int32_t) * (size_t)cap);
    }
    eu[ne] = (int32_t)a;
    ev[ne] = (int32_t)b;
    ++ne;
    if (a > max_node) max_node = a;
    if (b > max_node) max_node = b;
  }
  free(line);
  fclose(f);
  if (max_node + 1 <= 0) {
    snprintf(err, errlen, "Invalid node count.");
    free(eu);
    free(ev);
    return -1;
  }
  g->n = max_node + 1;
  g->edges = ne;
  g->row_ptr = (int64_t*)calloc((size_t)g->n + 1, sizeof(int64_t));
  g->col = (int32_t*)malloc(sizeof(int32_t) * (size_t)(2 * ne + 1));
  for (int64_t i = 0; i < ne; ++i) {
    g->row_ptr[eu[i] + 1]++;
    g->row_ptr[ev[i] + 1]++;
  }
  for (int64_t i = 0; i < g->n; ++i) g->row_ptr[i + 1] += g->row_ptr[i];
  int64_t* cur = (int64_t*)malloc(sizeof(int64_t) * (size_t)g->n);
  memcpy(cur, g->row_ptr, sizeof(int64_t) * (size_t)g->n);
  for (int64_t i = 0; i < ne; ++i) {
    g->col[cur[eu[i]]++] = ev[i];
    g->col[cur[ev[i]]++] = eu[i];
  }
  for (int64_t v = 0; v < g->n; ++v) {
    qsort(g->col + g->row_ptr[v], (size_t)(g->row_ptr[v + 1] - g->row_ptr[v]), sizeof(int32_t), cmp_i32);
  }
  free(cur);
  free(eu);
  free(ev);
  return 0;
bad:
  free(line);
  fclose(f);
  free(eu);
  free(ev);
  return -1;
}

static void metric_i(const char* k, long long v) { printf("metric.%s=%lld\n", k, v); }
static void metric_u(const char* k, unsigned long long v) { printf("metric.%s=%llu\n", k, v); }
static void metric_d(const char* k, double v) { printf("metric.%s=%.6f\n", k, v); }

static int expect(const char* flag, const char* got, const char* want) {
  if (strcmp(got, want) != 0) {
    printf("Error: the oracle restates only %s %s (got %s)\n", flag, want, got);
    return 0;
  }
  return 1;
}

int main(int argc, char** argv) {
  beam_oracle_config cfg;
  beam_oracle_default_config(&cfg);
  cfg.ea_use_threshold = 0;
  const char* input = NULL;
  const char* out_dir = NULL;
  int iterations = 20, write_output = 0;
  double error_bound = 0.0;
  for (int i = 1; i < argc; ++i) {
    const char* a = argv[i];
    const char* v = i + 1 < argc ? argv[i + 1] : NULL;
#define TAKE(flag) (strcmp(a, flag) == 0 && v && (++i, 1))
    if (TAKE("--input")) input = v;
    else if (TAKE("--merge-mode")) { if (!expect(a, v, "batch-ea-blocked")) return 1; }
    else if (TAKE("--scoring-backend")) {}
    else if (TAKE("--cost-objective")) { if (!expect(a, v, "mags-compatible")) return 1; }
    else if (TAKE("--state-backend")) { if (!expect(a, v, "persistent")) return 1; }
    else if (TAKE("--quotient-update")) { if (!expect(a, v, "incremental")) return 1; }
    else if (TAKE("--candidate-index")) { if (!expect(a, v, "legacy")) return 1; }
    else if (TAKE("--certification")) { if (!expect(a, v, "off")) return 1; }
    else if (TAKE("--commit-policy")) { if (!expect(a, v, "g0")) return 1; }
    else if (TAKE("--threshold-policy")) { if (!expect(a, v, "reciprocal")) return 1; }
    else if (TAKE("--top-k")) cfg.top_k = atoi(v);
    else if (TAKE("--group-batch-size")) cfg.group_batch_size = atoi(v);
    else if (TAKE("--divide-hash-dims")) cfg.divide_hash_dims = atoi(v);
    else if (TAKE("--divide-max-group")) cfg.divide_max_group = atoi(v);
    else if (TAKE("--iterations")) iterations = atoi(v);
    else if (TAKE("--print-offset")) {}
    else if (TAKE("--profiling")) {}
    else if (TAKE("--seed")) cfg.seed = strtoull(v, NULL, 10);
    else if (TAKE("--error-bound")) error_bound = atof(v);
    else if (TAKE("--out")) out_dir = v;
    else if (TAKE("--threads")) cfg.threads = atoi(v);
    else if (strcmp(a, "--ea-use-threshold") == 0) cfg.ea_use_threshold = 1;
    else if (strcmp(a, "--write-output") == 0) write_output = 1;
    else {
      fprintf(stderr, "Unknown or incomplete argument: %s\n", a);
      return 1;
    }
#undef TAKE
  }
  if (!input) return fail("--input is required");
  if (write_output && !out_dir) return fail("--write-output requires --out <dir>.");
  if (error_bound != 0.0) return fail("the oracle restates only --error-bound 0");
  csr g;
  char err[512];
  if (load_text(input, &g, err, sizeof(err)) != 0) return fail(err);
  beam_oracle* o = beam_oracle_create((int32_t)g.n, g.row_ptr[g.n], g.row_ptr, g.col, &cfg);
  if (!o) return fail(beam_oracle_last_error());
  if (beam_oracle_run(o, iterations) != 0) return fail(beam_oracle_last_error());
  if (write_output) mkdir(out_dir, 0755);
  beam_oracle_encoding enc;
  if (beam_oracle_encode(o, write_output ? out_dir : NULL, &enc) != 0) return fail(beam_oracle_last_error());
  const int64_t exact = beam_oracle_exact_partition_cost(o);
  if (exact != enc.encoding_cost_mags_x2 / 2) return fail("MAGS-compatible payload cost differs from exact partition cost");
  beam_oracle_stats st;
  beam_oracle_get_stats(o, &st);
  metric_i("n", g.n);
  metric_i("input_edges_raw", g.edges);
  metric_i("graph_arcs", 2 * g.edges);
  metric_i("iterations", iterations);
  metric_u("partition_hash", (unsigned long long)beam_oracle_partition_hash(o));
  metric_i("exact_partition_cost", exact);
  metric_i("supernode_count", enc.n_supernodes);
  metric_i("P", enc.p);
  metric_i("Cp", enc.cp);
  metric_i("Cm", enc.cm);
  metric_i("num_superedges_nonloop", enc.num_superedges_nonloop);
  metric_i("num_superedges_loop", enc.num_superedges_loop);
  metric_i("encoding_cost_mags_x2", enc.encoding_cost_mags_x2);
  metric_d("cost_ratio_mags_compatible", enc.cost_ratio_mags_compatible);
  metric_d("runtime_run_ms", st.runtime_run_ms);
  metric_d("runtime_divide_ms", st.runtime_divide_ms);
  metric_d("runtime_merge_ms", st.runtime_merge_ms);
  metric_i("divide_max_group_size", st.divide_max_group_size);
  metric_i("divide_fallback_splits", st.divide_fallback_splits);
  metric_d("merge_prepare_wall_ms", st.merge_prepare_wall_ms);
  metric_d("merge_gain_scoring_ms", st.merge_gain_scoring_ms);
  metric_d("merge_selection_ms", st.merge_selection_ms);
  metric_d("merge_update_ms", st.merge_update_ms);
  metric_i("merge_candidate_pairs", st.merge_candidate_pairs);
  metric_i("merge_selected_pairs", st.merge_selected_pairs);
  metric_i("merge_total_local_gain", st.merge_total_local_gain);
  metric_u("merge_group_count", st.merge_group_count);
  metric_u("merge_group_max_size", st.merge_group_max_size);
  metric_u("merge_raw_pair_count", st.merge_raw_pair_count);
  metric_u("merge_candidate_pairs_after_prune", st.merge_candidate_pairs_after_prune);
  metric_u("merge_exact_gain_calls", st.merge_exact_gain_calls);
  metric_u("merge_positive_gain_pairs", st.merge_positive_gain_pairs);
  metric_u("merge_rejected_by_overlap", st.merge_rejected_by_overlap);
  metric_u("merge_rejected_by_threshold", st.merge_rejected_by_threshold);
  metric_i("isolated_gain_sum", st.isolated_gain_sum);
  metric_u("selected_merges_for_validation", st.selected_merges_for_validation);
  metric_u("accepted_merges_after_validation", st.accepted_merges_after_validation);
  metric_u("rejected_nonpositive", st.rejected_nonpositive);
  metric_u("stale_endpoint", st.stale_endpoint);
  metric_u("validation_exact_calls", st.validation_exact_calls);
  metric_u("validation_exact_row_entry_work", st.validation_exact_row_entry_work);
  metric_u("update_touched_quotient_entries", st.update_touched_quotient_entries);
  metric_u("quotient_nnz_final", st.quotient_nnz_final);
  metric_u("exact_raw_entries_a", st.exact_raw_entries_a);
  metric_u("exact_raw_entries_b", st.exact_raw_entries_b);
  metric_u("exact_union_neighbors", st.exact_union_neighbors);
  metric_u("exact_overlap_neighbors", st.exact_overlap_neighbors);
  metric_u("candidate_proxy_pairs_examined", st.candidate_proxy_pairs_examined);
  metric_u("exact_gain_input_nnz", st.exact_gain_input_nnz);
  beam_oracle_free(o);
  free(g.row_ptr);
  free(g.col);
  return 0;
}
