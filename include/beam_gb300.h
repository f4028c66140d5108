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

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif  /* BEAM_GB300_H_ */
