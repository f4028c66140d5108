// ORACLE — test infrastructure only, never shipped. Exposes the reference's
// own host-side check of its CUDA scoring backend (ComputeLocalGainHostFromFlat
// in src/cuda_scoring.cu, a function of that file's anonymous namespace) by
// compiling the reference's translation unit into this one from where its
// sources lie (the include path names the reference's src/ directory; the
// recipe is oracle/Makefile's `ref-legacy` target). Used only to make the
// golden vectors of tests/golden/legacy_gain.json.

#include "cuda_scoring.cu"

extern "C" int ref_legacy_flat_gains(const int32_t* offsets, const int32_t* reps, const int64_t* row_sizes,
                                     const int64_t* self_loops, int32_t rows, const int32_t* nb,
                                     const int64_t* wt, const int64_t* nsz, int64_t entries,
                                     const int32_t* pairs, int64_t count, int64_t* gain, int64_t* before) {
  Sweg::FlatAggCSR f;
  f.offsets.assign(offsets, offsets + rows + 1);
  f.row_rep_ids.assign(reps, reps + rows);
  f.row_sizes.assign(row_sizes, row_sizes + rows);
  f.row_self_loops.assign(self_loops, self_loops + rows);
  f.neighbors.assign(nb, nb + entries);
  f.weights.assign(wt, wt + entries);
  f.neighbor_sizes.assign(nsz, nsz + entries);
  for (int64_t p = 0; p < count; ++p) {
    const Sweg::LocalGainResult r = ComputeLocalGainHostFromFlat(f, pairs[2 * p], pairs[2 * p + 1]);
    gain[p] = r.gain;
    before[p] = r.before_cost;
  }
  return 0;
}
