// Legacy-objective pair scoring over a flat per-block CSR: the service behind
// the reference's Sweg::ScoreCandidatesCuda (include/sweg.hpp:656-658,
// src/cuda_scoring.cu:714-885), which --scoring-backend cuda uses with
// --cost-objective legacy (the README's CUDA mode).
//
// Input is the reference's Sweg::FlatAggCSR (include/sweg.hpp:395-403): row i
// has representative row_rep_ids[i], size row_sizes[i], self-loop count
// row_self_loops[i] and the sorted, duplicate-free entries neighbors /
// weights / neighbor_sizes [offsets[i], offsets[i+1]). A candidate pair
// (a_idx, b_idx) names two rows. Output per pair is {gain, before_cost} with
// the legacy encoding cost min(e, 1 + cap - e) (cap = s(s-1)/2 against the
// row's own representative, s * s_x otherwise), summed over the union of the
// two rows plus the two representatives themselves when a row lacks them;
// counts toward a row's own representative drop its self-loops first
// (src/cuda_scoring.cu:146-252, 282-357).
//
// GB300 form: one warp per pair. Lanes take 32 entries of row a at a time and
// find each neighbour in row b by binary search; then 32 entries of row b at a
// time, skipping those present in row a. Terms are summed per lane and
// reduced once per pair. A call packs the host inputs into one pinned buffer,
// copies it with one H2D, runs one kernel and copies 16 bytes per pair back.

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "beam_gb300.h"
#include "engine.h"

namespace beam {
namespace {

constexpr int kLegacyThreads = 256;

struct FlatView {
  const int* off;
  const int* rep;
  const int* nb;
  const long long* wt;
  const long long* nsz;
  const long long* rsz;
  const long long* self;
};

// Count of neighbour `key` in the sorted flat row [s, e) (0 when absent), and
// whether it is present.
__device__ __forceinline__ long long FlatLookup(const int* nb, const long long* wt, int s, int e, int key,
                                                bool* found) {
  int lo = s, hi = e;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (nb[mid] < key) lo = mid + 1; else hi = mid;
  }
  *found = lo < e && nb[lo] == key;
  return *found ? wt[lo] : 0;
}

struct LegacyPair {
  int ra, rb;
  long long sa, sb, sm, la, lb;
};

// The before and after terms of one neighbour x of the pair.
__device__ __forceinline__ void LegacyTerm(const LegacyPair& p, int x, long long sx, long long ea_raw,
                                           long long eb_raw, long long* before, long long* after) {
  long long ea = ea_raw;
  if (x == p.ra) ea = ea_raw - p.la > 0 ? ea_raw - p.la : 0;
  long long eb = eb_raw;
  if (x == p.rb) eb = eb_raw - p.lb > 0 ? eb_raw - p.lb : 0;
  *before += EncodeCostForPair(p.ra, p.sa, x, sx, ea) + EncodeCostForPair(p.rb, p.sb, x, sx, eb);
  const int mrep = x == p.rb ? p.ra : x;
  const long long msz = x == p.rb ? p.sm : sx;
  *after += EncodeCostForPair(p.ra, p.sm, mrep, msz, ea + eb);
}

__global__ void __launch_bounds__(kLegacyThreads) LegacyFlatScoreKernel(FlatView F, const int2* pairs,
                                                                         long long count, long long* out) {
  constexpr unsigned kFull = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const long long warps = static_cast<long long>(gridDim.x) * (kLegacyThreads / 32);
  for (long long w = (static_cast<long long>(blockIdx.x) * kLegacyThreads + threadIdx.x) >> 5; w < count;
       w += warps) {
    const int2 pr = pairs[w];
    LegacyPair p;
    p.ra = F.rep[pr.x];
    p.rb = F.rep[pr.y];
    p.sa = F.rsz[pr.x];
    p.sb = F.rsz[pr.y];
    p.sm = p.sa + p.sb;
    p.la = F.self[pr.x];
    p.lb = F.self[pr.y];
    const int a0 = F.off[pr.x], a1 = F.off[pr.x + 1];
    const int b0 = F.off[pr.y], b1 = F.off[pr.y + 1];
    long long before = 0, after = 0;
    bool seen_a = false, seen_b = false;
    for (int k = a0 + lane; k < a1; k += 32) {
      const int x = F.nb[k];
      bool in_b = false;
      const long long eb = FlatLookup(F.nb, F.wt, b0, b1, x, &in_b);
      LegacyTerm(p, x, F.nsz[k], F.wt[k], eb, &before, &after);
      seen_a |= x == p.ra;
      seen_b |= x == p.rb;
    }
    for (int k = b0 + lane; k < b1; k += 32) {
      const int x = F.nb[k];
      bool in_a = false;
      FlatLookup(F.nb, F.wt, a0, a1, x, &in_a);
      if (in_a) continue;
      LegacyTerm(p, x, F.nsz[k], 0, F.wt[k], &before, &after);
      seen_a |= x == p.ra;
      seen_b |= x == p.rb;
    }
    before = WarpSum(before);
    after = WarpSum(after);
    seen_a = __any_sync(kFull, seen_a);
    seen_b = __any_sync(kFull, seen_b);
    if (lane == 0) {
      // a row that does not list its own representative still pays for it
      if (!seen_a) LegacyTerm(p, p.ra, p.sa, 0, 0, &before, &after);
      if (p.rb != p.ra && !seen_b) LegacyTerm(p, p.rb, p.sb, 0, 0, &before, &after);
      out[2 * w] = before - after;
      out[2 * w + 1] = before;
    }
  }
}

thread_local std::string g_flat_error;

size_t AlignUp(size_t v, size_t a) { return (v + a - 1) / a * a; }

}  // namespace
}  // namespace beam

struct beam_flat_scorer {
  int device = 0;
  beam::OwnedStream stream;
  beam::DevBuf<unsigned char> d_in;
  beam::DevBuf<long long> d_out;
  beam::PinnedBuf<unsigned char> h_in;
  beam::PinnedBuf<long long> h_out;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  beam_flat_scorer_stats stats{};
  ~beam_flat_scorer() {
    for (cudaEvent_t e : ev) {
      if (e) cudaEventDestroy(e);
    }
    if (stream.s) cudaStreamSynchronize(stream.s);
    d_in.release();
    d_out.release();
  }
};

namespace {

int FlatFail(const std::string& msg) {
  beam::g_flat_error = msg;
  return -1;
}

}  // namespace

extern "C" {

const char* beam_flat_scorer_last_error(void) { return beam::g_flat_error.c_str(); }

int beam_flat_scorer_create(int32_t device, beam_flat_scorer** out) {
  if (!out) return FlatFail("null output handle");
  *out = nullptr;
  try {
    auto* s = new beam_flat_scorer();
    s->device = device;
    beam::CheckCuda(cudaSetDevice(device), "cudaSetDevice");
    beam::CheckCuda(cudaStreamCreateWithFlags(&s->stream.s, cudaStreamNonBlocking), "cudaStreamCreate");
    for (cudaEvent_t& e : s->ev) beam::CheckCuda(cudaEventCreate(&e), "cudaEventCreate");
    *out = s;
    return 0;
  } catch (const std::exception& ex) {
    return FlatFail(ex.what());
  }
}

void beam_flat_scorer_destroy(beam_flat_scorer* s) {
  if (!s) return;
  cudaSetDevice(s->device);
  delete s;
}

int beam_flat_scorer_memory_budget(beam_flat_scorer* s, int64_t* bytes) {
  if (!s || !bytes) return FlatFail("null argument");
  size_t free_b = 0, total_b = 0;
  cudaError_t st = cudaSetDevice(s->device);
  if (st == cudaSuccess) st = cudaMemGetInfo(&free_b, &total_b);
  if (st != cudaSuccess) return FlatFail(std::string("cudaMemGetInfo: ") + cudaGetErrorString(st));
  *bytes = static_cast<int64_t>(std::min<size_t>(free_b / 4, size_t{4} << 30));
  return 0;
}

int beam_flat_scorer_get_stats(const beam_flat_scorer* s, beam_flat_scorer_stats* out) {
  if (!s || !out) return FlatFail("null argument");
  *out = s->stats;
  return 0;
}

int beam_flat_scorer_score(beam_flat_scorer* s, const int32_t* pairs, int64_t count, const int32_t* offsets,
                           const int32_t* row_rep_ids, const int64_t* row_sizes, const int64_t* row_self_loops,
                           int32_t rows, const int32_t* neighbors, const int64_t* weights,
                           const int64_t* neighbor_sizes, int64_t entries, int64_t* gain, int64_t* before_cost) {
  using namespace beam;
  if (!s) return FlatFail("null scorer");
  if (count < 0 || rows < 0 || entries < 0) return FlatFail("negative size");
  if (count == 0) return 0;
  if (!pairs || !gain || !before_cost || !offsets || !row_rep_ids || !row_sizes || !row_self_loops ||
      (entries > 0 && (!neighbors || !weights || !neighbor_sizes))) {
    return FlatFail("null input or output pointer");
  }
  if (entries > INT32_MAX) return FlatFail("entries exceed the int offsets of FlatAggCSR");
  // the layout the kernel relies on: offsets rising from 0 to entries, rows
  // sorted by neighbour without repeats, pair indices naming rows
  if (offsets[0] != 0 || offsets[rows] != entries) return FlatFail("offsets must rise from 0 to entries");
  for (int32_t i = 0; i < rows; ++i) {
    if (offsets[i] > offsets[i + 1]) return FlatFail("offsets must rise from 0 to entries");
    for (int32_t k = offsets[i] + 1; k < offsets[i + 1]; ++k) {
      if (neighbors[k - 1] >= neighbors[k]) {
        return FlatFail("row " + std::to_string(i) + " is not sorted by neighbour without repeats");
      }
    }
  }
  for (int64_t p = 0; p < count; ++p) {
    if (pairs[2 * p] < 0 || pairs[2 * p] >= rows || pairs[2 * p + 1] < 0 || pairs[2 * p + 1] >= rows) {
      return FlatFail("pair " + std::to_string(p) + " names a row outside [0, rows)");
    }
  }
  try {
    CheckCuda(cudaSetDevice(s->device), "cudaSetDevice");
    AllocScope alloc(s->stream.s);
    // packed input: offsets | reps | neighbours | pairs (4-byte) then
    // weights | neighbour sizes | row sizes | self loops (8-byte)
    const size_t r1 = static_cast<size_t>(rows) + 1;
    const size_t ur = static_cast<size_t>(rows);
    const size_t ue = static_cast<size_t>(entries);
    const size_t up = static_cast<size_t>(count);
    size_t at = 0;
    const size_t o_off = at;
    at += 4 * r1;
    const size_t o_rep = at;
    at += 4 * ur;
    const size_t o_nb = at;
    at += 4 * ue;
    const size_t o_pair = at = AlignUp(at, 8);
    at += 8 * up;
    const size_t o_wt = at;
    at += 8 * ue;
    const size_t o_nsz = at;
    at += 8 * ue;
    const size_t o_rsz = at;
    at += 8 * ur;
    const size_t o_self = at;
    at += 8 * ur;
    const size_t total = at;
    s->h_in.ensure(total);
    s->d_in.ensure(total);
    s->h_out.ensure(2 * up);
    s->d_out.ensure(2 * up);
    unsigned char* h = s->h_in.p;
    std::memcpy(h + o_off, offsets, 4 * r1);
    std::memcpy(h + o_rep, row_rep_ids, 4 * ur);
    if (ue) std::memcpy(h + o_nb, neighbors, 4 * ue);
    std::memcpy(h + o_pair, pairs, 8 * up);
    if (ue) std::memcpy(h + o_wt, weights, 8 * ue);
    if (ue) std::memcpy(h + o_nsz, neighbor_sizes, 8 * ue);
    std::memcpy(h + o_rsz, row_sizes, 8 * ur);
    std::memcpy(h + o_self, row_self_loops, 8 * ur);
    cudaStream_t st = s->stream.s;
    unsigned char* d = s->d_in.p;
    CheckCuda(cudaMemcpyAsync(d, h, total, cudaMemcpyHostToDevice, st), "h2d flat block");
    FlatView F{reinterpret_cast<const int*>(d + o_off), reinterpret_cast<const int*>(d + o_rep),
               reinterpret_cast<const int*>(d + o_nb), reinterpret_cast<const long long*>(d + o_wt),
               reinterpret_cast<const long long*>(d + o_nsz), reinterpret_cast<const long long*>(d + o_rsz),
               reinterpret_cast<const long long*>(d + o_self)};
    const int grid = static_cast<int>(std::min<int64_t>((count + 7) / 8, 152 * 16));
    CheckCuda(cudaEventRecord(s->ev[0], st), "event");
    LegacyFlatScoreKernel<<<grid, kLegacyThreads, 0, st>>>(F, reinterpret_cast<const int2*>(d + o_pair), count,
                                                            s->d_out.p);
    CheckCuda(cudaGetLastError(), "legacy scoring launch");
    CheckCuda(cudaEventRecord(s->ev[1], st), "event");
    CheckCuda(cudaMemcpyAsync(s->h_out.p, s->d_out.p, 16 * up, cudaMemcpyDeviceToHost, st), "d2h results");
    CheckCuda(cudaStreamSynchronize(st), "sync");
    float ms = 0.f;
    CheckCuda(cudaEventElapsedTime(&ms, s->ev[0], s->ev[1]), "event elapsed");
    for (size_t p = 0; p < up; ++p) {
      gain[p] = s->h_out.p[2 * p];
      before_cost[p] = s->h_out.p[2 * p + 1];
    }
    s->stats.calls += 1;
    s->stats.kernel_launches += 1;
    s->stats.pairs += count;
    s->stats.h2d_bytes += static_cast<int64_t>(total);
    s->stats.d2h_bytes += static_cast<int64_t>(16 * up);
    s->stats.kernel_ms += ms;
    s->stats.max_pairs_per_launch = std::max<int64_t>(s->stats.max_pairs_per_launch, count);
    return 0;
  } catch (const std::exception& ex) {
    return FlatFail(ex.what());
  }
}

}  // extern "C"
