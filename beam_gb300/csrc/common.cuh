// Device-side building blocks shared by the merge-loop kernels: the packed
// quotient-row entry, the exact integer block cost, the min-hash ranks, warp
// reductions and the counters the kernels accumulate.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace beam {

// One quotient-row entry: neighbour supernode id in the high 32 bits, edge
// count in the low 32 bits, so sorting the packed value sorts by neighbour.
using Entry = unsigned long long;

__host__ __device__ __forceinline__ int EntNb(Entry e) { return static_cast<int>(e >> 32); }
__host__ __device__ __forceinline__ long long EntCnt(Entry e) {
  return static_cast<long long>(static_cast<uint32_t>(e & 0xffffffffull));
}
__host__ __device__ __forceinline__ Entry MakeEnt(int nb, long long cnt) {
  return (static_cast<Entry>(static_cast<uint32_t>(nb)) << 32) |
         static_cast<Entry>(static_cast<uint32_t>(cnt));
}

// Counters accumulated on the device; names follow the reference's
// RuntimeStats / IterationProfile fields (include/sweg.hpp:83-386).
enum Stat : int {
  kStGroupCount = 0,          // merge_group_count
  kStGroupMaxSize,            // merge_group_max_size (atomicMax)
  kStRawPairCount,            // merge_raw_pair_count
  kStCandAfterPrune,          // merge_candidate_pairs_after_prune
  kStProxyExamined,           // candidate_proxy_pairs_examined
  kStExactCalls,              // merge_exact_gain_calls
  kStInputNnz,                // exact_gain_input_nnz (row-view sizes)
  kStRawA,                    // exact_raw_entries_a
  kStRawB,                    // exact_raw_entries_b
  kStUnion,                   // exact_union_neighbors
  kStOverlap,                 // exact_overlap_neighbors
  kStPositive,                // merge_positive_gain_pairs
  kStRejThreshold,            // merge_rejected_by_threshold
  kStRejOverlap,              // merge_rejected_by_overlap
  kStCandPairs,               // merge_candidate_pairs
  kStSelected,                // merge_selected_pairs
  kStLocalGain,               // merge_total_local_gain
  kStValidationCalls,         // validation_exact_calls
  kStValidationWork,          // validation_exact_row_entry_work
  kStAccepted,                // accepted_merges_after_validation
  kStRejNonpositive,          // rejected_nonpositive
  kStTouched,                 // update_touched_quotient_entries
  kStIsolatedGain,            // isolated_gain_sum
  kStRowsRewritten,           // neighbour rows rewritten (beam-gb300's own counter)
  kStRowEntriesRewritten,     // entries read by row rewrites (beam-gb300's own counter)
  kStDivideMaxGroup,          // divide_max_group_size (atomicMax)
  kStDivideFallback,          // divide_fallback_splits
  kStScoreBytes,              // algorithmic bytes of the scoring kernel
  kStPrepareBytes,            // algorithmic bytes of the prepare kernel
  kStUpdateBytes,             // algorithmic bytes of the row-update kernels
  kStDivideBytes,             // algorithmic bytes of the min-hash kernel
  kStRkRanked,                // candidate pairs scored by the ranker
  kStRkPruned,                // of which pruned before exact scoring
  kStRkAuditPassing,          // audit: ranked pairs passing the threshold filter
  kStRkAuditLost,             // audit: pruned pairs among them
  kStCount
};

// Error codes raised by kernels; the host turns them into messages.
enum ErrCode : int {
  kErrNone = 0,
  kErrBlockCost = 1,        // edge count outside [0, capacity]
  kErrAsymmetric = 2,       // e(a,b) differs between rows a and b
  kErrGroupTooLarge = 3,    // group beyond the compiled maximum
  kErrScratch = 4,          // per-block scratch exhausted
  kErrPool = 5,             // quotient entry pool exhausted
  kErrValidation = 6,       // commit-time gain differs from the scored gain
  kErrKeyRange = 7,         // gain outside the packed sort-key range
  kErrInactive = 8,         // scoring request on an inactive supernode
  kErrSlots = 9,            // a group's row entries exceed its sort slots
  kErrGraph = 10,           // a neighbour out of range or a self-loop in the input CSR
};

struct DevError {
  int code;
  int a;
  int b;
  int c;
};

__device__ __forceinline__ void RaiseError(DevError* err, int code, int a, int b, int c) {
  if (atomicCAS(&err->code, 0, code) == 0) {
    err->a = a;
    err->b = b;
    err->c = c;
  }
}

// CostOracle::BlockCost (src/cost_oracle.cpp:93-110): min(e, 1 + cap - e)
// with cap = s(s-1)/2 inside a supernode and s1*s2 across. Sizes are below
// 2^31, so every product fits in int64; an edge count outside [0, cap] marks
// the state invalid.
__device__ __forceinline__ long long BlockCost(long long s1, long long s2, long long e, bool internal,
                                               int& bad) {
  const long long cap = internal ? s1 * (s1 - 1) / 2 : s1 * s2;
  bad |= (e < 0) | (e > cap);
  const long long alt = 1 + cap - e;
  return e < alt ? e : alt;
}

// Sweg::EncodeCostForPair (src/sweg.cpp:1423-1433), no range checks.
__device__ __forceinline__ long long EncodeCostForPair(int rep_u, long long size_u, int rep_x,
                                                       long long size_x, long long edges) {
  const long long cap = rep_u == rep_x ? size_u * (size_u - 1) / 2 : size_u * size_x;
  const long long alt = 1 + cap - edges;
  return edges < alt ? edges : alt;
}

// Sweg::SplitMix64 and the rank hashes (src/sweg.cpp:731-752, 2290-2295).
__host__ __device__ __forceinline__ uint64_t SplitMix64(uint64_t x) {
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}
// HashRank64 with the node-independent part precomputed:
// base = seed ^ K2*(dim+1) ^ K3*(iter+1).
__host__ __device__ __forceinline__ uint64_t HashRankWithBase(uint64_t base, int node) {
  return SplitMix64(base ^ (0x9e3779b97f4a7c15ull * static_cast<uint64_t>(node + 1)));
}
__host__ __device__ __forceinline__ uint64_t HashRankBase(uint64_t seed, int dim, int iter) {
  return seed ^ (0xbf58476d1ce4e5b9ull * static_cast<uint64_t>(dim + 1)) ^
         (0x94d049bb133111ebull * static_cast<uint64_t>(iter + 1));
}
__host__ __device__ __forceinline__ uint64_t DimRank(uint64_t seed, int dim, int iter) {
  uint64_t x = seed;
  x ^= 0x9e3779b97f4a7c15ull * static_cast<uint64_t>(dim + 1);
  x ^= 0xbf58476d1ce4e5b9ull * static_cast<uint64_t>(iter + 1);
  return SplitMix64(x);
}
__host__ __device__ __forceinline__ uint64_t FallbackRank(uint64_t seed, int rep, int iter) {
  uint64_t x = seed;
  x ^= 0x9e3779b97f4a7c15ull * static_cast<uint64_t>(rep + 1);
  x ^= 0xbf58476d1ce4e5b9ull * static_cast<uint64_t>(iter + 1);
  x ^= 0xd6e8feb86659fd93ull;
  return SplitMix64(x);
}

__device__ __forceinline__ long long WarpSum(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
// one redux.sync instead of five shuffles (the same two's-complement sum)
__device__ __forceinline__ int WarpSumInt(int v) { return __reduce_add_sync(0xffffffffu, v); }
__device__ __forceinline__ long long WarpMax(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}

// Lower bound of neighbour id `key` in a sorted row.
__device__ __forceinline__ int RowLowerBound(const Entry* row, int len, int key) {
  int lo = 0, hi = len;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (EntNb(row[mid]) < key) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// Edge count to neighbour `key` (0 when absent).
__device__ __forceinline__ long long RowLookup(const Entry* row, int len, int key) {
  const int p = RowLowerBound(row, len, key);
  return (p < len && EntNb(row[p]) == key) ? EntCnt(row[p]) : 0;
}

// Index of the real group owning a candidate slot: last ri in [lo, hi) with
// off[ri] <= slot.
__device__ __forceinline__ int OwnerOfSlot(const long long* off, int lo, int hi, long long slot) {
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (off[mid] <= slot) lo = mid; else hi = mid;
  }
  return lo;
}

// Device view of the quotient graph.
struct QuotientView {
  Entry* ent;           // entry pool
  long long* off;       // row offset into the pool
  int* len;             // row length
  int* cap;             // row capacity
  int* size;            // supernode size (0 when inactive)
  long long* internal;  // internal edge count
};

}  // namespace beam
