// Divide on the GPU: min-hash grouping of the active supernodes
// (Sweg::Divide, src/sweg.cpp:853-890, with SplitGroupByHashDims /
// FallbackSplitGroup / SupernodeMinHash at src/sweg.cpp:754-851).
//
// The reference recursion sorts a range by (min-hash of dimension
// dim_order[depth], rep) and recurses on equal-hash runs longer than
// divide_max_group. The same order is produced breadth-first: every
// unfinished segment (a run longer than divide_max_group) is already sorted by
// rep (it is a run of equal hashes of the previous depth, tie-broken by rep),
// so one stable sort by (segment, next hash) per depth - stable LSD radix
// sorts over the unfinished items, by the hash's high word then by segment
// index, followed by a fix-up that puts runs of equal high words into full
// hash order - yields (hash, rep) order inside each segment; equal-hash
// boundaries become new segment heads. After divide_hash_dims depths the remaining long segments are
// stably sorted by FallbackRank and cut into divide_max_group chunks. Groups
// are the final segments in position order, exactly the reference's DFS order.
//
// Min-hash per supernode = min over member nodes v and their CSR neighbours u
// of HashRank64(., dim, iter): one pass over the arcs whose source belongs to
// a supernode still in an unfinished segment, warp-aggregated atomicMin per
// supernode, plus one self term per node.

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cstring>
#include <numeric>

#include "engine.h"

namespace beam {
namespace {

__global__ void ActiveFlagsKernel(const int* __restrict__ qsize, int n, int* __restrict__ flags) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flags[i] = qsize[i] > 0 ? 1 : 0;
}

// order[scan[i]] = i for active reps; scan is exclusive.
__global__ void ScatterActiveKernel(const int* __restrict__ qsize, const int* __restrict__ scan, int n,
                                    int* __restrict__ order, int* __restrict__ head_flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && qsize[i] > 0) {
    const int p = scan[i];
    order[p] = i;
    head_flag[p] = p == 0 ? 1 : 0;
  }
}

// Segment descriptors from head flags: segid (inclusive scan - 1) per
// position, start per segment.
__global__ void SegStartsKernel(const int* __restrict__ head_flag, const int* __restrict__ incl, int count,
                                int* __restrict__ seg_start) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < count && head_flag[p]) seg_start[incl[p] - 1] = p;
}

__global__ void SegLenKernel(const int* __restrict__ seg_start, int segs, int count, int max_group,
                             int* __restrict__ seg_len, int* __restrict__ unf_flag, int* __restrict__ unf_len) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < segs) {
    const int end = s + 1 < segs ? seg_start[s + 1] : count;
    const int len = end - seg_start[s];
    seg_len[s] = len;
    const int unf = len > max_group ? 1 : 0;
    unf_flag[s] = unf;
    unf_len[s] = unf ? len : 0;
  }
}

// SegLenKernel over all count positions with the segment count read on the
// device (no host round trip): entries past the last segment are zeroed, so
// scans over count elements equal scans over the segments.
// unf_pk[s] = unfinished flag << 32 | unfinished item count: one exclusive
// scan gives both the unfinished-segment index (high word) and the compact
// item offset (low word, < 2^31, so no carry reaches the high word).
__global__ void SegLenAllKernel(const int* __restrict__ seg_start, const int* __restrict__ segs_p, int count,
                                int max_group, int* __restrict__ seg_len, int* __restrict__ unf_flag,
                                unsigned long long* __restrict__ unf_pk) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= count) return;
  const int segs = *segs_p;
  if (s < segs) {
    const int end = s + 1 < segs ? seg_start[s + 1] : count;
    const int len = end - seg_start[s];
    seg_len[s] = len;
    const int unf = len > max_group ? 1 : 0;
    unf_flag[s] = unf;
    unf_pk[s] = unf ? (1ull << 32) | static_cast<unsigned>(len) : 0ull;
  } else {
    unf_flag[s] = 0;
    unf_pk[s] = 0;
  }
}

// {segments, unfinished segments, their items} of a depth, for one read-back.
// Depth 0: one segment of all `count` active supernodes (only position 0
// carries a head flag). Writes what the scans and SegStarts / SegLenAll
// would: every item's inclusive head count is 1, and segment 0's start,
// length and unfinished flag, with both exclusive offsets 0.
__global__ void DepthZeroKernel(int count, int max_group, int* __restrict__ incl, int* __restrict__ seg_start,
                                int* __restrict__ seg_len, int* __restrict__ unf_flag,
                                unsigned long long* __restrict__ unf_ex) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= count) return;
  incl[p] = 1;
  if (p == 0) {
    const int unf = count > max_group ? 1 : 0;
    seg_start[0] = 0;
    seg_len[0] = count;
    unf_flag[0] = unf;
    unf_ex[0] = 0;
  }
}

__global__ void DepthCountsKernel(const int* __restrict__ incl_last, const unsigned long long* __restrict__ ex_last,
                                  const unsigned long long* __restrict__ pk_last, int* __restrict__ out) {
  const unsigned long long total = *ex_last + *pk_last;
  out[0] = *incl_last;
  out[1] = static_cast<int>(total >> 32);
  out[2] = static_cast<int>(total & 0xffffffffull);
}

// Compact the items of unfinished segments: pos_map[k] = position,
// item_seg[k] = compact segment index; segment begin/end in compact space.
__global__ void CompactItemsKernel(const int* __restrict__ incl, const int* __restrict__ seg_start,
                                   const int* __restrict__ seg_len, const int* __restrict__ unf_flag,
                                   const unsigned long long* __restrict__ unf_ex, int count,
                                   int* __restrict__ pos_map, int* __restrict__ item_seg,
                                   int* __restrict__ ubeg, int* __restrict__ uend) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= count) return;
  const int s = incl[p] - 1;
  if (!unf_flag[s]) return;
  const int r = p - seg_start[s];
  const int ui = static_cast<int>(unf_ex[s] >> 32);          // unfinished-segment index
  const int uo = static_cast<int>(unf_ex[s] & 0xffffffffull);  // its first compact item
  const int k = uo + r;
  pos_map[k] = p;
  item_seg[k] = ui;
  if (r == 0) {
    ubeg[ui] = uo;
    uend[ui] = uo + seg_len[s];
  }
}

__global__ void MarkNeedKernel(const int* __restrict__ order, const int* __restrict__ pos_map, int items,
                               int* __restrict__ need, int stamp, unsigned long long* __restrict__ hash) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < items) {
    const int rep = order[pos_map[k]];
    need[rep] = stamp;
    hash[rep] = ~0ull;
  }
}

// One lane per arc (plus one per node for the node's own rank). Lanes of a
// warp whose sources share a supernode combine their minima before a single
// atomicMin; arcs are grouped by source, so this removes most atomics.
// Each warp takes kHashUnroll consecutive 32-item steps at a time and issues
// each level of the dependent chain (source, its label, the label's need
// stamp, the target) for all of them before the next level, so a lane keeps
// kHashUnroll loads in flight instead of one: the pass is bound by that
// chain's latency, not by its bytes. Steps whose lanes need nothing (most of
// them past depth 0, where only the oversized segments are hashed) skip the
// warp reduction.
constexpr int kHashUnroll = 4;

__global__ void __launch_bounds__(256) MinHashKernel(const int* __restrict__ arc_src, const int* __restrict__ col,
                                                     const int* __restrict__ label, const int* __restrict__ need,
                                                     long long arcs, int n, int stamp, uint64_t base,
                                                     unsigned long long* __restrict__ hash,
                                                     unsigned long long* __restrict__ stats) {
  const long long total = arcs + n;
  // algorithmic bytes of one dimension: per arc its source, the source's
  // label and its need stamp (12 B), per node its label and stamp (8 B), and
  // the target of every arc that is hashed (4 B, counted per warp below)
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    atomicAdd(&stats[kStDivideBytes], 12ull * static_cast<unsigned long long>(arcs) +
                                          8ull * static_cast<unsigned long long>(n));
  }
  unsigned hashed_arcs = 0;  // warp-uniform; a warp's share of one launch stays far below 2^32
  const int lane = threadIdx.x & 31;
  const long long warp = (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = (static_cast<long long>(gridDim.x) * blockDim.x) >> 5;
  constexpr long long kTile = 32ll * kHashUnroll;
  for (long long t0 = warp * kTile; t0 < total; t0 += nwarps * kTile) {
    int node[kHashUnroll], rep[kHashUnroll];
#pragma unroll
    for (int u = 0; u < kHashUnroll; ++u) {
      const long long t = t0 + 32 * u + lane;
      node[u] = t < arcs ? arc_src[t] : t < total ? static_cast<int>(t - arcs) : -1;
    }
#pragma unroll
    for (int u = 0; u < kHashUnroll; ++u) rep[u] = node[u] >= 0 ? label[node[u]] : -1;
#pragma unroll
    for (int u = 0; u < kHashUnroll; ++u) {
      if (rep[u] >= 0 && need[rep[u]] != stamp) rep[u] = -1;
    }
    int x[kHashUnroll];
#pragma unroll
    for (int u = 0; u < kHashUnroll; ++u) {
      const long long t = t0 + 32 * u + lane;
      x[u] = rep[u] < 0 ? 0 : t < arcs ? col[t] : node[u];
      hashed_arcs += __popc(__ballot_sync(0xffffffffu, rep[u] >= 0 && t < arcs));
    }
#pragma unroll
    for (int u = 0; u < kHashUnroll; ++u) {
      if (__ballot_sync(0xffffffffu, rep[u] >= 0) == 0u) continue;
      const unsigned long long h = rep[u] >= 0 ? HashRankWithBase(base, x[u]) : ~0ull;
      // exact minimum over the lanes holding the same supernode: high words
      // first, then low words among the lanes that hold the minimal high word
      const unsigned mask = __match_any_sync(0xffffffffu, rep[u]);
      const unsigned hi = static_cast<unsigned>(h >> 32);
      const unsigned lo = static_cast<unsigned>(h & 0xffffffffu);
      const unsigned mhi = __reduce_min_sync(mask, hi);
      const unsigned mlo = __reduce_min_sync(mask, hi == mhi ? lo : 0xffffffffu);
      const unsigned long long g = (static_cast<unsigned long long>(mhi) << 32) | mlo;
      const int leader = __ffs(mask) - 1;
      if (rep[u] >= 0 && lane == leader) atomicMin(&hash[rep[u]], g);
    }
  }
  if (lane == 0 && hashed_arcs) atomicAdd(&stats[kStDivideBytes], 4ull * static_cast<unsigned long long>(hashed_arcs));
}

__global__ void GatherKeysKernel(const int* __restrict__ order, const int* __restrict__ pos_map, int items,
                                 const unsigned long long* __restrict__ hash, int fallback, uint64_t seed,
                                 int iter, unsigned long long* __restrict__ keys, unsigned* __restrict__ keys_hi,
                                 int* __restrict__ vals) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < items) {
    const int rep = order[pos_map[k]];
    const unsigned long long key = fallback ? FallbackRank(seed, rep, iter) : hash[rep];
    keys[k] = key;
    keys_hi[k] = static_cast<unsigned>(key >> 32);  // the radix sort's key
    vals[k] = rep;
  }
}

__global__ void IotaKernel(int* __restrict__ out, int items) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < items) out[k] = k;
}

__global__ void SegKeyKernel(const int* __restrict__ item_seg, const int* __restrict__ perm, int items,
                             int* __restrict__ segkey) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < items) segkey[j] = item_seg[perm[j]];
}

__global__ void GatherSortedKernel(const int* __restrict__ perm, int items, const unsigned long long* __restrict__ keys,
                                   const int* __restrict__ vals, unsigned long long* __restrict__ keys_out,
                                   int* __restrict__ vals_out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < items) {
    keys_out[j] = keys[perm[j]];
    vals_out[j] = vals[perm[j]];
  }
}

// The radix sort orders the items by the high 32 bits of their keys only
// (half the passes); items with equal high words stay in input order. Where
// such a run mixes low words it is put in full-key order below, which gives
// the order of a stable sort by the whole key. Such runs need two distinct
// 64-bit hashes with equal high words, so they are few and short.
// First pass (keys are only read): the first position of each run where the
// low word changes records the run's start.
__global__ void MixedRunsKernel(const unsigned long long* __restrict__ keys, const int* __restrict__ item_seg,
                                const int* __restrict__ ubeg, int items, int* __restrict__ list,
                                int* __restrict__ cnt) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x + 1; j < items; j += gridDim.x * blockDim.x) {
    const unsigned long long kj = keys[j];
    const unsigned long long kp = keys[j - 1];
    if (kj == kp || (kj >> 32) != (kp >> 32)) continue;
    const int sg = item_seg[j];
    if (item_seg[j - 1] != sg) continue;
    const int b = ubeg[sg];
    const unsigned long long hi = kj >> 32;
    int r0 = j - 1;
    bool first = true;
    while (r0 > b && (keys[r0 - 1] >> 32) == hi) {
      if (keys[r0 - 1] != keys[r0]) {
        first = false;  // an earlier change records this run
        break;
      }
      --r0;
    }
    if (first) list[atomicAdd(cnt, 1)] = r0;
  }
}

// Second pass, a warp per recorded run: the run is reordered stably by its
// keys (the items of the smallest remaining key move first, in their order)
// via the scratch arrays. A run shares its high word, so each round takes the
// smallest remaining low word by one warp reduction and moves its items by a
// ballot compaction; a long run (a large segment of one min-hash colliding
// with another) is read 32 items at a time instead of by one thread.
__global__ void __launch_bounds__(256) SortMixedRunsKernel(unsigned long long* __restrict__ keys,
                                                           int* __restrict__ vals, const int* __restrict__ item_seg,
                                                           const int* __restrict__ uend, const int* __restrict__ list,
                                                           const int* __restrict__ cnt,
                                                           unsigned long long* __restrict__ tk, int* __restrict__ tv) {
  constexpr unsigned kFull = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const int nruns = *cnt;
  const int nwarps = static_cast<int>((static_cast<long long>(gridDim.x) * blockDim.x) >> 5);
  for (int t = static_cast<int>((static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5); t < nruns;
       t += nwarps) {
    const int r0 = list[t];
    const unsigned hi = static_cast<unsigned>(keys[r0] >> 32);
    const int e = uend[item_seg[r0]];
    int r1 = r0 + 1;  // one past the run: the first later item of another high word
    for (;;) {
      const int i = r1 + lane;
      const unsigned in = __ballot_sync(kFull, i < e && static_cast<unsigned>(keys[i] >> 32) == hi);
      if (in != kFull) {
        r1 += __ffs(~in) - 1;
        break;
      }
      r1 += 32;
    }
    int w = r0;
    unsigned last = 0;
    bool any = false;  // a low word has been moved (last is valid)
    while (w < r1) {
      unsigned mn = 0xffffffffu;
      bool have = false;
      for (int i = r0 + lane; i < r1; i += 32) {
        const unsigned lo = static_cast<unsigned>(keys[i]);
        if ((!any || lo > last) && lo <= mn) {
          mn = lo;
          have = true;
        }
      }
      mn = __reduce_min_sync(kFull, have ? mn : 0xffffffffu);
      if (__ballot_sync(kFull, have) == 0u) break;  // every item moved
      for (int i0 = r0; i0 < r1; i0 += 32) {
        const int i = i0 + lane;
        unsigned long long k = 0;
        bool hit = false;
        if (i < r1) {
          k = keys[i];
          hit = static_cast<unsigned>(k) == mn && (!any || mn > last);
        }
        const unsigned m = __ballot_sync(kFull, hit);
        if (hit) {
          const int at = w + __popc(m & lt);
          tk[at] = k;
          tv[at] = vals[i];
        }
        w += __popc(m);
      }
      last = mn;
      any = true;
    }
    __syncwarp();
    for (int i = r0 + lane; i < r1; i += 32) {
      keys[i] = tk[i];
      vals[i] = tv[i];
    }
    __syncwarp();
  }
}

__global__ void ScatterSortedKernel(const int* __restrict__ pos_map, const int* __restrict__ item_seg,
                                    const int* __restrict__ ubeg, int items,
                                    const unsigned long long* __restrict__ keys, const int* __restrict__ vals,
                                    int fallback, int max_group, int* __restrict__ order,
                                    int* __restrict__ head_flag) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= items) return;
  const int p = pos_map[k];
  order[p] = vals[k];
  const int r = k - ubeg[item_seg[k]];
  if (r > 0) {
    const bool head = fallback ? (r % max_group) == 0 : keys[k] != keys[k - 1];
    if (head) head_flag[p] = 1;
  }
}

__global__ void GroupInfoKernel(const int* __restrict__ order, const int* __restrict__ incl,
                                const int* __restrict__ seg_start, const int* __restrict__ seg_len, int count,
                                int* __restrict__ group_of, int* __restrict__ idx_in_group,
                                const int* __restrict__ qlen, unsigned* __restrict__ gent,
                                unsigned long long* __restrict__ stats) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= count) return;
  const int s = incl[p] - 1;
  const int rep = order[p];
  group_of[rep] = s;
  idx_in_group[rep] = p - seg_start[s];
  // row entries per group: routing to a prepare kernel and, as an upper
  // bound for the iteration, the deferred groups' sort slots
  atomicAdd(&gent[s], static_cast<unsigned>(qlen[rep]));
  // largest group: warp maximum first, one atomic per warp
  unsigned v = p == seg_start[s] ? static_cast<unsigned>(seg_len[s]) : 0u;
  const unsigned active = __activemask();
  v = __reduce_max_sync(active, v);
  if ((threadIdx.x & 31) == __ffs(active) - 1 && v > 0) {
    atomicMax(&stats[kStDivideMaxGroup], static_cast<unsigned long long>(v));
  }
}

inline int Blocks(long long items, int threads) {
  return static_cast<int>((items + threads - 1) / threads);
}

}  // namespace

void Engine::Divide(int iter) {
  AllocScope alloc(stream_);
  const int n = n_;
  const int T = 256;
  cudaStream_t s = stream_;
  // scratch arrays: d_counts_ holds [flags | scan | seg_len | unf_flag | unf_len | (2 spare) | ubeg | uend]
  d_counts_.ensure(static_cast<size_t>(n) * 9 + 64);  // + 3 depth counts after uend
  int* flags = d_counts_.p;
  int* scan = flags + n;
  int* seg_len = scan + n;
  int* unf_flag = seg_len + n;
  int* unf_len = unf_flag + n;
  int* ubeg = unf_len + 3 * n;
  int* uend = ubeg + n;
  int* seg_start = d_seg_beg_.p;
  int* item_seg = d_seg_end_.p;
  int* fix_cnt = uend + n + 8;  // mixed-run counter (cleared before each first pass)
  d_fix_list_.ensure(static_cast<size_t>(n) + 1);
  d_keys_hi_[0].ensure(static_cast<size_t>(n) + 1);
  d_unf_pk_[0].ensure(static_cast<size_t>(n) + 1);
  d_unf_pk_[1].ensure(static_cast<size_t>(n) + 1);
  unsigned long long* unf_pk = d_unf_pk_[0].p;  // per segment: unfinished flag << 32 | unfinished items
  unsigned long long* unf_ex = d_unf_pk_[1].p;  // its exclusive scan
  d_keys_hi_[1].ensure(static_cast<size_t>(n) + 1);
  CheckCuda(cudaMemsetAsync(fix_cnt, 0, sizeof(int), s), "memset mixed-run counter");

  auto scan_excl = [&](const int* in, int* out, int items) {
    size_t bytes = 0;
    CheckCuda(cub::DeviceScan::ExclusiveSum(nullptr, bytes, in, out, items, s), "cub scan size");
    d_cub_tmp_.ensure(bytes);
    CheckCuda(cub::DeviceScan::ExclusiveSum(d_cub_tmp_.p, bytes, in, out, items, s), "cub exclusive scan");
  };
  auto scan_incl = [&](const int* in, int* out, int items) {
    size_t bytes = 0;
    CheckCuda(cub::DeviceScan::InclusiveSum(nullptr, bytes, in, out, items, s), "cub scan size");
    d_cub_tmp_.ensure(bytes);
    CheckCuda(cub::DeviceScan::InclusiveSum(d_cub_tmp_.p, bytes, in, out, items, s), "cub inclusive scan");
  };
  auto fetch2 = [&](const int* a, const int* b, int* ha, int* hb) {
    CheckCuda(cudaMemcpyAsync(h_pin_.p, a, sizeof(int), cudaMemcpyDeviceToHost, s), "d2h");
    CheckCuda(cudaMemcpyAsync(reinterpret_cast<int*>(h_pin_.p) + 1, b, sizeof(int), cudaMemcpyDeviceToHost, s),
              "d2h");
    CheckCuda(cudaStreamSynchronize(s), "sync");
    *ha = reinterpret_cast<int*>(h_pin_.p)[0];
    *hb = reinterpret_cast<int*>(h_pin_.p)[1];
  };

  // Active supernodes in ascending id order.
  ++launches_;
  ActiveFlagsKernel<<<Blocks(n, T), T, 0, s>>>(d_qsize_.p, n, flags);
  scan_excl(flags, scan, n);
  CheckCuda(cudaMemsetAsync(d_head_flag_.p, 0, sizeof(int) * static_cast<size_t>(n), s), "memset");
  ++launches_;
  ScatterActiveKernel<<<Blocks(n, T), T, 0, s>>>(d_qsize_.p, scan, n, d_order_.p, d_head_flag_.p);
  // active supernodes: known on the host after a Merge (n - accepted
  // merges, read back with the Merge's final synchronisation), else read
  int count = 0;
  if (known_active_ >= 0) {
    count = static_cast<int>(known_active_);
  } else {
    int last_scan = 0, last_flag = 0;
    fetch2(scan + n - 1, flags + n - 1, &last_scan, &last_flag);
    count = last_scan + last_flag;
  }
  n_active_ = count;

  // dim_order: dims stable-sorted by (DimRank, dim)
  std::vector<int> dim_order(static_cast<size_t>(cfg_.divide_hash_dims));
  std::iota(dim_order.begin(), dim_order.end(), 0);
  std::stable_sort(dim_order.begin(), dim_order.end(), [&](int a, int b) {
    const uint64_t ra = DimRank(cfg_.seed, a, iter);
    const uint64_t rb = DimRank(cfg_.seed, b, iter);
    if (ra != rb) return ra < rb;
    return a < b;
  });

  int segs = 0;
  if (count > 0) {
    bool settled = false;  // the loop ended with segs / seg_start / seg_len of the final groups
    for (int depth = 0; depth <= cfg_.divide_hash_dims; ++depth) {
      const bool fallback = depth == cfg_.divide_hash_dims;
      if (depth == 0) {
        ++launches_;
        DepthZeroKernel<<<Blocks(count, T), T, 0, s>>>(count, cfg_.divide_max_group, scan, seg_start, seg_len,
                                                       unf_flag, unf_ex);
      } else {
        scan_incl(d_head_flag_.p, scan, count);
        ++launches_;
        SegStartsKernel<<<Blocks(count, T), T, 0, s>>>(d_head_flag_.p, scan, count, seg_start);
        ++launches_;
        SegLenAllKernel<<<Blocks(count, T), T, 0, s>>>(seg_start, scan + count - 1, count, cfg_.divide_max_group,
                                                       seg_len, unf_flag, unf_pk);
        size_t pk_bytes = 0;
        CheckCuda(cub::DeviceScan::ExclusiveSum(nullptr, pk_bytes, unf_pk, unf_ex, count, s), "cub scan size");
        d_cub_tmp_.ensure(pk_bytes);
        CheckCuda(cub::DeviceScan::ExclusiveSum(d_cub_tmp_.p, pk_bytes, unf_pk, unf_ex, count, s),
                  "cub exclusive scan");
      }
      // segments, unfinished segments and their items: known on the host at
      // depth 0 (one segment of all active supernodes), one read-back later
      int hc[3];
      if (depth == 0) {
        hc[0] = 1;
        hc[1] = count > cfg_.divide_max_group ? 1 : 0;
        hc[2] = hc[1] ? count : 0;
      } else {
        int* dc = uend + n;
        ++launches_;
        DepthCountsKernel<<<1, 1, 0, s>>>(scan + count - 1, unf_ex + count - 1, unf_pk + count - 1, dc);
        CheckCuda(cudaMemcpyAsync(h_pin_.p, dc, 3 * sizeof(int), cudaMemcpyDeviceToHost, s), "d2h depth counts");
        CheckCuda(cudaStreamSynchronize(s), "sync");
        std::memcpy(hc, h_pin_.p, sizeof(hc));
      }
      segs = hc[0];
      const int nu = hc[1];
      if (nu == 0) {
        settled = true;
        break;
      }
      const int items = hc[2];
      ++launches_;
      CompactItemsKernel<<<Blocks(count, T), T, 0, s>>>(scan, seg_start, seg_len, unf_flag, unf_ex, count,
                                                        d_pos_map_.p, item_seg, ubeg, uend);
      if (fallback) {
        hstats_.divide_fallback_splits += static_cast<uint64_t>(nu);
      } else {
        ++need_stamp_;
        ++launches_;
        MarkNeedKernel<<<Blocks(items, T), T, 0, s>>>(d_order_.p, d_pos_map_.p, items, d_need_.p, need_stamp_,
                                                      d_hash_.p);
        const uint64_t base = HashRankBase(cfg_.seed, dim_order[static_cast<size_t>(depth)], iter);
        BeginTimed(kTimeDivide);
        ++launches_;
        MinHashKernel<<<152 * 8, 256, 0, s>>>(d_arc_src_.p, d_col_.p, d_label_.p, d_need_.p, arcs_, n,
                                              need_stamp_, base, d_hash_.p, d_stats_.p);
        EndTimed(kTimeDivide);
      }
      ++launches_;
      GatherKeysKernel<<<Blocks(items, T), T, 0, s>>>(d_order_.p, d_pos_map_.p, items, d_hash_.p, fallback ? 1 : 0,
                                                      cfg_.seed, iter, d_keys_.p, d_keys_hi_[0].p, d_vals_.p);
      // (segment, key) order, stable on the rep order inside each segment:
      // a stable LSD radix sort by key, then a stable one by segment index.
      ++launches_;
      IotaKernel<<<Blocks(items, T), T, 0, s>>>(d_perm_.p, items);
      size_t bytes = 0;
      // by the high key words (equal-high runs are put in key order below;
      // the full keys follow the permutation in GatherSortedKernel)
      CheckCuda(cub::DeviceRadixSort::SortPairs(nullptr, bytes, d_keys_hi_[0].p, d_keys_hi_[1].p, d_perm_.p,
                                                d_perm_alt_.p, items, 0, 32, s), "cub radix sort size");
      d_cub_tmp_.ensure(bytes);
      CheckCuda(cub::DeviceRadixSort::SortPairs(d_cub_tmp_.p, bytes, d_keys_hi_[0].p, d_keys_hi_[1].p, d_perm_.p,
                                                d_perm_alt_.p, items, 0, 32, s), "cub radix sort");
      int* perm = d_perm_alt_.p;
      if (nu > 1) {
        int bits = 1;
        while ((1 << bits) < nu) ++bits;
        ++launches_;
        SegKeyKernel<<<Blocks(items, T), T, 0, s>>>(item_seg, d_perm_alt_.p, items, d_segkey_.p);
        bytes = 0;
        CheckCuda(cub::DeviceRadixSort::SortPairs(nullptr, bytes, d_segkey_.p, d_segkey_alt_.p, d_perm_alt_.p,
                                                  d_perm_.p, items, 0, bits, s), "cub radix sort size");
        d_cub_tmp_.ensure(bytes);
        CheckCuda(cub::DeviceRadixSort::SortPairs(d_cub_tmp_.p, bytes, d_segkey_.p, d_segkey_alt_.p,
                                                  d_perm_alt_.p, d_perm_.p, items, 0, bits, s), "cub radix sort");
        perm = d_perm_.p;
      }
      ++launches_;
      GatherSortedKernel<<<Blocks(items, T), T, 0, s>>>(perm, items, d_keys_.p, d_vals_.p, d_keys_alt_.p,
                                                        d_vals_alt_.p);
      // runs of equal high words with mixed low words into full-key order
      // (d_keys_ / d_vals_ are free once gathered)
      ++launches_;
      CheckCuda(cudaMemsetAsync(fix_cnt, 0, sizeof(int), s), "memset mixed-run counter");
      MixedRunsKernel<<<Blocks(items, T), T, 0, s>>>(d_keys_alt_.p, item_seg, ubeg, items, d_fix_list_.p, fix_cnt);
      ++launches_;
      SortMixedRunsKernel<<<152 * 2, 256, 0, s>>>(d_keys_alt_.p, d_vals_alt_.p, item_seg, uend, d_fix_list_.p,
                                                  fix_cnt, d_keys_.p, d_vals_.p);
      ++launches_;
      ScatterSortedKernel<<<Blocks(items, T), T, 0, s>>>(d_pos_map_.p, item_seg, ubeg, items, d_keys_alt_.p,
                                                         d_vals_alt_.p, fallback ? 1 : 0, cfg_.divide_max_group,
                                                         d_order_.p, d_head_flag_.p);
    }
    // final segments are the groups (already described when the loop
    // settled; after the fallback depth they are recounted)
    if (!settled) {
      scan_incl(d_head_flag_.p, scan, count);
      ++launches_;
      SegStartsKernel<<<Blocks(count, T), T, 0, s>>>(d_head_flag_.p, scan, count, seg_start);
      int seg_total = 0, dummy = 0;
      fetch2(scan + count - 1, scan + count - 1, &seg_total, &dummy);
      segs = seg_total;
      ++launches_;
      SegLenKernel<<<Blocks(segs, T), T, 0, s>>>(seg_start, segs, count, cfg_.divide_max_group, seg_len, unf_flag,
                                                 unf_len);
    }
    d_gent_.ensure(static_cast<size_t>(segs) + 1);
    CheckCuda(cudaMemsetAsync(d_gent_.p, 0, sizeof(unsigned) * static_cast<size_t>(segs), s), "memset gent");
    ++launches_;
    GroupInfoKernel<<<Blocks(count, T), T, 0, s>>>(d_order_.p, scan, seg_start, seg_len, count, d_group_of_.p,
                                                   d_idx_in_group_.p, d_qlen_.p, d_gent_.p, d_stats_.p);
    CheckCuda(cudaMemcpyAsync(d_gstart_.p, seg_start, sizeof(int) * static_cast<size_t>(segs),
                              cudaMemcpyDeviceToDevice, s), "copy gstart");
    CheckCuda(cudaMemcpyAsync(d_glen_.p, seg_len, sizeof(int) * static_cast<size_t>(segs),
                              cudaMemcpyDeviceToDevice, s), "copy glen");
  }
  n_groups_ = segs;
  // one block of every group: Merge plans the iteration on the device from
  // d_glen_ / d_gent_, so nothing is read back here
  plan_on_device_ = static_cast<long long>(cfg_.group_batch_size) >= static_cast<long long>(segs);
  if (!plan_on_device_) {
    h_glen_.resize(static_cast<size_t>(segs));
    h_gent_.resize(static_cast<size_t>(segs));
    if (segs > 0) {
      CheckCuda(cudaMemcpyAsync(h_glen_.data(), d_glen_.p, sizeof(int) * static_cast<size_t>(segs),
                                cudaMemcpyDeviceToHost, s), "d2h glen");
      CheckCuda(cudaMemcpyAsync(h_gent_.data(), d_gent_.p, sizeof(unsigned) * static_cast<size_t>(segs),
                                cudaMemcpyDeviceToHost, s), "d2h gent");
    }
    CheckCuda(cudaStreamSynchronize(s), "divide sync");
  }
  hstats_.groups_last = static_cast<uint64_t>(segs);
  hstats_.active_last = static_cast<uint64_t>(count);
}

}  // namespace beam
