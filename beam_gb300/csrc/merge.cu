// Merge on the GPU: the blocked EA merge loop (Sweg::Merge, blocked mode,
// src/sweg.cpp:953-1145), one block of group_batch_size groups at a time
// (64 in the reference's recommended mode; one block of all groups in the
// batched form).
//
//   Plan*Kernel        the block bookkeeping of a one-block iteration on the
//                      device (lists and offsets of the groups)
//   Prepare*Kernel     EA-proxy candidates per group (src/sweg.cpp:1598-1727,
//                      1800-1999): a warp per small group; big groups by CTA
//                      or by a GPU-wide sort of their row entries
//   ScoreKernel        exact merge gain per candidate pair
//                      (QuotientGraph::ExactMergeGainPersistentImpl,
//                      src/quotient_graph.cpp:340-462)
//   Select*Kernel      reciprocal threshold filter + g0 greedy selection
//                      (src/sweg.cpp:2146-2186, 2188-2281)
//   Commit*Kernel,     CommitSelectedPairs + Update_S + QuotientGraph::Merge
//   RewriteRowsKernel  for the block (src/sweg.cpp:2665-2769, 2977-3015,
//                      src/quotient_graph.cpp:628-742): sizes, internal
//                      counts, member lists, keep rows rebuilt from
//                      keep+remove, neighbour rows of removed supernodes
//                      rewritten in place
//   VerifyKernel       optional commit-time re-scoring (--verify-cuda-gain)
//
// The reference validates every selected pair of a block before applying any
// of them (Update_S runs after the validation loop), and the pairs of a block
// are endpoint-disjoint, so the block's merges are applied as one batch; the
// resulting rows are the canonical sorted, count-summed rows, identical to
// the reference's sequential incremental updates.

#include <cub/block/block_reduce.cuh>
#include <cub/block/block_scan.cuh>
#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "engine.h"

namespace beam {
namespace {

constexpr int kPrepThreads = 512;
constexpr int kLaneTopK = 32;        // per-lane candidate lists for top_k up to this
constexpr int kSmemEntries = 2048;   // bucket entries held in shared memory
constexpr int kSmemHeads = 4096;     // bucket hash heads in shared memory
// Groups of more than this many members take the sorted (GPU-wide) path
// even when their rows fit the shared-memory table: the pairs of members
// sharing a target grow with the square of the member count, too much work
// for one CTA.
constexpr int kSmemMaxGroup = 48;
constexpr int kScoreThreads = 256;
constexpr int kFewGroups = 256;  // blocks of at most this many groups take fewer, wider launches
// Selection by group size: at most kSelectSmallGroup members, a warp each;
// up to kSelectMidGroup, a small CTA each (sort + greedy pass); larger groups,
// matching rounds. The two are equal: the matching rounds measured faster
// than the small CTAs for groups of 9..32 members.
constexpr int kSelectMidGroup = 8;
constexpr int kSelectMidThreads = 128;
constexpr int kSelectMidKeys = 512;   // >= min(C(32,2), 16 * 32) candidates
constexpr int kRowsThreads = 256;
constexpr int kRowSmem = 2048;       // staged row entries in shared memory
constexpr int kWarpRow = 32;         // neighbour rows rewritten by one warp in registers
constexpr int kWarpRowMax = 256;     // neighbour rows rewritten by one warp through shared memory
constexpr int kKeyIdxBits = 10;      // a_idx, b_idx < kMaxGroup
constexpr long long kKeyGainMax = (1ll << (64 - 2 * kKeyIdxBits)) - 1;

__device__ __forceinline__ unsigned long long* ScratchAlloc(unsigned char* base, unsigned long long cap,
                                                           BlockCtl* ctl, unsigned long long bytes,
                                                           DevError* err) {
  bytes = (bytes + 255) & ~255ull;
  const unsigned long long at = atomicAdd(&ctl->scratch_top, bytes);
  if (at + bytes > cap) {
    RaiseError(err, kErrScratch, static_cast<int>(bytes >> 20), static_cast<int>(cap >> 20), 0);
    return nullptr;
  }
  return reinterpret_cast<unsigned long long*>(base + at);
}

// ------------------------------------------------------------ exact gain

struct GainWork {
  long long raw_a, raw_b, uni, ovl;
  long long bytes;  // algorithmic bytes of the gain computations
};

// Warp-cooperative ExactMergeGainPersistentImpl as a tiled merge of the two
// sorted rows: each step loads the next 32 entries of both rows (coalesced);
// with lim = the smaller of the two tiles' last neighbours, every entry <= lim
// is final in this step (an equal neighbour in the other row, if any, is in
// the other tile), and each lane finds its entry in the other tile by a
// 5-step shuffle search. Shared neighbours give two before-terms, one-sided
// neighbours one; e(a,b) is read from both rows and must agree. Every term
// is exact int64; the work is O(|R_a| + |R_b|).
__device__ void WarpExactGain(const QuotientView& Q, int a, int b, long long* gain_out, long long* before_out,
                              GainWork* work, DevError* err) {
  constexpr unsigned kFull = 0xffffffffu;
  constexpr Entry kPadEntry = static_cast<Entry>(0x7fffffffull) << 32;  // neighbour INT_MAX, count 0
  const int lane = threadIdx.x & 31;
  const long long sa = Q.size[a];
  const long long sb = Q.size[b];
  const long long sw = sa + sb;
  const Entry* ra = Q.ent + Q.off[a];
  const Entry* rb = Q.ent + Q.off[b];
  const int la = Q.len[a];
  const int lb = Q.len[b];
  long long before = 0, after = 0, eab_a = 0, eab_b = 0;
  int uni = 0, ovl = 0, bad = 0;
  int pa = 0, pb = 0;
  while (pa < la || pb < lb) {
    const bool va = pa + lane < la;
    const bool vb = pb + lane < lb;
    const Entry ea_e = va ? ra[pa + lane] : kPadEntry;
    const Entry eb_e = vb ? rb[pb + lane] : kPadEntry;
    const int xa = EntNb(ea_e);
    const int xb = EntNb(eb_e);
    const int last_a = __shfl_sync(kFull, xa, 31);
    const int last_b = __shfl_sync(kFull, xb, 31);
    const int lim = last_a < last_b ? last_a : last_b;
    // lower bound of xa in the b tile and of xb in the a tile
    int pos_b = 0, pos_a = 0;
#pragma unroll
    for (int step = 16; step > 0; step >>= 1) {
      const int probe_b = __shfl_sync(kFull, xb, pos_b + step - 1);
      const int probe_a = __shfl_sync(kFull, xa, pos_a + step - 1);
      if (probe_b < xa) pos_b += step;
      if (probe_a < xb) pos_a += step;
    }
    const Entry cand_b = __shfl_sync(kFull, eb_e, pos_b);
    const Entry cand_a = __shfl_sync(kFull, ea_e, pos_a);
    const bool fin_a = va && xa <= lim;
    const bool fin_b = vb && xb <= lim;
    if (fin_a) {
      const long long ca = EntCnt(ea_e);
      if (xa == b) {
        eab_a = ca;
      } else {
        const long long sx = Q.size[xa];
        if (EntNb(cand_b) == xa) {
          const long long cb = EntCnt(cand_b);
          before += BlockCost(sa, sx, ca, false, bad) + BlockCost(sb, sx, cb, false, bad);
          after += BlockCost(sw, sx, ca + cb, false, bad);
          ++ovl;
        } else {
          before += BlockCost(sa, sx, ca, false, bad);
          after += BlockCost(sw, sx, ca, false, bad);
        }
        ++uni;
      }
    }
    if (fin_b) {
      const long long cb = EntCnt(eb_e);
      if (xb == a) {
        eab_b = cb;
      } else if (EntNb(cand_a) != xb) {
        const long long sx = Q.size[xb];
        before += BlockCost(sb, sx, cb, false, bad);
        after += BlockCost(sw, sx, cb, false, bad);
        ++uni;
      }
    }
    pa += __popc(__ballot_sync(kFull, fin_a));
    pb += __popc(__ballot_sync(kFull, fin_b));
  }
  before = WarpSum(before);
  after = WarpSum(after);
  // e(a,b) is read by one lane per row (counts < 2^32)
  eab_a = __reduce_max_sync(kFull, static_cast<unsigned>(eab_a));
  eab_b = __reduce_max_sync(kFull, static_cast<unsigned>(eab_b));
  uni = static_cast<int>(__reduce_add_sync(kFull, static_cast<unsigned>(uni)));
  ovl = static_cast<int>(__reduce_add_sync(kFull, static_cast<unsigned>(ovl)));
  bad = __any_sync(kFull, bad);
  if (eab_a != eab_b) {
    if (lane == 0) RaiseError(err, kErrAsymmetric, a, b, 0);
  }
  const long long ia = Q.internal[a];
  const long long ib = Q.internal[b];
  before += BlockCost(sa, sa, ia, true, bad) + BlockCost(sb, sb, ib, true, bad) + BlockCost(sa, sb, eab_a, false, bad);
  after += BlockCost(sw, sw, ia + ib + eab_a, true, bad);
  if (bad && lane == 0) RaiseError(err, kErrBlockCost, a, b, 0);
  *gain_out = before - after;
  *before_out = before;
  if (work) {
    work->raw_a += la;
    work->raw_b += lb;
    work->uni += uni;
    work->ovl += ovl;
    // 8 B per row entry, 4 B per union-neighbour size gather
    work->bytes += 8ll * (la + lb) + 4ll * uni;
  }
}

// Per-row sums of the block-start state, for WarpExactGainShared:
//   before[r] = sum over the row of BlockCost(size_r, size_x, c_rx),
//   light[r]  = sum of c_rx over the row's light entries,
// where an entry is light when 1 + (size_r + 1) * size_x >= 2 c_rx: its
// after-merge term min(c, 1 + s * size_x - c) is c for every merged size
// s >= size_r + 1. The positions of the heavy entries are kept when there
// are at most kHeavyMax of them; a row with more is scored by the full merge.
constexpr int kHeavyMax = 4;

struct RowConsts {
  const long long* before;
  const long long* light;
  const int4* heavy;   // positions of the heavy entries, -1 unused
  const int* nheavy;   // heavy entries of the row
};

// Row sums are written by the prepare kernels, which read every member row
// of the block's groups with the target sizes anyway.
__device__ __forceinline__ bool HeavyEntry(long long size_r, long long size_x, long long c) {
  return 1 + (size_r + 1) * size_x < 2 * c;
}

// Warp-uniform call per 32-entry step of a row: records the positions of the
// step's heavy entries after the nh found so far.
__device__ __forceinline__ void RecordHeavy(int4* slot, int& nh, bool heavy, int k) {
  const int lane = threadIdx.x & 31;
  const unsigned hm = __ballot_sync(0xffffffffu, heavy);
  if (heavy) {
    const int rank = nh + __popc(hm & ((1u << lane) - 1u));
    if (rank < kHeavyMax) reinterpret_cast<int*>(slot)[rank] = k;
  }
  nh += __popc(hm);
}

// Skewed pairs (the long row at least kProbeMinLong entries and kProbeRatio
// times the short one) look the short row up in the long one.
constexpr int kProbeMinLong = 256;
constexpr int kProbeRatio = 8;

// The last index i of [lo, hi) with a[i] <= x, for a non-decreasing array
// with a[lo] <= x, found by the whole warp (warp-uniform arguments): each
// round probes 32 points of the remaining span, so the search takes about
// log32 of the span in dependent loads instead of log2.
__device__ __forceinline__ int WarpLastLE(const long long* __restrict__ a, int lo, int hi, long long x) {
  const int lane = threadIdx.x & 31;
  while (hi - lo > 1) {
    // lo < p, p <= hi - 1, non-decreasing over the lanes
    const int p = lo + 1 + static_cast<int>((static_cast<long long>(hi - lo - 1) * lane) >> 5);
    const int k = __popc(__ballot_sync(0xffffffffu, a[p] <= x));  // lanes 0..k-1 hold
    const int p_lo = __shfl_sync(0xffffffffu, p, k > 0 ? k - 1 : 0);
    const int p_hi = __shfl_sync(0xffffffffu, p, k < 32 ? k : 31);
    if (k > 0) lo = p_lo;
    if (k < 32) hi = p_hi;
  }
  return lo;
}

// First position of a sorted row whose neighbour is >= x.
__device__ __forceinline__ int RowLowerBound(const Entry* row, int len, int x) {
  int lo = 0, hi = len;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (EntNb(row[mid]) < x) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// ExactMergeGainPersistentImpl from the row sums: with s = size_a + size_b,
//   before = before[a] + before[b] - BC(s_b, s_a, e_ab) + BC_int(a) + BC_int(b)
//   after  = F_a(s) + F_b(s) - BC(s, s_b, e_ab) - BC(s, s_a, e_ab)
//            + sum over shared x of [BC(s, s_x, c_ax + c_bx) - BC(s, s_x, c_ax) - BC(s, s_x, c_bx)]
//            + BC_int(s, i_a + i_b + e_ab),
// F_r(s) = light[r] + the heavy entries' exact terms. Only the shared
// neighbours need sizes and cost terms; the tiled merge that finds them is
// the one of WarpExactGain. The same integers as the full merge, term by
// term regrouped.
// The scalars of one row that the row-sum gain reads: staged in shared memory
// by the scoring warp for a whole fetch of pairs at once (independent loads,
// one latency for all of them), then read by every lane as broadcasts.
struct RowMeta {
  long long off, internal, before, light;
  int4 heavy;
  int len, size, nheavy;
  int rep;  // the row's supernode
};

__device__ __forceinline__ void LoadRowMeta(const QuotientView& Q, const RowConsts& RC, int r, RowMeta* m) {
  RowMeta v;
  v.off = Q.off[r];
  v.internal = Q.internal[r];
  v.before = RC.before[r];
  v.light = RC.light[r];
  v.heavy = RC.heavy[r];
  v.len = Q.len[r];
  v.size = Q.size[r];
  v.nheavy = RC.nheavy[r];
  v.rep = r;
  *m = v;
}

__device__ void WarpExactGainShared(const QuotientView& Q, int a, int b, const RowMeta& A, const RowMeta& B,
                                    long long* gain_out, long long* before_out, GainWork* work, DevError* err) {
  constexpr unsigned kFull = 0xffffffffu;
  constexpr Entry kPadEntry = static_cast<Entry>(0x7fffffffull) << 32;
  const int ha = A.nheavy;
  const int hb = B.nheavy;
  if (ha > kHeavyMax || hb > kHeavyMax) {
    WarpExactGain(Q, a, b, gain_out, before_out, work, err);
    return;
  }
  const int lane = threadIdx.x & 31;
  const long long sa = A.size;
  const long long sb = B.size;
  const long long sw = sa + sb;
  const Entry* ra = Q.ent + A.off;
  const Entry* rb = Q.ent + B.off;
  const int la = A.len;
  const int lb = B.len;
  long long shared = 0, eab_a = 0, eab_b = 0;
  int ovl = 0, bad = 0;
  const bool a_long = la >= lb;
  const int ll = a_long ? la : lb;
  const int ls = a_long ? lb : la;
  const bool probe = ll >= kProbeMinLong && ll >= kProbeRatio * ls;
  if (probe) {
    // skewed pair: each entry of the short row is looked up in the long row
    // by binary search instead of streaming the long row
    const Entry* rl = a_long ? ra : rb;
    const Entry* rs = a_long ? rb : ra;
    const int long_rep = a_long ? a : b;
    const int short_rep = a_long ? b : a;
    long long e_long = 0, e_short = 0;  // e(a, b) as read from the long / the short row
    for (int k0 = 0; k0 < ls; k0 += 32) {
      const int k = k0 + lane;
      if (k < ls) {
        const Entry e = rs[k];
        const int x = EntNb(e);
        const long long cs = EntCnt(e);
        if (x == long_rep) {
          e_short = cs;
        } else {
          const int at = RowLowerBound(rl, ll, x);
          if (at < ll && EntNb(rl[at]) == x) {
            const long long cl = EntCnt(rl[at]);
            const long long ca = a_long ? cl : cs;
            const long long cb = a_long ? cs : cl;
            const long long sx = Q.size[x];
            shared += BlockCost(sw, sx, ca + cb, false, bad) - BlockCost(sw, sx, ca, false, bad) -
                      BlockCost(sw, sx, cb, false, bad);
            ++ovl;
          }
        }
      }
    }
    if (lane == 0) {
      const int at = RowLowerBound(rl, ll, short_rep);
      if (at < ll && EntNb(rl[at]) == short_rep) e_long = EntCnt(rl[at]);
    }
    eab_a = a_long ? e_long : e_short;
    eab_b = a_long ? e_short : e_long;
  }
  // otherwise the tiled merge of the two rows
  int pa = probe ? la : 0;
  int pb = probe ? lb : 0;
  while (pa < la || pb < lb) {
    const bool va = pa + lane < la;
    const bool vb = pb + lane < lb;
    const Entry ea_e = va ? ra[pa + lane] : kPadEntry;
    const Entry eb_e = vb ? rb[pb + lane] : kPadEntry;
    const int xa = EntNb(ea_e);
    const int xb = EntNb(eb_e);
    const int last_a = __shfl_sync(kFull, xa, 31);
    const int last_b = __shfl_sync(kFull, xb, 31);
    const int lim = last_a < last_b ? last_a : last_b;
    int pos_b = 0;
#pragma unroll
    for (int step = 16; step > 0; step >>= 1) {
      const int probe_b = __shfl_sync(kFull, xb, pos_b + step - 1);
      if (probe_b < xa) pos_b += step;
    }
    const Entry cand_b = __shfl_sync(kFull, eb_e, pos_b);
    const bool fin_a = va && xa <= lim;
    const bool fin_b = vb && xb <= lim;
    if (fin_a) {
      if (xa == b) {
        eab_a = EntCnt(ea_e);
      } else if (EntNb(cand_b) == xa) {
        const long long ca = EntCnt(ea_e);
        const long long cb = EntCnt(cand_b);
        const long long sx = Q.size[xa];
        shared += BlockCost(sw, sx, ca + cb, false, bad) - BlockCost(sw, sx, ca, false, bad) -
                  BlockCost(sw, sx, cb, false, bad);
        ++ovl;
      }
    }
    if (fin_b && xb == a) eab_b = EntCnt(eb_e);
    pa += __popc(__ballot_sync(kFull, fin_a));
    pb += __popc(__ballot_sync(kFull, fin_b));
  }
  // heavy entries: lanes 0..3 of row a, lanes 4..7 of row b
  long long heavy_a = 0, heavy_b = 0;
  if (lane < 2 * kHeavyMax) {
    const bool on_a = lane < kHeavyMax;
    const int h = on_a ? lane : lane - kHeavyMax;
    if (h < (on_a ? ha : hb)) {
      const int4 hp = on_a ? A.heavy : B.heavy;
      const int pos = h == 0 ? hp.x : h == 1 ? hp.y : h == 2 ? hp.z : hp.w;
      const Entry e = (on_a ? ra : rb)[pos];
      const long long term = BlockCost(sw, Q.size[EntNb(e)], EntCnt(e), false, bad);
      (on_a ? heavy_a : heavy_b) = term;
    }
  }
  // one 64-bit sum; e(a,b) is read by one lane per row (counts < 2^32)
  shared = WarpSum(shared + heavy_a + heavy_b);
  eab_a = __reduce_max_sync(kFull, static_cast<unsigned>(eab_a));
  eab_b = __reduce_max_sync(kFull, static_cast<unsigned>(eab_b));
  ovl = static_cast<int>(__reduce_add_sync(kFull, static_cast<unsigned>(ovl)));
  bad = __any_sync(kFull, bad);
  if (eab_a != eab_b) {
    if (lane == 0) RaiseError(err, kErrAsymmetric, a, b, 0);
  }
  const long long ia = A.internal;
  const long long ib = B.internal;
  const long long before = A.before + B.before - BlockCost(sb, sa, eab_b, false, bad) +
                           BlockCost(sa, sa, ia, true, bad) + BlockCost(sb, sb, ib, true, bad);
  const long long after = A.light + B.light - BlockCost(sw, sb, eab_a, false, bad) -
                          BlockCost(sw, sa, eab_b, false, bad) + shared +
                          BlockCost(sw, sw, ia + ib + eab_a, true, bad);
  if (bad && lane == 0) RaiseError(err, kErrBlockCost, a, b, 0);
  *gain_out = before - after;
  *before_out = before;
  if (work) {
    work->raw_a += la;
    work->raw_b += lb;
    work->uni += (la - (eab_a > 0 ? 1 : 0)) + (lb - (eab_b > 0 ? 1 : 0)) - ovl;
    work->ovl += ovl;
    // 8 B per row entry, 4 B per shared-neighbour size gather, 36 B of row sums
    work->bytes += 8ll * (la + lb) + 4ll * ovl + 36;
  }
}

// ------------------------------------------------------------ prepare

// Per-group arrays of the merge kernels (cand_off, cand_cnt, mat_off,
// sel_off, sel_cnt) are indexed by the group's position in the iteration's
// list of groups with at least two members ("real" groups); real[ri] is the
// Divide group id. A block covers the real groups [rg0, rg0 + nrg).
// A big group with more than kSmemMaxGroup members, or whose row entries
// (counted at Divide time, an upper bound for the rest of the iteration: rows
// of supernodes not yet merged only shrink) exceed the shared-memory bucket
// table, is deferred. PrepareKernel stages its row offsets and member scalars
// in block scratch; PrepareFillKernel writes one (group, target) key and one
// (member, count) value per row entry into the group's sort slots, a radix
// sort brings the entries of every (group, target) together, and
// PrepareAccumKernel pairs the entries of each run, a warp per 32 sorted
// slots. No group is bound to one SM.
// Scratch layout: eoff int32[g+1] | mq int32[g] | msz int32[g].
struct BigDesc {
  unsigned char* base;  // nullptr: not deferred
  int E;
  int pad;
};

struct DeferredView {
  int* eoff;
  int* mq;
  int* msz;
};

__host__ __device__ __forceinline__ unsigned long long DeferredBytes(int g) {
  return 4ull * (3ull * static_cast<unsigned long long>(g) + 1);
}

__device__ __forceinline__ DeferredView Deferred(unsigned char* base, int g) {
  DeferredView V;
  V.eoff = reinterpret_cast<int*>(base);
  V.mq = V.eoff + g + 1;
  V.msz = V.mq + g;
  return V;
}

constexpr unsigned long long kSlotPad = ~0ull;  // key of an unused sort slot

struct PrepareParams {
  QuotientView Q;
  const int* order;
  const int* gstart;
  const int* glen;
  const int* group_of;
  const int* idx_in_group;
  const int* real;
  const int* list;  // real-group positions handled by this launch
  int list0;
  int nlist;
  const long long* moff;  // member-count prefix over the big-group list
  BigDesc* desc;          // per big-group list entry
  float2* cand_feat;      // per candidate: proxy gain, proxy ratio (ranker features; nullptr: off)
  int2* cand_rep;         // per candidate slot: the pair's supernode ids (unused slots stay -1)
  const long long* soff;  // sort-slot prefix over the big-group list (0 slots: not deferred)
  long long slot0;        // soff of the launch's first entry
  int tbits;                 // bits of a target supernode id in a sort key
  unsigned long long* skey;  // unsorted keys / values of the launch's slots
  unsigned long long* sval;
  const unsigned long long* skey_sorted;
  const unsigned long long* sval_sorted;
  long long nslots;
  const long long* cand_off;
  int2* cand;
  int* cand_cnt;
  const long long* mat_off;
  unsigned char* mat;
  int mat_zeroed;  // the pair tables were cleared by one memset of the block
  // row sums for the scoring pass (rc_before == nullptr: not needed)
  long long* rc_before;
  long long* rc_light;
  int4* rc_heavy;
  int* rc_nheavy;
  unsigned char* scratch;
  unsigned long long scratch_cap;
  BlockCtl* ctl;
  int top_k;
  unsigned long long* stats;
  DevError* err;
};

// Per big group: proxy int64[g*g] | kept flag u8[g*g] | old cost int64[g];
// the flag table starts at FlagOffset and the old costs at OldCostOffset
// (rounded up to 8-byte alignment).
__host__ __device__ __forceinline__ long long FlagOffset(long long gg) { return 8 * gg; }
__host__ __device__ __forceinline__ long long OldCostOffset(long long gg) { return (9 * gg + 7) & ~7ll; }

// rb: the bits of the candidate's double ratio (the reference's rounded
// quotient, computed once per candidate); positive doubles order like their
// bit patterns, so candidates are compared on the integer pipes (this GPU's
// FP64 rate is a small fraction of its integer rate)
struct RankKey {
  unsigned long long rb;
  long long pg;
  int lo, hi, j;
};

// ranked_better (src/sweg.cpp:1926-1938): ratio desc, proxy gain desc,
// rep_lo asc, rep_hi asc.
__device__ __forceinline__ bool Better(const RankKey& x, const RankKey& y) {
  if (x.rb != y.rb) return x.rb > y.rb;
  if (x.pg != y.pg) return x.pg > y.pg;
  if (x.lo != y.lo) return x.lo < y.lo;
  return x.hi < y.hi;
}

// The reference's threshold test RN(gain / before) >= threshold (doubles, gain
// and before > 0) on the integer pipes, with threshold = m * 2^-e exactly
// (split on the host; e < 0: no split). Rounding is monotonic, so a quotient
// at or above the threshold passes, and one more than 2^-51 (relative) below
// it rounds below it and fails; only the band in between, and counts of 2^53
// or more (which the double conversion rounds), take the double division.
struct ThresholdBits {
  unsigned long long m;
  int e;
};

__host__ inline ThresholdBits SplitThreshold(double threshold) {
  ThresholdBits t{0, -1};
  if (threshold > 0.0 && std::isfinite(threshold)) {
    int ex = 0;
    const double f = std::frexp(threshold, &ex);  // threshold = f * 2^ex, f in [0.5, 1)
    t.m = static_cast<unsigned long long>(std::ldexp(f, 53));
    t.e = 53 - ex;
  }
  return t;
}

__device__ __forceinline__ bool RatioAtLeast(long long gain, long long before, double threshold, ThresholdBits t) {
  if (t.e >= 0 && t.e <= 63 && gain < (1ll << 53) && before < (1ll << 53)) {
    const unsigned __int128 l = static_cast<unsigned __int128>(static_cast<unsigned long long>(gain)) << t.e;
    const unsigned __int128 r = static_cast<unsigned __int128>(t.m) * static_cast<unsigned long long>(before);
    if (l >= r) return true;
    if (l + (r >> 51) < r) return false;
  }
  return static_cast<double>(gain) / static_cast<double>(before) >= threshold;
}

__device__ __forceinline__ unsigned BucketHash(int t, unsigned mask) {
  return (static_cast<unsigned>(t) * 0x9E3779B1u) >> 7 & mask;
}

struct PrepSmem {
  int q[kMaxGroup];
  int sz[kMaxGroup];
  int len[kMaxGroup];
  long long off[kMaxGroup];
  long long old[kMaxGroup];
  int eoff[kMaxGroup + 1];
  int heads[kSmemHeads];
  int et[kSmemEntries];
  int ei[kSmemEntries];
  unsigned ee[kSmemEntries];
  int enx[kSmemEntries];
  unsigned long long examined;
  int total;
};

__global__ void __launch_bounds__(kPrepThreads) PrepareKernel(PrepareParams P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  PrepSmem& S = *reinterpret_cast<PrepSmem*>(smem_raw);
  using BlockScan = cub::BlockScan<int, kPrepThreads>;
  __shared__ typename BlockScan::TempStorage scan_tmp;
  __shared__ int carry;
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const int nwarps = kPrepThreads / 32;
  const int ri = P.list[P.list0 + blockIdx.x];
  const int gid = P.real[ri];
  const int g = P.glen[gid];
  BigDesc* desc = P.desc + P.list0 + blockIdx.x;
  if (tid == 0) {
    desc->base = nullptr;
    desc->E = 0;
  }
  // sort slots of a deferred group start as padding, so that every exit
  // below leaves them well-defined for the sort and the accumulate pass
  const long long slot_beg = P.soff[P.list0 + blockIdx.x];
  const long long slots = P.soff[P.list0 + blockIdx.x + 1] - slot_beg;
  {
    unsigned long long* key = P.skey + (slot_beg - P.slot0);
    for (long long k = tid; k < slots; k += kPrepThreads) key[k] = kSlotPad;
  }
  if (g < 2) {
    if (tid == 0) P.cand_cnt[ri] = 0;
    return;
  }
  if (g > kMaxGroup) {
    if (tid == 0) {
      RaiseError(P.err, kErrGroupTooLarge, gid, g, 0);
      P.cand_cnt[ri] = 0;
    }
    return;
  }
  const QuotientView& Q = P.Q;
  const int start = P.gstart[gid];
  for (int i = tid; i < g; i += kPrepThreads) {
    const int rep = P.order[start + i];
    S.q[i] = rep;
    S.sz[i] = Q.size[rep];
    S.len[i] = Q.len[rep];
    S.off[i] = Q.off[rep];
  }
  if (tid == 0) {
    S.examined = 0;
    carry = 0;
  }
  __syncthreads();
  // exclusive scan of row lengths -> entry offsets
  for (int base = 0; base < g; base += kPrepThreads) {
    const int i = base + tid;
    const int v = i < g ? S.len[i] : 0;
    int ex = 0, agg = 0;
    BlockScan(scan_tmp).ExclusiveSum(v, ex, agg);
    if (i < g) S.eoff[i] = carry + ex;
    __syncthreads();
    if (tid == 0) carry += agg;
    __syncthreads();
  }
  const int E = carry;
  if (tid == 0) S.eoff[g] = E;
  const long long gg = static_cast<long long>(g) * g;
  unsigned char* mat = P.mat + P.mat_off[ri];
  long long* pmat = reinterpret_cast<long long*>(mat);
  unsigned char* fmat = mat + FlagOffset(gg);
  if (slots > 0) {
    // deferred group: row offsets and member scalars in block scratch, pair
    // tables zeroed, unused sort slots padded; fill / sort / accumulate follow
    if (E > slots) {
      if (tid == 0) {
        RaiseError(P.err, kErrSlots, gid, E, static_cast<int>(slots));
        P.cand_cnt[ri] = 0;
      }
      return;
    }
    __shared__ unsigned char* dbase;
    if (tid == 0) {
      dbase = reinterpret_cast<unsigned char*>(ScratchAlloc(P.scratch, P.scratch_cap, P.ctl, DeferredBytes(g), P.err));
    }
    __syncthreads();
    if (dbase == nullptr) {
      if (tid == 0) P.cand_cnt[ri] = 0;
      return;
    }
    const DeferredView V = Deferred(dbase, g);
    long long* old_out = reinterpret_cast<long long*>(mat + OldCostOffset(gg));
    for (int i = tid; i < g; i += kPrepThreads) {
      V.eoff[i] = S.eoff[i];
      V.mq[i] = S.q[i];
      V.msz[i] = S.sz[i];
      // the fill pass adds the row terms of the approximate old cost
      const long long si = S.sz[i];
      const long long internal = Q.internal[S.q[i]];
      old_out[i] = internal > 0 ? EncodeCostForPair(S.q[i], si, S.q[i], si, 2 * internal) : 0;
      if (P.rc_before) {
        // the fill pass adds the row sums
        P.rc_before[S.q[i]] = 0;
        P.rc_light[S.q[i]] = 0;
        P.rc_nheavy[S.q[i]] = 0;
        P.rc_heavy[S.q[i]] = make_int4(-1, -1, -1, -1);
      }
    }
    if (tid == 0) V.eoff[g] = E;
    if (!P.mat_zeroed) {
      for (long long k = tid; k < gg; k += kPrepThreads) {
        pmat[k] = 0;
        fmat[k] = 0;
      }
    }
    if (tid == 0) {
      desc->base = dbase;
      desc->E = E;
      atomicAdd(&P.stats[kStGroupCount], 1ull);
      atomicMax(&P.stats[kStGroupMaxSize], static_cast<unsigned long long>(g));
      atomicAdd(&P.stats[kStRawPairCount], static_cast<unsigned long long>(g) * (g - 1) / 2);
      atomicAdd(&P.stats[kStPrepareBytes], 12ull * static_cast<unsigned long long>(E));
    }
    return;
  }
  if (E > kSmemEntries) {
    if (tid == 0) {
      RaiseError(P.err, kErrSlots, gid, E, 0);
      P.cand_cnt[ri] = 0;
    }
    return;
  }
  // bucket table in shared memory
  int* heads = S.heads;
  int* et = S.et;
  int* ei = S.ei;
  unsigned* ee = S.ee;
  int* enx = S.enx;
  const unsigned hmask = kSmemHeads - 1;
  for (unsigned h = tid; h <= hmask; h += kPrepThreads) heads[h] = -1;
  // per-group tables: proxy int64[g*g] | kept flag u8[g*g] | old cost int64[g]
  if (!P.mat_zeroed) {
    for (long long k = tid; k < gg; k += kPrepThreads) {
      pmat[k] = 0;
      fmat[k] = 0;
    }
  }
  __syncthreads();
  // entries, approximate old costs and direct in-group edges
  for (int i = warp; i < g; i += nwarps) {
    const int rep = S.q[i];
    const long long si = S.sz[i];
    const Entry* row = Q.ent + S.off[i];
    const int len = S.len[i];
    const int eo = S.eoff[i];
    long long old = 0, light = 0;
    int nh = 0;
    if (P.rc_before && lane == 0) P.rc_heavy[rep] = make_int4(-1, -1, -1, -1);
    __syncwarp();
    for (int k0 = 0; k0 < len; k0 += 32) {
      const int k = k0 + lane;
      bool heavy = false;
      if (k < len) {
        const Entry e = row[k];
        const int t = EntNb(e);
        const long long c = EntCnt(e);
        const long long st = Q.size[t];
        old += EncodeCostForPair(rep, si, t, st, c);
        heavy = HeavyEntry(si, st, c);
        if (!heavy) light += c;
        et[eo + k] = t;
        ei[eo + k] = i;
        ee[eo + k] = static_cast<unsigned>(c);
        enx[eo + k] = atomicExch(&heads[BucketHash(t, hmask)], eo + k);
        // direct in-group edge: row i holds j and row j holds i with the same
        // count, so each half of the table gets it once
        if (P.group_of[t] == gid) pmat[static_cast<long long>(i) * g + P.idx_in_group[t]] = c;
      }
      if (P.rc_before) RecordHeavy(P.rc_heavy + rep, nh, heavy, k);
    }
    old = WarpSum(old);
    if (P.rc_before) light = WarpSum(light);
    if (lane == 0) {
      if (P.rc_before) {
        P.rc_before[rep] = old;
        P.rc_light[rep] = light;
        P.rc_nheavy[rep] = nh;
      }
      const long long internal = Q.internal[rep];
      if (internal > 0) old += EncodeCostForPair(rep, si, rep, si, 2 * internal);
      S.old[i] = old;
    }
  }
  __syncthreads();
  // every two members sharing a target: proxy += max(0, old - new)
  unsigned long long examined = 0;
  for (int idx = tid; idx < E; idx += kPrepThreads) {
    const int t = et[idx];
    const int i = ei[idx];
    const long long c = ee[idx];
    long long st = -1;
    for (int k = enx[idx]; k != -1; k = enx[k]) {
      if (et[k] != t) continue;
      if (st < 0) st = Q.size[t];
      const int j = ei[k];
      const int a = i < j ? i : j;
      const int b = i < j ? j : i;
      const long long ea = a == i ? c : static_cast<long long>(ee[k]);
      const long long eb = a == i ? static_cast<long long>(ee[k]) : c;
      const long long sa = S.sz[a];
      const long long sb = S.sz[b];
      const int qa = S.q[a];
      const int qb = S.q[b];
      ++examined;
      const long long oldc = EncodeCostForPair(qa, sa, t, st, ea) + EncodeCostForPair(qb, sb, t, st, eb);
      const long long newc = EncodeCostForPair(qa, sa + sb, t, st, ea + eb);
      const long long delta = oldc - newc;
      if (delta > 0) {
        // both halves, so every member's partners are one contiguous row
        atomicAdd(reinterpret_cast<unsigned long long*>(&pmat[static_cast<long long>(a) * g + b]),
                  static_cast<unsigned long long>(delta));
        atomicAdd(reinterpret_cast<unsigned long long*>(&pmat[static_cast<long long>(b) * g + a]),
                  static_cast<unsigned long long>(delta));
      }
    }
  }
  examined = WarpSum(static_cast<long long>(examined));
  if (lane == 0 && examined) atomicAdd(&S.examined, examined);
  __syncthreads();
  // old costs for the member pass, counters of the group
  long long* old_out = reinterpret_cast<long long*>(mat + OldCostOffset(gg));
  for (int i = tid; i < g; i += kPrepThreads) old_out[i] = S.old[i];
  if (tid == 0) {
    atomicAdd(&P.stats[kStGroupCount], 1ull);
    atomicMax(&P.stats[kStGroupMaxSize], static_cast<unsigned long long>(g));
    atomicAdd(&P.stats[kStRawPairCount], static_cast<unsigned long long>(g) * (g - 1) / 2);
    atomicAdd(&P.stats[kStProxyExamined], S.examined);
    // algorithmic bytes: member rows (8 B/entry) + target size gathers (4 B/entry)
    atomicAdd(&P.stats[kStPrepareBytes], 12ull * static_cast<unsigned long long>(E));
  }
}

// Fill pass of the deferred groups: one thread per sort slot of the launch
// (the groups' slot ranges, soff, laid end to end), CTAs striding over windows
// of kFillWindow slots, so the grid follows the total row entries and a hub
// member's long row is spread over many warps. A window's first group is
// found by a binary search of soff; each lane walks forward from it, and
// finds its member by a binary search of the group's row offsets (entries of
// one member are contiguous). Per entry: its sort key (launch-local group
// index, target) and value (member, count), the entry's approximate-old-cost
// term (summed per member run by a segmented warp scan, one atomic per run),
// and direct in-group edges, which go to both halves of the pair table (row i
// holds j and row j holds i with the same count), so no mirror pass is
// needed. Slots past a group's entries keep the padding key.
constexpr int kFillThreads = 256;
constexpr int kFillWindow = 2048;
constexpr int kAccumThreads = 256;

__global__ void __launch_bounds__(kFillThreads) PrepareFillKernel(PrepareParams P) {
  __shared__ int first_group;
  const int lane = threadIdx.x & 31;
  const QuotientView& Q = P.Q;
  const long long windows = (P.nslots + kFillWindow - 1) / kFillWindow;
  for (long long w = blockIdx.x; w < windows; w += gridDim.x) {
    const long long w0 = w * kFillWindow;
    if (threadIdx.x == 0) {
      int lo = 0, hi = P.nlist;  // last group whose slot range starts at or before w0
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (P.soff[P.list0 + mid] - P.slot0 <= w0) lo = mid; else hi = mid;
      }
      first_group = lo;
    }
    __syncthreads();
    int k = first_group;
    int i = -1;  // member of the previous slot (same group), -1 none
    for (int off = threadIdx.x; off < kFillWindow; off += kFillThreads) {
      const long long s = w0 + off;
      long long run = -1;  // (group, member) of this lane's entry, -1 none
      long long cost = 0, light = 0;
      int rep = -1;
      if (s < P.nslots) {
        const int k0 = k;
        while (k + 1 < P.nlist && P.soff[P.list0 + k + 1] - P.slot0 <= s) ++k;
        if (k != k0) i = -1;
        const BigDesc d = P.desc[P.list0 + k];
        const long long idx = s - (P.soff[P.list0 + k] - P.slot0);
        if (d.base != nullptr && idx < d.E) {
          const int ri = P.list[P.list0 + k];
          const int gid = P.real[ri];
          const int g = P.glen[gid];
          const DeferredView V = Deferred(d.base, g);
          if (i < 0 || idx >= V.eoff[i + 1] || idx < V.eoff[i]) {
            int lo = 0, hi = g;  // last member with eoff <= idx
            while (hi - lo > 1) {
              const int mid = (lo + hi) >> 1;
              if (V.eoff[mid] <= idx) lo = mid; else hi = mid;
            }
            i = lo;
          }
          rep = V.mq[i];
          const int e0 = V.eoff[i];
          const Entry e = Q.ent[Q.off[rep] + (idx - e0)];
          const int t = EntNb(e);
          const long long c = EntCnt(e);
          const long long st = Q.size[t];
          cost = EncodeCostForPair(rep, V.msz[i], t, st, c);
          if (P.rc_before) {
            if (HeavyEntry(V.msz[i], st, c)) {
              const int rank = atomicAdd(&P.rc_nheavy[rep], 1);
              if (rank < kHeavyMax) reinterpret_cast<int*>(&P.rc_heavy[rep])[rank] = static_cast<int>(idx - e0);
            } else {
              light = c;
            }
          }
          const long long slot = P.soff[P.list0 + k] - P.slot0 + idx;
          P.skey[slot] = (static_cast<unsigned long long>(k) << P.tbits) | static_cast<unsigned>(t);
          P.sval[slot] = static_cast<unsigned long long>(i) << 32 | static_cast<unsigned long long>(c);
          if (P.group_of[t] == gid) {
            long long* pmat = reinterpret_cast<long long*>(P.mat + P.mat_off[ri]);
            pmat[static_cast<long long>(i) * g + P.idx_in_group[t]] = c;
          }
          run = (static_cast<long long>(k) << 11) | i;
        }
      }
      // segmented inclusive scan over runs of equal (group, member)
      for (int o = 1; o < 32; o <<= 1) {
        const long long vc = __shfl_up_sync(0xffffffffu, cost, o);
        const long long vl = __shfl_up_sync(0xffffffffu, light, o);
        const long long vr = __shfl_up_sync(0xffffffffu, run, o);
        if (lane >= o && vr == run) {
          cost += vc;
          light += vl;
        }
      }
      const long long next_run = __shfl_down_sync(0xffffffffu, run, 1);
      if (run >= 0 && (lane == 31 || next_run != run)) {
        const int ri = P.list[P.list0 + k];
        const int g = P.glen[P.real[ri]];
        unsigned long long* old_out =
            reinterpret_cast<unsigned long long*>(P.mat + P.mat_off[ri] + OldCostOffset(static_cast<long long>(g) * g));
        if (cost != 0) atomicAdd(&old_out[i], static_cast<unsigned long long>(cost));
        if (P.rc_before) {
          if (cost != 0) atomicAdd(reinterpret_cast<unsigned long long*>(&P.rc_before[rep]), static_cast<unsigned long long>(cost));
          if (light != 0) atomicAdd(reinterpret_cast<unsigned long long*>(&P.rc_light[rep]), static_cast<unsigned long long>(light));
        }
      }
    }
    __syncthreads();  // first_group is rewritten by the next window
  }
}

// Accumulate pass of the deferred groups over the sorted slots, a warp per
// 32 consecutive slots. The entries of one (group, target) are a contiguous
// run; each lane pairs its entry with the earlier entries of its run: those
// in its own chunk by shuffles, and, for the run that reaches back past the
// chunk's start, those of the earlier chunks, 32 at a time. Every member pair
// sharing a target is visited once and adds proxy += max(0, old - new) to
// both halves of the pair table.
struct RunEntry {
  unsigned long long key;
  long long c, s;  // edge count to the target, member size
  int i, q;        // member index, member supernode
};

__device__ __forceinline__ RunEntry LoadRunEntry(const PrepareParams& P, long long p, const DeferredView& V) {
  RunEntry r;
  const unsigned long long v = P.sval_sorted[p];
  r.i = static_cast<int>(v >> 32);
  r.c = static_cast<long long>(v & 0xffffffffu);
  r.s = V.msz[r.i];
  r.q = V.mq[r.i];
  return r;
}

__device__ __forceinline__ RunEntry ShflRunEntry(const RunEntry& r, int src) {
  RunEntry o;
  o.key = __shfl_sync(0xffffffffu, r.key, src);
  o.c = __shfl_sync(0xffffffffu, r.c, src);
  o.s = __shfl_sync(0xffffffffu, r.s, src);
  o.i = __shfl_sync(0xffffffffu, r.i, src);
  o.q = __shfl_sync(0xffffffffu, r.q, src);
  return o;
}

__device__ __forceinline__ void AccumPair(const RunEntry& a, const RunEntry& b, int t, long long st, int g,
                                          long long* pmat, unsigned long long& examined) {
  ++examined;
  const long long oldc = EncodeCostForPair(a.q, a.s, t, st, a.c) + EncodeCostForPair(b.q, b.s, t, st, b.c);
  const long long newc = EncodeCostForPair(a.q, a.s + b.s, t, st, a.c + b.c);
  const long long delta = oldc - newc;
  if (delta > 0) {
    atomicAdd(reinterpret_cast<unsigned long long*>(&pmat[static_cast<long long>(a.i) * g + b.i]),
              static_cast<unsigned long long>(delta));
    atomicAdd(reinterpret_cast<unsigned long long*>(&pmat[static_cast<long long>(b.i) * g + a.i]),
              static_cast<unsigned long long>(delta));
  }
}

// kAccumSplit warps share a chunk: warp y pairs the chunk with the earlier
// chunks y + 1, y + 1 + kAccumSplit, ... of its run (warp 0 also within the
// chunk), so a chunk deep in a long run is not one warp's long loop.
constexpr int kAccumSplit = 4;
// Work items are fetched from a queue, kAccumFetch at a time: a run over a
// hub target makes some chunks far longer than others, so a static stride
// leaves most warps idle behind a few. A fetch unit is one y of kAccumFetch
// chunks spread over the whole slot range (chunk g, g + G, g + 2G, ... with G
// fetch groups), so the consecutive chunks of one long run land on different
// warps, and so do the split warps of one chunk.
constexpr int kAccumFetch = 8;

__global__ void __launch_bounds__(kAccumThreads, 6) PrepareAccumKernel(PrepareParams P) {
  const int lane = threadIdx.x & 31;
  unsigned long long examined = 0;
  const long long nchunks = (P.nslots + 31) >> 5;
  const long long ngroups8 = (nchunks + kAccumFetch - 1) / kAccumFetch;
  const long long nfetch = ngroups8 * kAccumSplit;
  long long fetched = -1, left = 0;
  for (;;) {
    if (left == 0) {
      long long f = 0;
      if (lane == 0) f = static_cast<long long>(atomicAdd(&P.ctl->work_next[0], 1ull));
      fetched = __shfl_sync(0xffffffffu, f, 0);
      if (fetched >= nfetch) break;
      left = kAccumFetch;
    }
    --left;
    // fetch unit u = (chunk group g, y): chunks g + k * ngroups8, k < kAccumFetch
    const int y = static_cast<int>(fetched % kAccumSplit);
    const long long ch = (fetched / kAccumSplit) + (kAccumFetch - 1 - left) * ngroups8;
    if (ch >= nchunks) continue;
    const long long p0 = ch << 5;
    if (y > 0) {
      // nothing unless the chunk's first run reaches back at least y + 1 chunks
      if (p0 < 32ll * (y + 1)) continue;
      const unsigned long long f = P.skey_sorted[p0];
      if (f == kSlotPad || P.skey_sorted[p0 - 32ll * y - 1] != f) continue;
    }
    const long long p = p0 + lane;
    RunEntry me;
    me.key = p < P.nslots ? P.skey_sorted[p] : kSlotPad;
    me.c = me.s = 0;
    me.i = me.q = 0;
    const bool valid = me.key != kSlotPad && static_cast<int>(me.key >> P.tbits) < P.nlist;
    int t = 0, g = 0;
    long long st = 0;
    long long* pmat = nullptr;
    if (valid) {
      const int bl = static_cast<int>(me.key >> P.tbits);
      t = static_cast<int>(me.key & ((1ull << P.tbits) - 1ull));
      const int ri = P.list[P.list0 + bl];
      g = P.glen[P.real[ri]];
      pmat = reinterpret_cast<long long*>(P.mat + P.mat_off[ri]);
      const RunEntry r = LoadRunEntry(P, p, Deferred(P.desc[P.list0 + bl].base, g));
      me.c = r.c;
      me.s = r.s;
      me.i = r.i;
      me.q = r.q;
      st = P.Q.size[t];
    }
    // pairs inside the chunk: each lane visits the earlier lanes holding its
    // key, one per round (a chunk whose targets are all distinct, the common
    // case, takes no round)
    if (y == 0) {
      unsigned earlier = __match_any_sync(0xffffffffu, me.key) & ((1u << lane) - 1u);
      if (!valid) earlier = 0u;
      const int rounds = static_cast<int>(__reduce_max_sync(0xffffffffu, static_cast<unsigned>(__popc(earlier))));
      for (int r = 0; r < rounds; ++r) {
        const int src = earlier != 0u ? __ffs(earlier) - 1 : lane;
        const RunEntry o = ShflRunEntry(me, src);
        if (earlier != 0u) {
          AccumPair(me, o, t, st, g, pmat, examined);
          earlier &= earlier - 1u;
        }
      }
    }
    // the run holding the chunk's first slot may start in earlier chunks
    const unsigned long long first = __shfl_sync(0xffffffffu, me.key, 0);
    if (first == kSlotPad || p0 == 0 || P.skey_sorted[p0 - 1] != first) continue;
    const int fbl = static_cast<int>(first >> P.tbits);
    if (fbl >= P.nlist) continue;
    const int fg = P.glen[P.real[P.list[P.list0 + fbl]]];
    const DeferredView FV = Deferred(P.desc[P.list0 + fbl].base, fg);
    const bool mine = valid && me.key == first;
    for (long long c0 = p0 - 32ll * (y + 1);; c0 -= 32ll * kAccumSplit) {
      // c0 >= 0; the chunk holds run entries iff its last slot is in the run
      if (P.skey_sorted[c0 + 31] != first) break;
      RunEntry o;
      o.key = P.skey_sorted[c0 + lane];
      o.c = o.s = 0;
      o.i = o.q = 0;
      if (o.key == first) o = [&] { RunEntry r = LoadRunEntry(P, c0 + lane, FV); r.key = first; return r; }();
      for (int src = 0; src < 32; ++src) {
        const RunEntry b = ShflRunEntry(o, src);
        if (mine && b.key == first) AccumPair(me, b, t, st, g, pmat, examined);
      }
      // the run continues below this chunk iff its first slot is in the run
      if (c0 < 32ll * kAccumSplit || __shfl_sync(0xffffffffu, o.key, 0) != first) break;
    }
  }
  examined = static_cast<unsigned long long>(WarpSum(static_cast<long long>(examined)));
  if (lane == 0 && examined) atomicAdd(&P.stats[kStProxyExamined], examined);
}

// Top-k partners of member i of a big group whose partners fill NT slots of
// 32 (the fp32 prescreen branch of PrepareMembersKernel).
template <int NT>
__device__ __forceinline__ void MembersTopK(int lane, int g, int i, int qi, int top_k, int cnt, const long long* prow,
                                            const long long* old, long long old_i, const int* q, int* cj,
                                            unsigned char* fmat) {
  auto ratio_of = [&](int j, long long pg) {
    long long denom = old_i + old[j];
    if (denom < 1) denom = 1;
    return static_cast<unsigned long long>(
        __double_as_longlong(static_cast<double>(pg) / static_cast<double>(denom)));
  };
  // fp32 prescreen: the exact (double) ratio is only computed for the
  // candidates that can be in the member's top_k. The fp32 ratio of a
  // candidate is within relative 3 * 2^-24 of its double ratio, so every
  // candidate of the exact top_k has an fp32 ratio >= tau * (1 - 2^-20),
  // where tau is the top_k-th largest fp32 ratio (found by bisection on the
  // float bit patterns, which order like the positive values).
  float rf[NT];
#pragma unroll
  for (int t = 0; t < NT; ++t) {
    const int j = lane + 32 * t;
    float v = 0.0f;  // not a candidate
    if (j < g && j != i) {
      const long long pg = prow[j];
      if (pg > 0) {
        long long denom = old_i + old[j];
        if (denom < 1) denom = 1;
        v = __fdiv_rn(static_cast<float>(pg), static_cast<float>(denom));
      }
    }
    rf[t] = v;
  }
  float cut = 0.0f;
  if (cnt > top_k + 16) {
    // count(bits >= lo) >= top_k > count(bits >= hi), starting from the
    // smallest and one past the largest positive ratio (the cnt candidates)
    unsigned lo = 0x7f800000u, hi = 0;
#pragma unroll
    for (int t = 0; t < NT; ++t) {
      const unsigned b = __float_as_uint(rf[t]);
      if (rf[t] > 0.0f) {
        lo = b < lo ? b : lo;
        hi = b > hi ? b : hi;
      }
    }
    lo = __reduce_min_sync(0xffffffffu, lo);
    hi = __reduce_max_sync(0xffffffffu, hi) + 1u;
    while (hi - lo > 1) {
      const unsigned mid = lo + ((hi - lo) >> 1);
      int c = 0;
#pragma unroll
      for (int t = 0; t < NT; ++t) c += __float_as_uint(rf[t]) >= mid ? 1 : 0;
      c = WarpSumInt(c);
      if (c >= top_k) lo = mid; else hi = mid;
    }
    cut = __uint_as_float(lo) * (1.0f - 9.5367431640625e-7f);
  }
  int npass = 0;
#pragma unroll
  for (int t = 0; t < NT; ++t) npass += (rf[t] > 0.0f && rf[t] >= cut) ? 1 : 0;
  npass = WarpSumInt(npass);
  if (npass <= 32) {
    // one surviving candidate per lane; its rank is the number of
    // candidates better than it under the strict order, and the top_k
    // ranks are kept
    int base = 0;
#pragma unroll
    for (int t = 0; t < NT; ++t) {
      const bool pass = rf[t] > 0.0f && rf[t] >= cut;
      const unsigned ball = __ballot_sync(0xffffffffu, pass);
      if (pass) cj[base + __popc(ball & ((1u << lane) - 1u))] = lane + 32 * t;
      base += __popc(ball);
    }
    __syncwarp();
    const bool have = lane < npass;
    RankKey mine;
    mine.rb = 0;
    mine.pg = 0;
    mine.lo = 0;
    mine.hi = 0;
    mine.j = -1;
    if (have) {
      const int j = cj[lane];
      const long long pg = prow[j];
      const int qj = q[j];
      mine.j = j;
      mine.rb = ratio_of(j, pg);
      mine.pg = pg;
      mine.lo = qi < qj ? qi : qj;
      mine.hi = qi < qj ? qj : qi;
    }
    int rank = 0;
    for (int o = 0; o < npass; ++o) {
      RankKey other;
      other.rb = __shfl_sync(0xffffffffu, mine.rb, o);
      other.pg = __shfl_sync(0xffffffffu, mine.pg, o);
      other.lo = __shfl_sync(0xffffffffu, mine.lo, o);
      other.hi = __shfl_sync(0xffffffffu, mine.hi, o);
      if (have && o != lane && Better(other, mine)) ++rank;
    }
    if (have && rank < top_k) {
      const int a = i < mine.j ? i : mine.j;
      const int b = i < mine.j ? mine.j : i;
      fmat[static_cast<long long>(a) * g + b] = 1;
    }
  } else {
    // each lane keeps its best top_k candidates sorted, then the warp merges
    // the 32 lists head by head (candidates are distinct, so no key ties)
    RankKey lst[kLaneTopK];
    int nl = 0;
  #pragma unroll
    for (int t = 0; t < NT; ++t) {
      const int j = lane + 32 * t;
      if (rf[t] <= 0.0f || rf[t] < cut) continue;
      const long long pg = prow[j];
      RankKey k;
      k.j = j;
      k.rb = ratio_of(j, pg);
      k.pg = pg;
      const int qj = q[j];
      k.lo = qi < qj ? qi : qj;
      k.hi = qi < qj ? qj : qi;
      if (nl == top_k && !Better(k, lst[nl - 1])) continue;
      int pos = nl < top_k ? nl : top_k - 1;
      while (pos > 0 && Better(k, lst[pos - 1])) {
        lst[pos] = lst[pos - 1];
        --pos;
      }
      lst[pos] = k;
      if (nl < top_k) ++nl;
    }
    int head = 0;
    for (int r = 0; r < top_k; ++r) {
      RankKey best;
      bool have = head < nl;
      if (have) best = lst[head];
      int src = lane;
      for (int o = 16; o > 0; o >>= 1) {
        RankKey other;
        other.rb = __shfl_xor_sync(0xffffffffu, best.rb, o);
        other.pg = __shfl_xor_sync(0xffffffffu, best.pg, o);
        other.lo = __shfl_xor_sync(0xffffffffu, best.lo, o);
        other.hi = __shfl_xor_sync(0xffffffffu, best.hi, o);
        other.j = __shfl_xor_sync(0xffffffffu, best.j, o);
        const int osrc = __shfl_xor_sync(0xffffffffu, src, o);
        const int ohave = __shfl_xor_sync(0xffffffffu, have ? 1 : 0, o);
        if (ohave && (!have || Better(other, best))) {
          best = other;
          have = true;
          src = osrc;
        }
      }
      if (!have) break;
      if (src == lane) ++head;
      if (lane == 0) {
        const int a = i < best.j ? i : best.j;
        const int b = i < best.j ? best.j : i;
        fmat[static_cast<long long>(a) * g + b] = 1;
      }
    }
  }
}

// Member pass of the big groups: one warp per member of every group in the
// launch's big-group list (moff = prefix of the member counts), so a large
// group's members are ranked by the whole GPU instead of one CTA.
__global__ void __launch_bounds__(256) PrepareMembersKernel(PrepareParams P) {
  __shared__ int cand_j[8][32];  // per warp: the candidates that survive the prescreen
  const int lane = threadIdx.x & 31;
  const long long wg = (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const long long total = P.moff[P.list0 + P.nlist] - P.moff[P.list0];
  if (wg >= total) return;
  const long long target = P.moff[P.list0] + wg;
  const int lo = WarpLastLE(P.moff, P.list0, P.list0 + P.nlist, target);  // last entry with moff <= target
  const int ri = P.list[lo];
  const int i = static_cast<int>(target - P.moff[lo]);
  const int gid = P.real[ri];
  const int g = P.glen[gid];
  const int* q = P.order + P.gstart[gid];
  const long long gg = static_cast<long long>(g) * g;
  unsigned char* mat = P.mat + P.mat_off[ri];
  const long long* pmat = reinterpret_cast<const long long*>(mat);
  unsigned char* fmat = mat + FlagOffset(gg);
  const long long* old = reinterpret_cast<const long long*>(mat + OldCostOffset(gg));
  // per member: candidates with positive proxy, ratio, top-k (the ratio is
  // recomputed where it is needed instead of being stored)
  int top_k = P.top_k < g - 1 ? P.top_k : g - 1;
  if (top_k < 1) top_k = 1;
  const long long* prow = pmat + static_cast<long long>(i) * g;
  const long long old_i = old[i];
  auto ratio_of = [&](int j, long long pg) {
    long long denom = old_i + old[j];
    if (denom < 1) denom = 1;
    return static_cast<unsigned long long>(
        __double_as_longlong(static_cast<double>(pg) / static_cast<double>(denom)));
  };
  int cnt = 0;
  for (int base = 0; base < g; base += 32) {
    const int j = base + lane;
    const bool pred = j < g && j != i && prow[j] > 0;
    cnt += __popc(__ballot_sync(0xffffffffu, pred));
  }
  const int qi = q[i];
  if (cnt <= top_k) {
    for (int j = lane; j < g; j += 32) {
      if (j == i || prow[j] <= 0) continue;
      const int a = i < j ? i : j;
      const int b = i < j ? j : i;
      fmat[static_cast<long long>(a) * g + b] = 1;
    }
  } else if (top_k <= kLaneTopK) {
    int* cj = cand_j[threadIdx.x >> 5];
    const int nt = (g + 31) >> 5;
    if (nt <= 1) {
      MembersTopK<1>(lane, g, i, qi, top_k, cnt, prow, old, old_i, q, cj, fmat);
    } else if (nt <= 2) {
      MembersTopK<2>(lane, g, i, qi, top_k, cnt, prow, old, old_i, q, cj, fmat);
    } else if (nt <= 4) {
      MembersTopK<4>(lane, g, i, qi, top_k, cnt, prow, old, old_i, q, cj, fmat);
    } else if (nt <= 8) {
      MembersTopK<8>(lane, g, i, qi, top_k, cnt, prow, old, old_i, q, cj, fmat);
    } else {
      MembersTopK<kMaxGroup / 32>(lane, g, i, qi, top_k, cnt, prow, old, old_i, q, cj, fmat);
    }
  } else {
    RankKey prev;
    bool have_prev = false;
    for (int r = 0; r < top_k; ++r) {
      RankKey best;
      bool have = false;
      for (int j = lane; j < g; j += 32) {
        if (j == i) continue;
        const long long pg = prow[j];
        if (pg <= 0) continue;
        RankKey k;
        k.j = j;
        k.rb = ratio_of(j, pg);
        k.pg = pg;
        const int qj = q[j];
        k.lo = qi < qj ? qi : qj;
        k.hi = qi < qj ? qj : qi;
        if (have_prev && !Better(prev, k)) continue;
        if (!have || Better(k, best)) {
          best = k;
          have = true;
        }
      }
      for (int o = 16; o > 0; o >>= 1) {
        RankKey other;
        other.rb = __shfl_xor_sync(0xffffffffu, best.rb, o);
        other.pg = __shfl_xor_sync(0xffffffffu, best.pg, o);
        other.lo = __shfl_xor_sync(0xffffffffu, best.lo, o);
        other.hi = __shfl_xor_sync(0xffffffffu, best.hi, o);
        other.j = __shfl_xor_sync(0xffffffffu, best.j, o);
        const int ohave = __shfl_xor_sync(0xffffffffu, have ? 1 : 0, o);
        if (ohave && (!have || Better(other, best))) {
          best = other;
          have = true;
        }
      }
      if (!have) break;
      if (lane == 0) {
        const int a = i < best.j ? i : best.j;
        const int b = i < best.j ? best.j : i;
        fmat[static_cast<long long>(a) * g + b] = 1;
      }
      prev = best;
      have_prev = true;
    }
  }
}

// Flag bytes (0 or 1) of table word w that lie in [beg, end), as a bit set
// with one bit per set flag (bit 8k for byte k).
__device__ __forceinline__ unsigned long long RowFlagBits(const unsigned long long* fw, long long w, long long beg,
                                                          long long end) {
  const long long lo = beg - w * 8;  // first byte of the range in this word
  const long long hi = end - w * 8;  // one past the last
  unsigned long long m = 0x0101010101010101ull;
  if (lo > 0) m &= ~0ull << (8 * lo);
  if (hi < 8) m &= (1ull << (8 * hi)) - 1ull;
  return fw[w] & m;
}

// Output pass of the big groups: the union of kept pairs in (a_idx, b_idx)
// order, one CTA per group.
__global__ void __launch_bounds__(kPrepThreads) PrepareOutputKernel(PrepareParams P) {
  using BlockScan = cub::BlockScan<int, kPrepThreads>;
  __shared__ typename BlockScan::TempStorage scan_tmp;
  __shared__ int carry;
  __shared__ int eoff[kMaxGroup + 1];
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const int nwarps = kPrepThreads / 32;
  const int ri = P.list[P.list0 + blockIdx.x];
  const int gid = P.real[ri];
  const int g = P.glen[gid];
  const long long gg = static_cast<long long>(g) * g;
  const unsigned char* fmat = P.mat + P.mat_off[ri] + FlagOffset(gg);
  const long long* pmat = reinterpret_cast<const long long*>(P.mat + P.mat_off[ri]);
  const long long* old = reinterpret_cast<const long long*>(P.mat + P.mat_off[ri] + OldCostOffset(gg));
  const int* q = P.order + P.gstart[gid];
  // union of kept pairs in (a_idx, b_idx) order. The flags of row a,
  // bytes [a*g + a + 1, a*g + g) of the table, are read as 8-byte words
  // (the table starts 8-byte aligned; the masked bytes past its end lie in
  // the group's old-cost array).
  const unsigned long long* fw = reinterpret_cast<const unsigned long long*>(fmat);
  for (int a = warp; a < g; a += nwarps) {
    const long long beg = static_cast<long long>(a) * g + a + 1;
    const long long end = static_cast<long long>(a) * g + g;
    int cnt = 0;
    for (long long w = (beg >> 3) + lane; w < (end + 7) >> 3; w += 32) cnt += __popcll(RowFlagBits(fw, w, beg, end));
    cnt = WarpSumInt(cnt);
    if (lane == 0) eoff[a] = cnt;
  }
  __syncthreads();
  if (tid == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < g; base += kPrepThreads) {
    const int i = base + tid;
    const int v = i < g ? eoff[i] : 0;
    int ex = 0, agg = 0;
    BlockScan(scan_tmp).ExclusiveSum(v, ex, agg);
    __syncthreads();
    if (i < g) eoff[i] = carry + ex;
    __syncthreads();
    if (tid == 0) carry += agg;
    __syncthreads();
  }
  const int nc = carry;
  int2* out = P.cand + P.cand_off[ri];
  for (int a = warp; a < g; a += nwarps) {
    const long long beg = static_cast<long long>(a) * g + a + 1;
    const long long end = static_cast<long long>(a) * g + g;
    const long long row0 = static_cast<long long>(a) * g;
    int pos = eoff[a];
    for (long long w0 = beg >> 3; w0 < (end + 7) >> 3; w0 += 32) {
      const long long w = w0 + lane;
      unsigned long long bits = w < (end + 7) >> 3 ? RowFlagBits(fw, w, beg, end) : 0ull;
      const int c = __popcll(bits);
      int incl = c;
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      long long at = pos + incl - c;
      while (bits) {
        const int k = (__ffsll(static_cast<long long>(bits)) - 1) >> 3;
        bits &= bits - 1;
        const int b = static_cast<int>(w * 8 + k - row0);
        out[at] = make_int2(a, b);
        P.cand_rep[P.cand_off[ri] + at] = make_int2(q[a], q[b]);
        if (P.cand_feat) {
          const long long pg = pmat[static_cast<long long>(a) * g + b];
          long long denom = old[a] + old[b];
          if (denom < 1) denom = 1;
          // a ranker feature, not a decision: single precision is enough
          P.cand_feat[P.cand_off[ri] + at] =
              make_float2(static_cast<float>(pg), __fdividef(static_cast<float>(pg), static_cast<float>(denom)));
        }
        ++at;
      }
      pos += __shfl_sync(0xffffffffu, incl, 31);
    }
  }
  if (tid == 0) {
    P.cand_cnt[ri] = nc;
    atomicAdd(&P.stats[kStCandAfterPrune], static_cast<unsigned long long>(nc));
  }
}

// ------------------------------------------------------------ prepare, small groups

// Groups of at most kSmallGroup members (99% of the real groups on R-MAT
// workloads): one warp per group, no block-wide barrier. The group's rows and
// their target sizes are staged in shared memory in one coalesced pass when
// they fit; the EA-proxy sum over targets shared by two members then equals,
// per member pair, the sum over the intersection of their two sorted rows (a
// row never holds its own rep, so the reference's own-rep exclusion is
// implied), which one lane computes per pair with a two-pointer merge while
// the other lanes do the other pairs. Groups whose rows do not fit are handled
// warp-cooperatively from global memory. Output and counters equal those of
// PrepareKernel.
constexpr int kSmallGroup = 32;
constexpr int kSmallWarps = 4;
constexpr int kSmallPairs = kSmallGroup * (kSmallGroup - 1) / 2;
constexpr int kSmallStage = 256;  // staged row entries per group

struct SmallWarpSmem {
  long long p[kSmallPairs];  // upper triangle, TriIndex(a, b)
  long long old[kSmallGroup];
  Entry ent[kSmallStage];
  int tsz[kSmallStage];
  int q[kSmallGroup];
  int sz[kSmallGroup];
  int len[kSmallGroup];
  int start[kSmallGroup + 1];
  unsigned fmask[kSmallGroup];
  long long off[kSmallGroup];
};

struct SmallSmem {
  SmallWarpSmem w[kSmallWarps];
};

__device__ __forceinline__ int TriIndex(int a, int b, int g) { return a * (2 * g - a - 1) / 2 + (b - a - 1); }

__global__ void __launch_bounds__(kSmallWarps * 32) PrepareSmallKernel(PrepareParams P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SmallWarpSmem& S = reinterpret_cast<SmallSmem*>(smem_raw)->w[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int li = blockIdx.x * kSmallWarps + (threadIdx.x >> 5);
  if (li >= P.nlist) return;
  const int ri = P.list[P.list0 + li];
  const int gid = P.real[ri];
  const int g = P.glen[gid];
  const QuotientView& Q = P.Q;
  const int* order = P.order + P.gstart[gid];
  long long off = 0;
  int len = 0;
  if (lane < g) {
    const int rep = order[lane];
    S.q[lane] = rep;
    S.sz[lane] = Q.size[rep];
    len = Q.len[rep];
    off = Q.off[rep];
    S.len[lane] = len;
    S.off[lane] = off;
    S.fmask[lane] = 0;
  }
  // row starts in the staging buffer
  int incl = len;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  const int E = __shfl_sync(0xffffffffu, incl, 31);
  if (lane < g) S.start[lane] = incl - len;
  if (lane == 0) S.start[g] = E;
  const int npairs = g * (g - 1) / 2;
  for (int k = lane; k < npairs; k += 32) S.p[k] = 0;
  const bool staged = E <= kSmallStage;
  __syncwarp();
  if (staged) {
    // one flat pass over the group's entries (independent loads), then the
    // target sizes
#pragma unroll 4
    for (int k = lane; k < E; k += 32) {
      int lo = 0, hi = g;  // row of entry k: last i with start[i] <= k
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (S.start[mid] <= k) lo = mid; else hi = mid;
      }
      S.ent[k] = Q.ent[S.off[lo] + (k - S.start[lo])];
    }
    __syncwarp();
#pragma unroll 4
    for (int k = lane; k < E; k += 32) S.tsz[k] = Q.size[EntNb(S.ent[k])];
  }
  __syncwarp();
  unsigned long long examined = 0;
  if (staged) {
    // approximate old cost: one lane per member
    if (lane < g) {
      const int rep = S.q[lane];
      const long long si = S.sz[lane];
      long long old = 0, light = 0;
      int nh = 0;
      int4 hp = make_int4(-1, -1, -1, -1);
      for (int k = S.start[lane]; k < S.start[lane + 1]; ++k) {
        const long long c = EntCnt(S.ent[k]);
        const long long st = S.tsz[k];
        old += EncodeCostForPair(rep, si, EntNb(S.ent[k]), st, c);
        if (HeavyEntry(si, st, c)) {
          const int pos = k - S.start[lane];
          if (nh == 0) hp.x = pos; else if (nh == 1) hp.y = pos; else if (nh == 2) hp.z = pos; else if (nh == 3) hp.w = pos;
          ++nh;
        } else {
          light += c;
        }
      }
      if (P.rc_before) {
        P.rc_before[rep] = old;
        P.rc_light[rep] = light;
        P.rc_heavy[rep] = hp;
        P.rc_nheavy[rep] = nh;
      }
      const long long internal = Q.internal[rep];
      if (internal > 0) old += EncodeCostForPair(rep, si, rep, si, 2 * internal);
      S.old[lane] = old;
    }
    // pair proxies: one lane per member pair
    for (int pidx = lane; pidx < npairs; pidx += 32) {
      int a = 0, rem = pidx;
      while (rem >= g - 1 - a) {
        rem -= g - 1 - a;
        ++a;
      }
      const int b = a + 1 + rem;
      const int qa = S.q[a], qb = S.q[b];
      const long long sa = S.sz[a], sb = S.sz[b];
      int ia = S.start[a];
      const int ea_end = S.start[a + 1];
      int ib = S.start[b];
      const int eb_end = S.start[b + 1];
      long long sum = 0, direct = 0;
      while (ia < ea_end && ib < eb_end) {
        const int ta = EntNb(S.ent[ia]);
        const int tb = EntNb(S.ent[ib]);
        if (ta < tb) {
          if (ta == qb) direct = EntCnt(S.ent[ia]);
          ++ia;
        } else if (tb < ta) {
          ++ib;
        } else {
          const long long ea = EntCnt(S.ent[ia]);
          const long long eb = EntCnt(S.ent[ib]);
          const long long st = S.tsz[ia];
          const long long delta = EncodeCostForPair(qa, sa, ta, st, ea) + EncodeCostForPair(qb, sb, ta, st, eb) -
                                  EncodeCostForPair(qa, sa + sb, ta, st, ea + eb);
          if (delta > 0) sum += delta;
          ++examined;
          ++ia;
          ++ib;
        }
      }
      for (; ia < ea_end; ++ia) {
        if (EntNb(S.ent[ia]) == qb) direct = EntCnt(S.ent[ia]);
      }
      S.p[pidx] = sum + direct;
    }
  } else {
    // rows too long to stage: warp-cooperative passes over global memory
    for (int i = 0; i < g; ++i) {
      const int rep = S.q[i];
      const long long si = S.sz[i];
      const long long oi = __shfl_sync(0xffffffffu, off, i);
      const int li2 = S.len[i];
      long long old = 0, light = 0;
      int nh = 0;
      if (P.rc_before && lane == 0) P.rc_heavy[rep] = make_int4(-1, -1, -1, -1);
      __syncwarp();
      for (int k0 = 0; k0 < li2; k0 += 32) {
        const int k = k0 + lane;
        bool heavy = false;
        if (k < li2) {
          const Entry e = Q.ent[oi + k];
          const long long c = EntCnt(e);
          const long long st = Q.size[EntNb(e)];
          old += EncodeCostForPair(rep, si, EntNb(e), st, c);
          heavy = HeavyEntry(si, st, c);
          if (!heavy) light += c;
        }
        if (P.rc_before) RecordHeavy(P.rc_heavy + rep, nh, heavy, k);
      }
      old = WarpSum(old);
      if (P.rc_before) light = WarpSum(light);
      if (lane == 0) {
        if (P.rc_before) {
          P.rc_before[rep] = old;
          P.rc_light[rep] = light;
          P.rc_nheavy[rep] = nh;
        }
        const long long internal = Q.internal[rep];
        if (internal > 0) old += EncodeCostForPair(rep, si, rep, si, 2 * internal);
        S.old[i] = old;
      }
    }
    for (int a = 0; a < g; ++a) {
      const int qa = S.q[a];
      const long long sa = S.sz[a];
      const Entry* ra = Q.ent + __shfl_sync(0xffffffffu, off, a);
      const int la = S.len[a];
      for (int b = a + 1; b < g; ++b) {
        const int qb = S.q[b];
        const long long sb = S.sz[b];
        const Entry* rb = Q.ent + __shfl_sync(0xffffffffu, off, b);
        const int lb = S.len[b];
        const bool a_short = la <= lb;
        const Entry* rs = a_short ? ra : rb;
        const Entry* rl = a_short ? rb : ra;
        const int ls = a_short ? la : lb;
        const int ll = a_short ? lb : la;
        long long sum = 0;
        int shared = 0;
        for (int k = lane; k < ls; k += 32) {
          const Entry e = rs[k];
          const int t = EntNb(e);
          const long long co = RowLookup(rl, ll, t);
          if (co == 0) continue;
          ++shared;
          const long long ea = a_short ? EntCnt(e) : co;
          const long long eb = a_short ? co : EntCnt(e);
          const long long st = Q.size[t];
          const long long delta = EncodeCostForPair(qa, sa, t, st, ea) + EncodeCostForPair(qb, sb, t, st, eb) -
                                  EncodeCostForPair(qa, sa + sb, t, st, ea + eb);
          if (delta > 0) sum += delta;
        }
        sum = WarpSum(sum);
        const int sh = WarpSumInt(shared);
        if (lane == 0) {
          examined += static_cast<unsigned long long>(sh);
          S.p[TriIndex(a, b, g)] = sum + RowLookup(ra, la, qb);
        }
      }
    }
  }
  __syncwarp();
  // per member (one lane each): positive partners, ratio, top-k
  int top_k = P.top_k < g - 1 ? P.top_k : g - 1;
  if (top_k < 1) top_k = 1;
  if (lane < g && g - 1 <= P.top_k) {
    // every member has at most top_k partners: all positive ones are kept
    const int i = lane;
    for (int j = i + 1; j < g; ++j) {
      if (S.p[TriIndex(i, j, g)] > 0) atomicOr(&S.fmask[i], 1u << j);
    }
  } else if (g - 1 > P.top_k) {
    // ranking, one member at a time by the whole warp, lane j holding
    // partner j: a partner's rank is the number of partners better than it
    // under ranked_better (ratio desc, proxy gain desc, rep_lo asc, rep_hi
    // asc), and the top_k ranks are kept. The ratio is the same correctly
    // rounded double as the reference's; positive doubles order like their
    // bit patterns, so every comparison is an integer one.
    const int j = lane;
    for (int i = 0; i < g; ++i) {
      long long pg = 0;
      if (j < g && j != i) pg = S.p[i < j ? TriIndex(i, j, g) : TriIndex(j, i, g)];
      const bool valid = pg > 0;
      const unsigned vm = __ballot_sync(0xffffffffu, valid);
      const int cnt = __popc(vm);
      if (cnt <= top_k) {
        if (valid) atomicOr(&S.fmask[i < j ? i : j], 1u << (i < j ? j : i));
        continue;
      }
      long long rbits = 0;
      int lo = 0, hi = 0;
      if (valid) {
        long long denom = S.old[i] + S.old[j];
        if (denom < 1) denom = 1;
        rbits = __double_as_longlong(static_cast<double>(pg) / static_cast<double>(denom));
        const int qi = S.q[i];
        const int qj = S.q[j];
        lo = qi < qj ? qi : qj;
        hi = qi < qj ? qj : qi;
      }
      int rank = 0;
      for (unsigned rest = vm; rest; rest &= rest - 1) {
        const int o = __ffs(rest) - 1;
        const long long orb = __shfl_sync(0xffffffffu, rbits, o);
        const long long opg = __shfl_sync(0xffffffffu, pg, o);
        const int olo = __shfl_sync(0xffffffffu, lo, o);
        const int ohi = __shfl_sync(0xffffffffu, hi, o);
        const bool better =
            orb != rbits ? orb > rbits : opg != pg ? opg > pg : olo != lo ? olo < lo : ohi < hi;
        rank += (valid && o != j && better) ? 1 : 0;
      }
      if (valid && rank < top_k) atomicOr(&S.fmask[i < j ? i : j], 1u << (i < j ? j : i));
    }
  }
  __syncwarp();
  // union of kept pairs in (a_idx, b_idx) order
  const unsigned mine = lane < g ? S.fmask[lane] : 0u;
  const int cnt = __popc(mine);
  int ex = cnt;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, ex, o);
    if (lane >= o) ex += y;
  }
  const int total = __shfl_sync(0xffffffffu, ex, 31);
  ex -= cnt;
  int2* out = P.cand + P.cand_off[ri];
  float2* feat = P.cand_feat ? P.cand_feat + P.cand_off[ri] : nullptr;
  unsigned bits = mine;
  while (bits) {
    const int b = __ffs(bits) - 1;
    bits &= bits - 1;
    if (feat) {
      const long long pg = S.p[TriIndex(lane, b, g)];
      long long denom = S.old[lane] + S.old[b];
      if (denom < 1) denom = 1;
      feat[ex] = make_float2(static_cast<float>(pg), __fdividef(static_cast<float>(pg), static_cast<float>(denom)));
    }
    P.cand_rep[P.cand_off[ri] + ex] = make_int2(S.q[lane], S.q[b]);
    out[ex++] = make_int2(lane, b);
  }
  examined = static_cast<unsigned long long>(WarpSum(static_cast<long long>(examined)));
  if (lane == 0) {
    P.cand_cnt[ri] = total;
    atomicAdd(&P.stats[kStGroupCount], 1ull);
    atomicMax(&P.stats[kStGroupMaxSize], static_cast<unsigned long long>(g));
    atomicAdd(&P.stats[kStRawPairCount], static_cast<unsigned long long>(g) * (g - 1) / 2);
    atomicAdd(&P.stats[kStCandAfterPrune], static_cast<unsigned long long>(total));
    atomicAdd(&P.stats[kStProxyExamined], examined);
    atomicAdd(&P.stats[kStPrepareBytes], 12ull * static_cast<unsigned long long>(E));
  }
}

// ------------------------------------------------------------ score

struct ScoreParams {
  QuotientView Q;
  BlockCtl* ctl;  // work queues of the scoring passes
  const int* order;
  const int* gstart;
  const int* real;
  int rg0;
  int nrg;
  const long long* cand_off;
  const int2* cand;
  const int* cand_cnt;
  const int2* cand_rep;  // the pair's supernode ids, -1 for unused slots
  longlong2* res;
  // learned ranker (phase 0: off, every slot scored). keep[slot]: 1 =
  // exploration slot, scored in phase 1; 2 = scored in phase 2 iff its logit
  // zbuf[slot] >= *cutoff (the cutoff comes from phase 1's passing pairs)
  int phase;
  const unsigned char* keep;
  const float* zbuf;
  float* zpos;        // phase 1: logits of the exploration pairs passing the filter
  long long* zgain;   // phase 1: their exact gains
  unsigned* npos;
  unsigned zcap;
  const float* cutoff;
  int audit;          // phase 2: score pruned slots aside and count the ones the filter passes
  double threshold;
  ThresholdBits thr;  // threshold split for the integer test
  int use_threshold;
  RowConsts rc;  // row sums of the block-start state (rc.before == nullptr: full merge)
  unsigned long long* stats;
  DevError* err;
};

// m: the two rows' staged scalars (read only with row sums)
__device__ __forceinline__ void ScoreGain(const ScoreParams& P, int a, int b, const RowMeta* m, long long* gain,
                                          long long* before, GainWork* w) {
  if (P.rc.before) {
    WarpExactGainShared(P.Q, a, b, m[0], m[1], gain, before, w, P.err);
  } else {
    WarpExactGain(P.Q, a, b, gain, before, w, P.err);
  }
}

__device__ __forceinline__ bool PassesFilter(long long gain, long long before, double threshold, ThresholdBits thr,
                                             int use_threshold) {
  if (gain <= 0) return false;
  if (!use_threshold) return true;
  return before > 0 && RatioAtLeast(gain, before, threshold, thr);
}

__device__ __forceinline__ void FlushScoreStats(unsigned long long* stats, const GainWork& w, long long pairs,
                                                long long view_nnz) {
  if (pairs == 0) return;
  atomicAdd(&stats[kStExactCalls], static_cast<unsigned long long>(pairs));
  atomicAdd(&stats[kStInputNnz], static_cast<unsigned long long>(view_nnz));
  atomicAdd(&stats[kStRawA], static_cast<unsigned long long>(w.raw_a));
  atomicAdd(&stats[kStRawB], static_cast<unsigned long long>(w.raw_b));
  atomicAdd(&stats[kStUnion], static_cast<unsigned long long>(w.uni));
  atomicAdd(&stats[kStOverlap], static_cast<unsigned long long>(w.ovl));
  // algorithmic bytes: the gain computations' own, 8 B pair + 16 B result per pair
  atomicAdd(&stats[kStScoreBytes], static_cast<unsigned long long>(w.bytes + 24 * pairs));
}

// One warp per candidate slot of the block (the concatenated per-group
// candidate capacities); slots past a group's candidate count hold -1 and
// are skipped.
// Slots are fetched from the block's queue kScoreFetch at a time (pairs over
// hub rows cost orders of magnitude more than the rest). Fetch c takes the
// slots c, c + F, c + 2F, ... (F = the number of fetches): the candidates of
// one member are consecutive slots, and a hub member's pairs must not all
// land on one warp. The warp loads the fetch's pair ids and (with row sums)
// the scalars of their rows together, one slot or row per lane, before it
// scores the pairs one by one: one load latency per fetch instead of a chain
// of them per pair.
constexpr int kScoreFetch = 16;
static_assert(2 * kScoreFetch == 32, "one staged row per lane");

__global__ void __launch_bounds__(kScoreThreads, 4) ScoreKernel(ScoreParams P) {
  __shared__ RowMeta s_meta[kScoreThreads / 32][2 * kScoreFetch];
  constexpr unsigned kFull = 0xffffffffu;
  const long long s0 = P.cand_off[P.rg0];
  const long long s1 = P.cand_off[P.rg0 + P.nrg];
  const int lane = threadIdx.x & 31;
  RowMeta* wm = s_meta[threadIdx.x >> 5];
  GainWork w = {0, 0, 0, 0, 0};
  long long pairs = 0, view_nnz = 0;
  unsigned long long pruned = 0;
  const float cutoff = P.phase == 2 ? *P.cutoff : 0.0f;
  unsigned long long* queue = &P.ctl->work_next[P.phase == 2 ? 2 : 1];
  const long long nfetch = (s1 - s0 + kScoreFetch - 1) / kScoreFetch;
  for (;;) {
    long long f = 0;
    if (lane == 0) f = static_cast<long long>(atomicAdd(queue, 1ull));
    f = __shfl_sync(kFull, f, 0);
    if (f >= nfetch) break;
    // lane j < kScoreFetch: slot j of the fetch, its pair, and what to do
    // with it (0 nothing, 1 score, 2 pruned by the ranker)
    const long long slot = s0 + f + static_cast<long long>(lane & (kScoreFetch - 1)) * nfetch;
    int2 ab = make_int2(-1, -1);
    int todo = 0;
    if (lane < kScoreFetch && slot < s1) {
      ab = P.cand_rep[slot];
      if (ab.x >= 0) {
        todo = 1;
        if (P.phase == 1 && P.keep[slot] != 1) todo = 0;  // phase 1 scores the exploration slots
        if (P.phase == 2) {
          if (P.keep[slot] == 1) {
            todo = 0;  // exploration slot, scored in phase 1
          } else if (P.zbuf[slot] < cutoff) {
            todo = 2;
          }
        }
      }
    }
    // lane l stages row (l & 1) of pair l >> 1: its supernode and, with row
    // sums, its scalars
    {
      const int j = lane >> 1;
      const int ja = __shfl_sync(kFull, ab.x, j);
      const int jb = __shfl_sync(kFull, ab.y, j);
      const int jt = __shfl_sync(kFull, todo, j);
      const int r = (lane & 1) ? jb : ja;
      if (P.rc.before && (jt == 1 || (jt == 2 && P.audit))) {
        LoadRowMeta(P.Q, P.rc, r, &wm[lane]);
      } else {
        wm[lane].rep = r;
      }
    }
    const unsigned prune = __ballot_sync(kFull, todo == 2);
    unsigned live = __ballot_sync(kFull, todo != 0);
    __syncwarp();
    for (; live != 0u; live &= live - 1u) {
      const int j = __ffs(live) - 1;
      const RowMeta* m = wm + 2 * j;
      const int a = m[0].rep;
      const int b = m[1].rep;
      const long long sj = s0 + f + static_cast<long long>(j) * nfetch;
      long long gain = 0, before = 0;
      if ((prune >> j) & 1u) {
        // pruned by the ranker: not scored (the audit scores it aside)
        if (P.audit) {
          GainWork aw = {0, 0, 0, 0, 0};
          ScoreGain(P, a, b, m, &gain, &before, &aw);
          if (lane == 0 && PassesFilter(gain, before, P.threshold, P.thr, P.use_threshold)) {
            atomicAdd(&P.stats[kStRkAuditPassing], 1ull);
            atomicAdd(&P.stats[kStRkAuditLost], 1ull);
          }
        }
        if (lane == 0) {
          P.res[sj] = make_longlong2(0, -1);
          ++pruned;
        }
        continue;
      }
      ScoreGain(P, a, b, m, &gain, &before, &w);
      if (lane == 0) {
        if (P.phase != 0 && PassesFilter(gain, before, P.threshold, P.thr, P.use_threshold)) {
          if (P.audit) atomicAdd(&P.stats[kStRkAuditPassing], 1ull);
          if (P.phase == 1) {
            const unsigned at = atomicAdd(P.npos, 1u);
            if (at < P.zcap) {
              P.zpos[at] = P.zbuf[sj];
              P.zgain[at] = gain;
            }
          }
        }
        P.res[sj] = make_longlong2(gain, before);
        ++pairs;
        if (P.rc.before) {
          view_nnz += m[0].len + (m[0].internal > 0 ? 1 : 0) + m[1].len + (m[1].internal > 0 ? 1 : 0);
        } else {
          view_nnz += P.Q.len[a] + (P.Q.internal[a] > 0 ? 1 : 0) + P.Q.len[b] + (P.Q.internal[b] > 0 ? 1 : 0);
        }
      }
    }
    __syncwarp();  // the next fetch restages this warp's rows
  }
  if (lane == 0) {
    FlushScoreStats(P.stats, w, pairs, view_nnz);
    if (pruned) atomicAdd(&P.stats[kStRkPruned], pruned);
  }
}

// Scoring service over an explicit pair list (ScoreCandidatesCuda's role).
__global__ void __launch_bounds__(kScoreThreads) ScorePairsKernel(QuotientView Q, const int* rep_a,
                                                                  const int* rep_b, long long count,
                                                                  longlong2* res, DevError* err) {
  const long long warp = (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const long long nw = (static_cast<long long>(gridDim.x) * blockDim.x) >> 5;
  const int lane = threadIdx.x & 31;
  for (long long p = warp; p < count; p += nw) {
    const int a = rep_a[p];
    const int b = rep_b[p];
    if (a == b || Q.size[a] <= 0 || Q.size[b] <= 0) {
      if (lane == 0) {
        RaiseError(err, kErrInactive, a, b, 0);
        res[p] = make_longlong2(0, 0);
      }
      continue;
    }
    long long gain = 0, before = 0;
    WarpExactGain(Q, a, b, &gain, &before, nullptr, err);
    if (lane == 0) res[p] = make_longlong2(gain, before);
  }
}

// ------------------------------------------------------------ select

struct SelectParams {
  const int* order;
  const int* gstart;
  const int* glen;
  const int* real;
  int rg0;
  const long long* cand_off;
  const int2* cand;
  const int* cand_cnt;
  const longlong2* res;
  const long long* sel_off;
  int* sel_keep;
  int* sel_rem;
  long long* sel_gain;
  int* sel_cnt;
  const int* qlen;
  int* stamp;
  int* partner;
  int* seq;
  int block_stamp;
  double threshold;
  ThresholdBits thr;  // threshold split for the integer test
  int use_threshold;
  unsigned char* scratch;
  unsigned long long scratch_cap;
  BlockCtl* ctl;
  unsigned long long* stats;
  DevError* err;
  const int* list;  // real-group positions handled by this launch
  int list0;
  int nlist;
  int* sel_list;    // selection slots of the selected pairs, appended (count: ctl->sel_total)
};

// In-place ascending bitonic sort of n (power of two) keys by one CTA.
__device__ void CtaBitonicSort(unsigned long long* keys, int n) {
  for (int k = 2; k <= n; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const unsigned long long a = keys[i];
          const unsigned long long b = keys[ixj];
          const bool up = (i & k) == 0;
          if ((a > b) == up) {
            keys[i] = b;
            keys[ixj] = a;
          }
        }
      }
      __syncthreads();
    }
  }
}

// Threshold filter, g0 order (gain desc, a_idx asc, b_idx asc) by a bitonic
// sort of packed keys, greedy endpoint-disjoint pass. The selected pairs are
// the block's commit list: the reference validates each against the same
// block-start state its score came from (gain > 0 by the filter), so every
// one is accepted; their endpoints are marked here (stamp, partner, commit
// order) for the commit kernel.
template <int kThreads, int kSmemKeys>
__global__ void __launch_bounds__(kThreads) SelectKernel(SelectParams P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned long long* skeys = reinterpret_cast<unsigned long long*>(smem_raw);
  __shared__ unsigned char used[kMaxGroup];
  __shared__ int nkeys;
  __shared__ unsigned long long* gkeys;
  __shared__ unsigned long long rej_thr, positive;
  const int tid = threadIdx.x;
  const int ri = P.list[P.list0 + blockIdx.x];
  const int gid = P.real[ri];
  const int g = P.glen[gid];
  const int cnt = g >= 2 && g <= kMaxGroup ? P.cand_cnt[ri] : 0;
  if (cnt == 0) {
    if (tid == 0) P.sel_cnt[ri] = 0;
    return;
  }
  int cap = 1;
  while (cap < cnt) cap <<= 1;
  if (tid == 0) {
    nkeys = 0;
    rej_thr = 0;
    positive = 0;
    gkeys = cap <= kSmemKeys ? skeys
                                   : ScratchAlloc(P.scratch, P.scratch_cap, P.ctl, 8ull * cap, P.err);
  }
  for (int i = tid; i < g; i += kThreads) used[i] = 0;
  __syncthreads();
  unsigned long long* keys = gkeys;
  if (keys == nullptr) {
    if (tid == 0) P.sel_cnt[ri] = 0;
    return;
  }
  const long long base = P.cand_off[ri];
  unsigned long long my_rej = 0, my_pos = 0;
  for (int c = tid; c < cnt; c += kThreads) {
    const longlong2 r = P.res[base + c];
    const long long gain = r.x;
    const long long before = r.y;
    if (before < 0) continue;  // pruned by the ranker before scoring
    if (gain <= 0) {
      ++my_rej;
      continue;
    }
    if (P.use_threshold) {
      if (before <= 0) {
        ++my_rej;
        continue;
      }
      if (!RatioAtLeast(gain, before, P.threshold, P.thr)) {
        ++my_rej;
        continue;
      }
    }
    ++my_pos;
    if (gain > kKeyGainMax) RaiseError(P.err, kErrKeyRange, gid, c, 0);
    const int2 ab = P.cand[base + c];
    const unsigned long long key = (static_cast<unsigned long long>(kKeyGainMax - gain) << (2 * kKeyIdxBits)) |
                                   (static_cast<unsigned long long>(ab.x) << kKeyIdxBits) |
                                   static_cast<unsigned long long>(ab.y);
    keys[atomicAdd(&nkeys, 1)] = key;
  }
  if (my_rej) atomicAdd(&rej_thr, my_rej);
  if (my_pos) atomicAdd(&positive, my_pos);
  __syncthreads();
  const int m = nkeys;
  int pow2 = 1;
  while (pow2 < m) pow2 <<= 1;
  for (int i = m + tid; i < pow2; i += kThreads) keys[i] = ~0ull;
  __syncthreads();
  if (m > 1) CtaBitonicSort(keys, pow2);
  if (tid == 0) {
    const int* q = P.order + P.gstart[gid];
    const long long so = P.sel_off[ri];
    int ns = 0;
    long long total = 0;
    unsigned long long overlap = 0, work = 0;
    const unsigned long long idx_mask = (1ull << kKeyIdxBits) - 1;
    for (int k = 0; k < m; ++k) {
      const unsigned long long key = keys[k];
      const int b = static_cast<int>(key & idx_mask);
      const int a = static_cast<int>((key >> kKeyIdxBits) & idx_mask);
      const long long gain = kKeyGainMax - static_cast<long long>(key >> (2 * kKeyIdxBits));
      if (used[a] || used[b]) {
        ++overlap;
        continue;
      }
      used[a] = 1;
      used[b] = 1;
      const int keep = q[a];
      const int rem = q[b];
      P.sel_keep[so + ns] = keep;
      P.sel_rem[so + ns] = rem;
      P.sel_gain[so + ns] = gain;
      P.stamp[keep] = 2 * P.block_stamp;
      P.stamp[rem] = 2 * P.block_stamp + 1;
      P.partner[keep] = rem;
      P.partner[rem] = keep;
      P.seq[rem] = static_cast<int>(so + ns);
      P.sel_list[atomicAdd(&P.ctl->sel_total, 1u)] = static_cast<int>(so + ns);
      work += static_cast<unsigned long long>(P.qlen[keep] + P.qlen[rem]);
      ++ns;
      total += gain;
    }
    P.sel_cnt[ri] = ns;
    atomicAdd(&P.stats[kStRejThreshold], rej_thr);
    atomicAdd(&P.stats[kStPositive], positive);
    atomicAdd(&P.stats[kStRejOverlap], overlap);
    atomicAdd(&P.stats[kStCandPairs], static_cast<unsigned long long>(m));
    atomicAdd(&P.stats[kStSelected], static_cast<unsigned long long>(ns));
    atomicAdd(&P.stats[kStLocalGain], static_cast<unsigned long long>(total));
    // CommitSelectedPairs validation counters (src/sweg.cpp:2683-2719): one
    // exact-gain call per selected pair, reading both rows, all accepted.
    atomicAdd(&P.stats[kStValidationCalls], static_cast<unsigned long long>(ns));
    atomicAdd(&P.stats[kStValidationWork], work);
    atomicAdd(&P.stats[kStIsolatedGain], static_cast<unsigned long long>(total));
  }
}

// Groups of more than kSelectMidGroup members: the g0 greedy pass over keys
// in ascending order selects exactly the edges that are, in some round of
// the following loop, the smallest live key at both of their endpoints
// (keys are distinct): per round every live key bids for its two endpoints
// (shared-memory atomicMin), keys that win both are selected, keys touching
// a selected endpoint die. Only the selected keys (at most g/2) are then
// sorted, which gives the greedy order of the commit list; a key is skipped
// by the greedy pass exactly when it is not selected, so the overlap count
// is the number of keys minus the selected ones.
constexpr int kMatchThreads = 512;
constexpr int kMatchSmemKeys = 8192;

__device__ __forceinline__ void SelectMatchGroup(const SelectParams& P, int ri) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned long long* skeys = reinterpret_cast<unsigned long long*>(smem_raw);
  __shared__ unsigned long long best[kMaxGroup];
  __shared__ unsigned long long chosen[kMaxGroup / 2];
  __shared__ unsigned char matched[kMaxGroup];
  __shared__ int nkeys, nchosen, live_any;
  __shared__ unsigned long long* gkeys;
  __shared__ unsigned long long rej_thr;
  const int tid = threadIdx.x;
  const int gid = P.real[ri];
  const int g = P.glen[gid];
  const int cnt = g >= 2 && g <= kMaxGroup ? P.cand_cnt[ri] : 0;
  if (cnt == 0) {
    if (tid == 0) P.sel_cnt[ri] = 0;
    return;
  }
  if (tid == 0) {
    nkeys = 0;
    nchosen = 0;
    rej_thr = 0;
    // two key buffers of cnt entries: the live keys are compacted from one
    // into the other every round
    gkeys = 2 * cnt <= kMatchSmemKeys ? skeys
                                      : ScratchAlloc(P.scratch, P.scratch_cap, P.ctl, 16ull * cnt, P.err);
  }
  for (int i = tid; i < g; i += kMatchThreads) matched[i] = 0;
  __syncthreads();
  unsigned long long* keys = gkeys;
  if (keys == nullptr) {
    if (tid == 0) P.sel_cnt[ri] = 0;
    return;
  }
  const long long base = P.cand_off[ri];
  unsigned long long my_rej = 0;
  for (int c = tid; c < cnt; c += kMatchThreads) {
    const longlong2 r = P.res[base + c];
    const long long gain = r.x;
    const long long before = r.y;
    if (before < 0) continue;  // pruned by the ranker before scoring
    bool ok = gain > 0;
    if (ok && P.use_threshold) {
      ok = before > 0 && RatioAtLeast(gain, before, P.threshold, P.thr);
    }
    if (!ok) {
      ++my_rej;
      continue;
    }
    if (gain > kKeyGainMax) RaiseError(P.err, kErrKeyRange, gid, c, 0);
    const int2 ab = P.cand[base + c];
    keys[atomicAdd(&nkeys, 1)] = (static_cast<unsigned long long>(kKeyGainMax - gain) << (2 * kKeyIdxBits)) |
                                 (static_cast<unsigned long long>(ab.x) << kKeyIdxBits) |
                                 static_cast<unsigned long long>(ab.y);
  }
  if (my_rej) atomicAdd(&rej_thr, my_rej);
  __syncthreads();
  const int m = nkeys;
  const unsigned long long idx_mask = (1ull << kKeyIdxBits) - 1;
  // rounds of locally dominant keys (each round selects at least the
  // smallest live key, so at most g/2 rounds); the keys still live after a
  // round move to the other buffer (the matching depends on the key values
  // only, not on their order)
  unsigned long long* kin = keys;
  unsigned long long* kout = keys + cnt;
  int nlive = m;
  for (int round = 0; round <= kMaxGroup / 2 && nlive > 0; ++round) {
    for (int i = tid; i < g; i += kMatchThreads) best[i] = ~0ull;
    if (tid == 0) live_any = 0;
    __syncthreads();
    for (int k = tid; k < nlive; k += kMatchThreads) {
      const unsigned long long key = kin[k];
      atomicMin(&best[(key >> kKeyIdxBits) & idx_mask], key);
      atomicMin(&best[key & idx_mask], key);
    }
    __syncthreads();
    for (int k = tid; k < nlive; k += kMatchThreads) {
      const unsigned long long key = kin[k];
      const int a = static_cast<int>((key >> kKeyIdxBits) & idx_mask);
      const int b = static_cast<int>(key & idx_mask);
      if (best[a] == key && best[b] == key) {
        matched[a] = 1;
        matched[b] = 1;
        chosen[atomicAdd(&nchosen, 1)] = key;
      }
    }
    __syncthreads();
    for (int k = tid; k < nlive; k += kMatchThreads) {
      const unsigned long long key = kin[k];
      if (!matched[(key >> kKeyIdxBits) & idx_mask] && !matched[key & idx_mask]) {
        kout[atomicAdd(&live_any, 1)] = key;
      }
    }
    __syncthreads();
    nlive = live_any;
    unsigned long long* t = kin;
    kin = kout;
    kout = t;
    __syncthreads();  // every thread has read live_any before the next round resets it
  }
  // the selected keys in greedy (ascending key) order
  const int ns = nchosen;
  int pow2 = 1;
  while (pow2 < ns) pow2 <<= 1;
  for (int i = ns + tid; i < pow2; i += kMatchThreads) chosen[i] = ~0ull;
  __syncthreads();
  if (ns > 1) CtaBitonicSort(chosen, pow2);
  const int* q = P.order + P.gstart[gid];
  const long long so = P.sel_off[ri];
  long long my_total = 0;
  unsigned long long my_work = 0;
  for (int i = tid; i < ns; i += kMatchThreads) {
    const unsigned long long key = chosen[i];
    const int a = static_cast<int>((key >> kKeyIdxBits) & idx_mask);
    const int b = static_cast<int>(key & idx_mask);
    const long long gain = kKeyGainMax - static_cast<long long>(key >> (2 * kKeyIdxBits));
    const int keep = q[a];
    const int rem = q[b];
    P.sel_keep[so + i] = keep;
    P.sel_rem[so + i] = rem;
    P.sel_gain[so + i] = gain;
    P.stamp[keep] = 2 * P.block_stamp;
    P.stamp[rem] = 2 * P.block_stamp + 1;
    P.partner[keep] = rem;
    P.partner[rem] = keep;
    P.seq[rem] = static_cast<int>(so + i);
    P.sel_list[atomicAdd(&P.ctl->sel_total, 1u)] = static_cast<int>(so + i);
    my_work += static_cast<unsigned long long>(P.qlen[keep] + P.qlen[rem]);
    my_total += gain;
  }
  // chosen[] is no longer needed: reuse best[] for the two sums
  __syncthreads();
  if (tid == 0) {
    best[0] = 0;
    best[1] = 0;
  }
  __syncthreads();
  my_total = WarpSum(my_total);
  my_work = static_cast<unsigned long long>(WarpSum(static_cast<long long>(my_work)));
  if ((tid & 31) == 0) {
    if (my_total) atomicAdd(&best[0], static_cast<unsigned long long>(my_total));
    if (my_work) atomicAdd(&best[1], my_work);
  }
  __syncthreads();
  if (tid == 0) {
    const unsigned long long total = best[0];
    P.sel_cnt[ri] = ns;
    atomicAdd(&P.stats[kStRejThreshold], rej_thr);
    atomicAdd(&P.stats[kStPositive], static_cast<unsigned long long>(m));
    atomicAdd(&P.stats[kStRejOverlap], static_cast<unsigned long long>(m - ns));
    atomicAdd(&P.stats[kStCandPairs], static_cast<unsigned long long>(m));
    atomicAdd(&P.stats[kStSelected], static_cast<unsigned long long>(ns));
    atomicAdd(&P.stats[kStLocalGain], total);
    atomicAdd(&P.stats[kStValidationCalls], static_cast<unsigned long long>(ns));
    atomicAdd(&P.stats[kStValidationWork], best[1]);
    atomicAdd(&P.stats[kStIsolatedGain], total);
  }
}

__global__ void __launch_bounds__(kMatchThreads) SelectMatchKernel(SelectParams P) {
  // list == nullptr: the real groups list0, list0 + 1, ... (a whole block)
  SelectMatchGroup(P, P.list ? P.list[P.list0 + blockIdx.x] : P.list0 + static_cast<int>(blockIdx.x));
}

// Groups of at most kSelectSmallGroup members (at most 28 candidates): one
// warp per group, one candidate per lane, a register bitonic sort across the
// lanes and the greedy pass over shuffled keys; counters are summed per CTA.
// Output and counters equal those of SelectKernel.
constexpr int kSelectSmallGroup = 8;
constexpr int kSelectSmallWarps = 8;

__device__ __forceinline__ unsigned long long WarpBitonicSortAsc(unsigned long long key, int lane) {
  for (int k = 2; k <= 32; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      const unsigned long long other = __shfl_xor_sync(0xffffffffu, key, j);
      const bool up = (lane & k) == 0;
      const bool lower = (lane & j) == 0;
      // the lower lane of a pair keeps the smaller key in an ascending run
      const bool take_min = lower == up;
      key = take_min ? (other < key ? other : key) : (other > key ? other : key);
    }
  }
  return key;
}

__global__ void __launch_bounds__(kSelectSmallWarps * 32) SelectSmallKernel(SelectParams P) {
  __shared__ unsigned long long acc[9];
  const int lane = threadIdx.x & 31;
  const int li = blockIdx.x * kSelectSmallWarps + (threadIdx.x >> 5);
  if (threadIdx.x < 9) acc[threadIdx.x] = 0;
  __syncthreads();
  if (li < P.nlist) {
    const int ri = P.list[P.list0 + li];
    const int gid = P.real[ri];
    const int g = P.glen[gid];
    const int cnt = P.cand_cnt[ri];
    const long long base = P.cand_off[ri];
    unsigned long long key = ~0ull;
    int rej = 0, pos = 0;
    if (lane < cnt) {
      const longlong2 r = P.res[base + lane];
      const long long gain = r.x;
      const long long before = r.y;
      if (before >= 0) {  // negative: pruned by the ranker before scoring
        bool ok = gain > 0;
        if (ok && P.use_threshold) {
          ok = before > 0 && RatioAtLeast(gain, before, P.threshold, P.thr);
        }
        if (!ok) {
          rej = 1;
        } else {
          pos = 1;
          if (gain > kKeyGainMax) RaiseError(P.err, kErrKeyRange, gid, lane, 0);
          const int2 ab = P.cand[base + lane];
          key = (static_cast<unsigned long long>(kKeyGainMax - gain) << (2 * kKeyIdxBits)) |
                (static_cast<unsigned long long>(ab.x) << kKeyIdxBits) | static_cast<unsigned long long>(ab.y);
        }
      }
    }
    const int m = __popc(__ballot_sync(0xffffffffu, pos != 0));
    const int nrej = __popc(__ballot_sync(0xffffffffu, rej != 0));
    key = WarpBitonicSortAsc(key, lane);
    const int* q = P.order + P.gstart[gid];
    const long long so = P.sel_off[ri];
    const unsigned long long idx_mask = (1ull << kKeyIdxBits) - 1;
    unsigned used = 0;
    int ns = 0;
    long long total = 0;
    unsigned long long overlap = 0, work = 0;
    for (int k = 0; k < m; ++k) {
      const unsigned long long kk = __shfl_sync(0xffffffffu, key, k);
      const int b = static_cast<int>(kk & idx_mask);
      const int a = static_cast<int>((kk >> kKeyIdxBits) & idx_mask);
      if ((used >> a & 1u) || (used >> b & 1u)) {
        ++overlap;
        continue;
      }
      used |= (1u << a) | (1u << b);
      const long long gain = kKeyGainMax - static_cast<long long>(kk >> (2 * kKeyIdxBits));
      if (lane == 0) {
        const int keep = q[a];
        const int rem = q[b];
        P.sel_keep[so + ns] = keep;
        P.sel_rem[so + ns] = rem;
        P.sel_gain[so + ns] = gain;
        P.stamp[keep] = 2 * P.block_stamp;
        P.stamp[rem] = 2 * P.block_stamp + 1;
        P.partner[keep] = rem;
        P.partner[rem] = keep;
        P.seq[rem] = static_cast<int>(so + ns);
        P.sel_list[atomicAdd(&P.ctl->sel_total, 1u)] = static_cast<int>(so + ns);
        work += static_cast<unsigned long long>(P.qlen[keep] + P.qlen[rem]);
      }
      ++ns;
      total += gain;
    }
    (void)g;
    if (lane == 0) {
      P.sel_cnt[ri] = ns;
      atomicAdd(&acc[0], static_cast<unsigned long long>(nrej));
      atomicAdd(&acc[1], static_cast<unsigned long long>(m));
      atomicAdd(&acc[2], overlap);
      atomicAdd(&acc[3], static_cast<unsigned long long>(m));
      atomicAdd(&acc[4], static_cast<unsigned long long>(ns));
      atomicAdd(&acc[5], static_cast<unsigned long long>(total));
      atomicAdd(&acc[6], work);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (acc[0]) atomicAdd(&P.stats[kStRejThreshold], acc[0]);
    if (acc[1]) atomicAdd(&P.stats[kStPositive], acc[1]);
    if (acc[2]) atomicAdd(&P.stats[kStRejOverlap], acc[2]);
    if (acc[3]) atomicAdd(&P.stats[kStCandPairs], acc[3]);
    if (acc[4]) {
      atomicAdd(&P.stats[kStSelected], acc[4]);
      atomicAdd(&P.stats[kStValidationCalls], acc[4]);
    }
    if (acc[5]) {
      atomicAdd(&P.stats[kStLocalGain], acc[5]);
      atomicAdd(&P.stats[kStIsolatedGain], acc[5]);
    }
    if (acc[6]) atomicAdd(&P.stats[kStValidationWork], acc[6]);
  }
}

// ------------------------------------------------------------ commit

struct CommitParams {
  QuotientView Q;
  int rg0;
  int nrg;
  const long long* sel_off;
  const int* sel_keep;
  const int* sel_rem;
  const long long* sel_gain;
  const int* sel_cnt;
  // Update_S state
  int* head;
  int* next;
  int* tail;
  int* fwd;
  int* stamp;
  int* partner;
  int* seq;
  int* claim;
  int block_stamp;
  unsigned long long* pool_top;
  unsigned long long pool_cap;
  unsigned char* scratch;
  unsigned long long scratch_cap;
  BlockCtl* ctl;
  unsigned long long* stats;
  DevError* err;
  int* rows_short;  // claimed neighbour rows of at most kWarpRowMax entries (count: ctl->short_cnt)
  int* rows_long;   // the other claimed neighbour rows (count: ctl->long_cnt)
  unsigned* ticket; // last-CTA counter of the rewrite kernel, left at 0
  const int* sel_list;  // selection slots of the block's selected pairs (count: ctl->sel_total)
  int warp_pairs;       // 1: pairs with at most kWarpRow row entries go to CommitShortKernel
};

// Optional re-validation (--verify-cuda-gain): recomputes the exact gain of
// every selected pair against the block-start state and checks it equals
// the scored gain and is positive.
__global__ void __launch_bounds__(256) VerifyKernel(CommitParams P) {
  const int lane = threadIdx.x & 31;
  const long long warp = (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const long long nw = (static_cast<long long>(gridDim.x) * blockDim.x) >> 5;
  const unsigned total = P.ctl->sel_total;
  for (long long idx = warp; idx < total; idx += nw) {
    const long long slot = P.sel_list[idx];
    const int k = P.sel_keep[slot];
    const int r = P.sel_rem[slot];
    long long gain = 0, before = 0;
    WarpExactGain(P.Q, k, r, &gain, &before, nullptr, P.err);
    if (lane == 0 && (gain != P.sel_gain[slot] || gain <= 0)) RaiseError(P.err, kErrValidation, k, r, 0);
  }
}

// Marks the endpoints of an explicit merge batch (no selection step).
__global__ void MarkKernel(const int* keep, const int* rem, int count, int* stamp, int* partner, int* seq,
                           int block_stamp, int* sel_list, BlockCtl* ctl) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) {
    stamp[keep[i]] = 2 * block_stamp;
    stamp[rem[i]] = 2 * block_stamp + 1;
    partner[keep[i]] = rem[i];
    partner[rem[i]] = keep[i];
    seq[rem[i]] = i;
    sel_list[i] = i;
  }
  if (i == 0) ctl->sel_total = static_cast<unsigned>(count);
}

struct RowsSmem {
  Entry s[kRowSmem];
  int d[kRowSmem + 1];
  Entry ins[kRowSmem];
};
// every warp of a rewrite CTA has a kWarpRowMax slice of s and of ins
static_assert(kWarpRowMax * (kRowsThreads / 32) <= kRowSmem, "warp slices of the rewrite buffers");

// Rewrites a staged sorted row S[0..L) (adjacent equal ids allowed: the keep
// row is staged as the merge of two rows) into out: duplicates are summed,
// ids sk / sr are dropped, entries of supernodes removed in this block move
// to their keep partner (summed into its entry, or inserted at its sorted
// position). Returns the new length.
__device__ int RewriteRow(const CommitParams& P, Entry* S, int L, int* D, Entry* INS, int sk, int sr, Entry* out) {
  using BlockScan = cub::BlockScan<int, kRowsThreads>;
  __shared__ typename BlockScan::TempStorage scan_tmp;
  __shared__ int nins, carry;
  const int tid = threadIdx.x;
  const int remove_stamp = 2 * P.block_stamp + 1;
  if (tid == 0) {
    nins = 0;
    carry = 0;
  }
  if (sk >= 0) {
    // a keep row staged as the merge of two rows: equal neighbours are adjacent
    for (int i = tid; i < L; i += kRowsThreads) {
      int drop = 0;
      if (i > 0 && EntNb(S[i]) == EntNb(S[i - 1])) {
        atomicAdd(reinterpret_cast<unsigned long long*>(&S[i - 1]), static_cast<unsigned long long>(EntCnt(S[i])));
        drop = 1;
      }
      D[i] = drop;
    }
  } else {
    // a neighbour row is canonical
    for (int i = tid; i < L; i += kRowsThreads) D[i] = 0;
  }
  __syncthreads();
  // entries of supernodes removed in this block: four lookups in flight per
  // thread
  for (int i0 = tid; i0 < L; i0 += 4 * kRowsThreads) {
    int id[4], st[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = i0 + u * kRowsThreads;
      id[u] = i < L && !D[i] ? EntNb(S[i]) : -1;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) st[u] = id[u] >= 0 && id[u] != sk && id[u] != sr ? P.stamp[id[u]] : 0;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = i0 + u * kRowsThreads;
      if (id[u] < 0) continue;
      if (id[u] == sk || id[u] == sr) {
        D[i] = 1;
        continue;
      }
      if (st[u] == remove_stamp) {
        const int kp = P.partner[id[u]];
        D[i] = 1;
        if (kp == sk) continue;
        const int p = RowLowerBound(S, L, kp);
        const long long c = EntCnt(S[i]);
        if (p < L && EntNb(S[p]) == kp) {
          atomicAdd(reinterpret_cast<unsigned long long*>(&S[p]), static_cast<unsigned long long>(c));
        } else {
          INS[atomicAdd(&nins, 1)] = MakeEnt(kp, c);
        }
      }
    }
  }
  __syncthreads();
  // exclusive scan of drop flags (D[L] = total), four flags per thread a step
  for (int base = 0; base < L; base += 4 * kRowsThreads) {
    const int i0 = base + 4 * tid;
    int v[4], sum = 0;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      v[u] = i0 + u < L ? D[i0 + u] : 0;
      sum += v[u];
    }
    int ex = 0, agg = 0;
    BlockScan(scan_tmp).ExclusiveSum(sum, ex, agg);
    __syncthreads();
    int run = carry + ex;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (i0 + u < L) D[i0 + u] = run;
      run += v[u];
    }
    __syncthreads();
    if (tid == 0) carry += agg;
    __syncthreads();
  }
  if (tid == 0) D[L] = carry;
  const int m = nins;
  int pow2 = 1;
  while (pow2 < m) pow2 <<= 1;
  for (int i = m + tid; i < pow2; i += kRowsThreads) INS[i] = ~0ull;
  __syncthreads();
  if (m > 1) CtaBitonicSort(INS, pow2);
  for (int i = tid; i < L; i += kRowsThreads) {
    if (D[i + 1] != D[i]) continue;  // dropped
    const Entry e = S[i];
    const int pos = i - D[i] + RowLowerBound(INS, m, EntNb(e));
    out[pos] = e;
  }
  for (int j = tid; j < m; j += kRowsThreads) {
    const Entry e = INS[j];
    const int p = RowLowerBound(S, L, EntNb(e));
    out[j + p - D[p]] = e;
  }
  __syncthreads();
  return L - D[L] + m;
}

// Staging buffers for a row of L entries: shared memory when it fits,
// block scratch otherwise. Returns false (error raised) when scratch is out.
__device__ bool StageBuffers(const CommitParams& P, RowsSmem& R, int L, Entry** S, int** D, Entry** INS) {
  __shared__ Entry* gbuf;
  if (L <= kRowSmem) {
    *S = R.s;
    *D = R.d;
    *INS = R.ins;
    return true;
  }
  int pow2 = 1;
  while (pow2 < L) pow2 <<= 1;
  if (threadIdx.x == 0) {
    gbuf = reinterpret_cast<Entry*>(ScratchAlloc(P.scratch, P.scratch_cap, P.ctl,
                                                 8ull * L + 4ull * (L + 1) + 8ull * pow2 + 512ull, P.err));
  }
  __syncthreads();
  if (gbuf == nullptr) return false;
  *S = gbuf;
  *INS = gbuf + L;
  *D = reinterpret_cast<int*>(gbuf + L + pow2);
  return true;
}

// One CTA per selected pair of the block (persistent grid over the block's
// selection slots). Per pair:
//   Update_S bookkeeping: size, internal count, member list, forwarding, and
//     QuotientGraph::Merge's touched-entry count replayed in commit order
//   keep row <- merge(row keep, row remove) with the block's removes folded
//     into their keeps, written to fresh pool space
//   every neighbour row of remove that is not a keep/remove of this block is
//     claimed once per block and rewritten in place (remove -> its keep)
// Rows of keeps and removes are only read (the keep row goes to new space),
// and a claimed neighbour row is touched by its claimant alone, so the CTAs
// need no ordering among themselves.
__global__ void __launch_bounds__(kRowsThreads) CommitKernel(CommitParams P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  RowsSmem& R = *reinterpret_cast<RowsSmem*>(smem_raw);
  __shared__ long long new_off;
  __shared__ int folded_sum;
  const QuotientView& Q = P.Q;
  const int tid = threadIdx.x;
  const int remove_stamp = 2 * P.block_stamp + 1;
  const unsigned total = P.ctl->sel_total;
  for (unsigned idx = blockIdx.x; idx < total; idx += gridDim.x) {
    const long long slot = P.sel_list[idx];
    const int k = P.sel_keep[slot];
    const int r = P.sel_rem[slot];
    const int lr = Q.len[r];
    const int lk = Q.len[k];
    if (P.warp_pairs && lk + lr <= kWarpRow) continue;  // CommitShortKernel's pair
    const Entry* rr = Q.ent + Q.off[r];
    const Entry* rk = Q.ent + Q.off[k];
    const int my_seq = static_cast<int>(slot);
    if (tid == 0) folded_sum = 0;
    __syncthreads();
    // touched count and neighbour-row claims (block-start row of remove); a
    // claimed row goes to the short or long rewrite list
    int folded = 0;
    for (int i = tid; i < lr; i += kRowsThreads) {
      const int x = EntNb(rr[i]);
      if (x == k) continue;
      const int sx = P.stamp[x];
      if (sx == remove_stamp && P.seq[x] < my_seq && RowLookup(rr, lr, P.partner[x]) != 0) ++folded;
      if ((sx >> 1) == P.block_stamp) continue;  // keep/remove rows are rebuilt by their own pair
      if (atomicExch(&P.claim[x], P.block_stamp) != P.block_stamp) {
        if (Q.len[x] <= kWarpRowMax) {
          P.rows_short[atomicAdd(&P.ctl->short_cnt, 1u)] = x;
        } else {
          P.rows_long[atomicAdd(&P.ctl->long_cnt, 1u)] = x;
        }
      }
    }
    folded = WarpSumInt(folded);
    if ((tid & 31) == 0 && folded) atomicAdd(&folded_sum, folded);
    __syncthreads();
    // keep row <- merge(row k, row r), staged with keep entries first on ties
    const int L = lk + lr;
    Entry *S, *INS;
    int* D;
    if (!StageBuffers(P, R, L, &S, &D, &INS)) return;
    for (int i = tid; i < lk; i += kRowsThreads) {
      const Entry e = rk[i];
      S[i + RowLowerBound(rr, lr, EntNb(e))] = e;
    }
    for (int j = tid; j < lr; j += kRowsThreads) {
      const Entry e = rr[j];
      const int key = EntNb(e);
      int lo = 0, hi = lk;  // upper bound in row k
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (EntNb(rk[mid]) <= key) lo = mid + 1; else hi = mid;
      }
      S[j + lo] = e;
    }
    if (tid == 0) {
      const unsigned long long want = static_cast<unsigned long long>(L > 0 ? L : 1);
      const unsigned long long at = atomicAdd(P.pool_top, want);
      if (at + want > P.pool_cap) {
        RaiseError(P.err, kErrPool, k, L, 0);
        new_off = -1;
      } else {
        new_off = static_cast<long long>(at);
      }
    }
    __syncthreads();
    if (new_off < 0) return;
    const long long ekr = RowLookup(rk, lk, r);
    const int nl = RewriteRow(P, S, L, D, INS, k, r, Q.ent + new_off);
    if (tid == 0) {
      Q.internal[k] += Q.internal[r] + ekr;
      Q.internal[r] = 0;
      Q.size[k] += Q.size[r];
      Q.size[r] = 0;
      P.next[P.tail[k]] = P.head[r];
      P.tail[k] = P.tail[r];
      P.head[r] = -1;
      P.fwd[r] = k;
      Q.off[k] = new_off;
      Q.len[k] = nl;
      Q.cap[k] = L > 0 ? L : 1;
      Q.len[r] = 0;
      atomicAdd(&P.stats[kStAccepted], 1ull);
      atomicAdd(&P.stats[kStTouched],
                static_cast<unsigned long long>(2 + 3 * (lr - (ekr > 0 ? 1 : 0) - folded_sum)));
      atomicAdd(&P.stats[kStUpdateBytes], 8ull * (2ull * L + nl));
    }
    __syncthreads();
  }
}

// Selected pairs whose keep and remove rows hold at most kWarpRow entries
// together, one warp per pair: the same work as CommitKernel (claims,
// touched-entry replay, keep row = the two rows with this block's removes
// renamed to their keeps, ids k and r dropped, equal neighbours summed,
// Update_S bookkeeping), with the keep row built in registers (bitonic sort
// across the lanes, segmented sum, compaction).
__global__ void __launch_bounds__(256) CommitShortKernel(CommitParams P) {
  const QuotientView& Q = P.Q;
  const int lane = threadIdx.x & 31;
  const int remove_stamp = 2 * P.block_stamp + 1;
  const unsigned total = P.ctl->sel_total;
  const long long nw = (static_cast<long long>(gridDim.x) * blockDim.x) >> 5;
  for (long long idx = (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; idx < total;
       idx += nw) {
    const long long slot = P.sel_list[idx];
    const int k = P.sel_keep[slot];
    const int r = P.sel_rem[slot];
    const int lr = Q.len[r];
    const int lk = Q.len[k];
    if (lk + lr > kWarpRow) continue;  // CommitKernel's pair
    const Entry* rr = Q.ent + Q.off[r];
    const Entry* rk = Q.ent + Q.off[k];
    const int my_seq = static_cast<int>(slot);
    // touched count and neighbour-row claims (lanes over the remove row)
    int folded = 0;
    if (lane < lr) {
      const int x = EntNb(rr[lane]);
      if (x != k) {
        const int sx = P.stamp[x];
        if (sx == remove_stamp && P.seq[x] < my_seq && RowLookup(rr, lr, P.partner[x]) != 0) folded = 1;
        if ((sx >> 1) != P.block_stamp && atomicExch(&P.claim[x], P.block_stamp) != P.block_stamp) {
          if (Q.len[x] <= kWarpRowMax) {
            P.rows_short[atomicAdd(&P.ctl->short_cnt, 1u)] = x;
          } else {
            P.rows_long[atomicAdd(&P.ctl->long_cnt, 1u)] = x;
          }
        }
      }
    }
    const int folded_sum = __popc(__ballot_sync(0xffffffffu, folded != 0));
    // the keep row: lane i < lk holds row k's entry i, lane lk + j row r's entry j
    unsigned long long key = ~0ull;
    long long ekr = 0;
    if (lane < lk + lr) {
      const Entry e = lane < lk ? rk[lane] : rr[lane - lk];
      int id = EntNb(e);
      if (lane < lk && id == r) ekr = EntCnt(e);
      if (id != k && id != r) {
        if (P.stamp[id] == remove_stamp) id = P.partner[id];
        key = static_cast<unsigned long long>(id) << 32 | static_cast<unsigned long long>(EntCnt(e));
      }
    }
    ekr = WarpMax(ekr);
    key = WarpBitonicSortAsc(key, lane);
    const bool valid = key != ~0ull;
    const int id = static_cast<int>(key >> 32);
    const long long c = valid ? static_cast<long long>(key & 0xffffffffull) : 0;
    const int prev = __shfl_up_sync(0xffffffffu, id, 1);
    const bool head = valid && (lane == 0 || prev != id);
    long long sum = c;
    bool more = head;
    for (int j = 1; j < 32; ++j) {
      const int idj = __shfl_down_sync(0xffffffffu, id, j);
      const long long cj = __shfl_down_sync(0xffffffffu, c, j);
      if (more && lane + j < 32 && idj == id) {
        sum += cj;
      } else {
        more = false;
      }
      if (!__any_sync(0xffffffffu, more)) break;
    }
    const unsigned heads = __ballot_sync(0xffffffffu, head);
    const int nl = __popc(heads);
    const int L = lk + lr;
    long long new_off = 0;
    if (lane == 0) {
      const unsigned long long want = static_cast<unsigned long long>(L > 0 ? L : 1);
      const unsigned long long at = atomicAdd(P.pool_top, want);
      if (at + want > P.pool_cap) {
        RaiseError(P.err, kErrPool, k, L, 0);
        new_off = -1;
      } else {
        new_off = static_cast<long long>(at);
      }
    }
    new_off = __shfl_sync(0xffffffffu, new_off, 0);
    if (new_off < 0) continue;
    if (head) Q.ent[new_off + __popc(heads & ((1u << lane) - 1u))] = MakeEnt(id, sum);
    if (lane == 0) {
      Q.internal[k] += Q.internal[r] + ekr;
      Q.internal[r] = 0;
      Q.size[k] += Q.size[r];
      Q.size[r] = 0;
      P.next[P.tail[k]] = P.head[r];
      P.tail[k] = P.tail[r];
      P.head[r] = -1;
      P.fwd[r] = k;
      Q.off[k] = new_off;
      Q.len[k] = nl;
      Q.cap[k] = L > 0 ? L : 1;
      Q.len[r] = 0;
      atomicAdd(&P.stats[kStAccepted], 1ull);
      atomicAdd(&P.stats[kStTouched],
                static_cast<unsigned long long>(2 + 3 * (lr - (ekr > 0 ? 1 : 0) - folded_sum)));
      atomicAdd(&P.stats[kStUpdateBytes], 8ull * (2ull * L + nl));
    }
  }
}

// A claimed neighbour row of kWarpRow < L <= kWarpRowMax entries, one warp,
// staged in the warp's slice S of shared memory. Only the entries of
// supernodes removed in this block change: each is renamed to its keep
// partner and summed into the partner's entry when the row has one, else
// inserted (INS, sorted). Every other entry keeps its order, so its new
// position is its old one less the renamed entries before it plus the
// inserted entries below it: no sort of the row. Returns the new length.
__device__ int RewriteMediumRow(const CommitParams& P, Entry* row, int L, Entry* S, Entry* INS) {
  constexpr int kChunks = kWarpRowMax / 32;
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const int remove_stamp = 2 * P.block_stamp + 1;
  for (int j = lane; j < L; j += 32) S[j] = row[j];
  __syncwarp();
  unsigned rm[kChunks];  // renamed entries of each 32-entry chunk (warp-uniform)
  int m = 0;             // inserted entries so far
#pragma unroll
  for (int t = 0; t < kChunks; ++t) {
    const int j = lane + 32 * t;
    bool renamed = false, insert = false;
    Entry ins = 0;
    if (j < L) {
      const Entry e = S[j];
      const int id = EntNb(e);
      if (P.stamp[id] == remove_stamp) {
        renamed = true;
        const int kp = P.partner[id];
        const long long c = EntCnt(e);
        int lo = 0, hi = L;  // kp among the staged ids (only counts change meanwhile)
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (EntNb(S[mid]) < kp) lo = mid + 1; else hi = mid;
        }
        if (lo < L && EntNb(S[lo]) == kp) {
          atomicAdd(reinterpret_cast<unsigned long long*>(&S[lo]), static_cast<unsigned long long>(c));
        } else {
          insert = true;
          ins = MakeEnt(kp, c);
        }
      }
    }
    rm[t] = __ballot_sync(0xffffffffu, renamed);
    const unsigned im = __ballot_sync(0xffffffffu, insert);
    if (insert) INS[m + __popc(im & lt)] = ins;
    m += __popc(im);
  }
  // the inserted entries in id order (distinct ids: one remove per keep)
  int pow2 = 1;
  while (pow2 < m) pow2 <<= 1;
  for (int i = m + lane; i < pow2; i += 32) INS[i] = ~0ull;
  __syncwarp();
  for (int k = 2; k <= pow2; k <<= 1) {
    for (int jj = k >> 1; jj > 0; jj >>= 1) {
      for (int i = lane; i < pow2; i += 32) {
        const int ixj = i ^ jj;
        if (ixj > i) {
          const Entry a = INS[i];
          const Entry b = INS[ixj];
          if ((a > b) == ((i & k) == 0)) {
            INS[i] = b;
            INS[ixj] = a;
          }
        }
      }
      __syncwarp();
    }
  }
  // renamed entries before position q of the staged row
  auto dropped_before = [&](int q) {
    int d = 0;
#pragma unroll
    for (int t = 0; t < kChunks; ++t) {
      if (32 * t + 32 <= q) d += __popc(rm[t]);
      else if (32 * t < q) d += __popc(rm[t] & ((1u << (q - 32 * t)) - 1u));
    }
    return d;
  };
  int k_total = 0;
#pragma unroll
  for (int t = 0; t < kChunks; ++t) k_total += __popc(rm[t]);
#pragma unroll
  for (int t = 0; t < kChunks; ++t) {
    const int j = lane + 32 * t;
    if (j < L && !((rm[t] >> lane) & 1u)) {
      const Entry e = S[j];
      int lo = 0, hi = m;  // inserted entries below this id
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (EntNb(INS[mid]) < EntNb(e)) lo = mid + 1; else hi = mid;
      }
      row[j - dropped_before(j) + lo] = e;
    }
  }
  for (int i = lane; i < m; i += 32) {
    const Entry e = INS[i];
    int lo = 0, hi = L;  // staged entries below the inserted id
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (EntNb(S[mid]) < EntNb(e)) lo = mid + 1; else hi = mid;
    }
    row[lo - dropped_before(lo) + i] = e;
  }
  __syncwarp();
  return L - k_total + m;
}

// Claimed neighbour rows of at most kWarpRowMax entries, one warp per row.
// Rows of at most kWarpRow entries: each entry of a supernode removed in this
// block is renamed to its keep partner, the row is sorted by neighbour
// (register bitonic sort), equal neighbours are summed and the row is
// compacted in place (it can only shrink). Longer ones: RewriteMediumRow with
// the warp's slice of the CTA's shared memory.
__device__ void RewriteShortRows(const CommitParams& P, RowsSmem& R) {
  const QuotientView& Q = P.Q;
  const int lane = threadIdx.x & 31;
  const int warp_in_cta = threadIdx.x >> 5;
  const unsigned cnt = P.ctl->short_cnt;
  const int remove_stamp = 2 * P.block_stamp + 1;
  const long long nw = (static_cast<long long>(gridDim.x) * blockDim.x) >> 5;
  unsigned long long rows = 0, entries = 0, bytes = 0;
  for (long long idx = (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; idx < cnt; idx += nw) {
    const int x = P.rows_short[idx];
    Entry* row = Q.ent + Q.off[x];
    const int lx = Q.len[x];
    if (lx > kWarpRow) {
      const int nl = RewriteMediumRow(P, row, lx, R.s + warp_in_cta * kWarpRowMax, R.ins + warp_in_cta * kWarpRowMax);
      if (lane == 0) {
        Q.len[x] = nl;
        ++rows;
        entries += static_cast<unsigned long long>(lx);
        bytes += 8ull * static_cast<unsigned long long>(lx + nl);
      }
      continue;
    }
    unsigned long long key = ~0ull;
    if (lane < lx) {
      const Entry e = row[lane];
      int id = EntNb(e);
      if (P.stamp[id] == remove_stamp) id = P.partner[id];
      key = static_cast<unsigned long long>(id) << 32 | static_cast<unsigned long long>(EntCnt(e));
    }
    key = WarpBitonicSortAsc(key, lane);
    const bool valid = key != ~0ull;
    const int id = static_cast<int>(key >> 32);
    const long long c = valid ? static_cast<long long>(key & 0xffffffffull) : 0;
    const int prev = __shfl_up_sync(0xffffffffu, id, 1);
    const bool head = valid && (lane == 0 || prev != id);
    long long total = c;
    bool more = head;
    for (int j = 1; j < 32; ++j) {
      const int idj = __shfl_down_sync(0xffffffffu, id, j);
      const long long cj = __shfl_down_sync(0xffffffffu, c, j);
      if (more && lane + j < 32 && idj == id) {
        total += cj;
      } else {
        more = false;
      }
      if (!__any_sync(0xffffffffu, more)) break;
    }
    const unsigned heads = __ballot_sync(0xffffffffu, head);
    if (head) row[__popc(heads & ((1u << lane) - 1u))] = MakeEnt(id, total);
    const int nl = __popc(heads);
    if (lane == 0) {
      Q.len[x] = nl;
      ++rows;
      entries += static_cast<unsigned long long>(lx);
      bytes += 8ull * static_cast<unsigned long long>(lx + nl);
    }
  }
  if (lane == 0 && rows) {
    atomicAdd(&P.stats[kStRowsRewritten], rows);
    atomicAdd(&P.stats[kStRowEntriesRewritten], entries);
    atomicAdd(&P.stats[kStUpdateBytes], bytes);
  }
}

// Claimed neighbour rows longer than kWarpRow entries, one CTA per row.
__device__ void RewriteLongRows(const CommitParams& P, RowsSmem& R) {
  const QuotientView& Q = P.Q;
  const unsigned cnt = P.ctl->long_cnt;
  for (unsigned idx = blockIdx.x; idx < cnt; idx += gridDim.x) {
    const int x = P.rows_long[idx];
    Entry* rowp = Q.ent + Q.off[x];
    const int lx = Q.len[x];
    Entry *S2, *INS2;
    int* D2;
    if (!StageBuffers(P, R, lx, &S2, &D2, &INS2)) return;
    for (int i = threadIdx.x; i < lx; i += kRowsThreads) S2[i] = rowp[i];
    __syncthreads();
    const int nlx = RewriteRow(P, S2, lx, D2, INS2, -1, -1, rowp);
    if (threadIdx.x == 0) {
      Q.len[x] = nlx;
      atomicAdd(&P.stats[kStRowsRewritten], 1ull);
      atomicAdd(&P.stats[kStRowEntriesRewritten], static_cast<unsigned long long>(lx));
      atomicAdd(&P.stats[kStUpdateBytes], 8ull * (lx + nlx));
    }
    __syncthreads();
  }
}

// All claimed neighbour rows of a block: the long ones by whole CTAs first,
// then the short ones by single warps.
__global__ void __launch_bounds__(kRowsThreads) RewriteRowsKernel(CommitParams P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  RowsSmem& R = *reinterpret_cast<RowsSmem*>(smem_raw);
  __shared__ bool last;
  RewriteLongRows(P, R);
  __syncthreads();  // the shared buffers pass from the CTA's long rows to its warps
  RewriteShortRows(P, R);
  // the last CTA to finish clears the block control words for the next
  // block (every CTA has read them and made its scratch allocations by now)
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(P.ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (last && threadIdx.x == 0) {
    P.ctl->scratch_top = 0;
    P.ctl->short_cnt = 0;
    P.ctl->long_cnt = 0;
    P.ctl->sel_total = 0;
    P.ctl->work_next[0] = 0;
    P.ctl->work_next[1] = 0;
    P.ctl->work_next[2] = 0;
    *P.ticket = 0u;
  }
}

__global__ void ScatterGroupKernel(const int* __restrict__ q, const int* __restrict__ idx, int g,
                                   int* __restrict__ group_of, int* __restrict__ idx_in_group) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < g) {
    group_of[q[i]] = 0;
    idx_in_group[q[i]] = idx[i];
  }
}

__global__ void RelabelKernel(int* __restrict__ label, const int* __restrict__ fwd, int n) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < n) label[v] = fwd[label[v]];
}

}  // namespace

// --------------------------------------------------------------- host side

void Engine::ConfigureKernels() {
  CheckCuda(cudaFuncSetAttribute(PrepareKernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(sizeof(PrepSmem))), "prepare smem attribute");
  CheckCuda(cudaFuncSetAttribute(PrepareSmallKernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(sizeof(SmallSmem))), "prepare-small smem attribute");
  CheckCuda(cudaFuncSetAttribute(SelectMatchKernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 8 * kMatchSmemKeys), "select smem attribute");
  CheckCuda(cudaFuncSetAttribute(CommitKernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(sizeof(RowsSmem))), "commit smem attribute");
  CheckCuda(cudaFuncSetAttribute(RewriteRowsKernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(sizeof(RowsSmem))), "rewrite smem attribute");
  // the queue-fed kernels launch exactly the CTAs that fit on the GPU at once
  int sms = 0, per_sm = 0;
  CheckCuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cfg_.device), "SM count");
  CheckCuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, PrepareAccumKernel, kAccumThreads, 0),
            "accumulate occupancy");
  accum_grid_ = std::max(1, sms * per_sm);
  CheckCuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ScoreKernel, kScoreThreads, 0), "score occupancy");
  score_grid_ = std::max(1, sms * per_sm);
}

// Per-iteration layout: the groups with >= 2 members in Divide order, their
// candidate / selection capacities (min(C(g,2), g*top_k) and g/2) as prefix
// offsets, pair-table offsets restarting at every block, and for every block
// the range of its real groups (empty blocks do no work).
namespace {

// ---- the plan of a one-block iteration, on the device ----
// Per Divide group, the classification and offsets of the host plan
// (PrepareIterationBuffers with one block of every group): tile sums, one
// CTA scanning the tile sums, then every real group's entries scattered into
// the lists in group order.
constexpr int kPlanThreads = 256;
constexpr int kPlanItems = 8;
constexpr int kPlanTile = kPlanThreads * kPlanItems;
enum PlanScalar : int {
  kPlanR = 0, kPlanCand, kPlanSel, kPlanSmall, kPlanBig, kPlanMembers, kPlanSlots, kPlanMat, kPlanMaxE,
  kPlanSelSmall, kPlanSelMid, kPlanSelBig, kPlanSmallBase, kPlanScalars = kPlanSmallBase + 4
};
// The small-group list is laid out by member count, largest class first
// (more than 24, 17..24, 9..16, at most 8 members): the longest warps start
// first instead of forming the prepare kernel's tail.
constexpr int kPlanSmallClasses = 4;
__device__ __forceinline__ int SmallClass(int g) { return g > 24 ? 0 : g > 16 ? 1 : g > 8 ? 2 : 3; }

struct PlanSums {
  long long cand, sel, moff, soff, mat;
  int real, big, ssmall, smid, sbig;
  int small[kPlanSmallClasses];
};

struct PlanSumOp {
  __device__ __forceinline__ PlanSums operator()(const PlanSums& a, const PlanSums& b) const {
    PlanSums r;
    r.cand = a.cand + b.cand;
    r.sel = a.sel + b.sel;
    r.moff = a.moff + b.moff;
    r.soff = a.soff + b.soff;
    r.mat = a.mat + b.mat;
    r.real = a.real + b.real;
#pragma unroll
    for (int c = 0; c < kPlanSmallClasses; ++c) r.small[c] = a.small[c] + b.small[c];
    r.big = a.big + b.big;
    r.ssmall = a.ssmall + b.ssmall;
    r.smid = a.smid + b.smid;
    r.sbig = a.sbig + b.sbig;
    return r;
  }
};

__device__ __forceinline__ PlanSums PlanZero() {
  PlanSums z;
  z.cand = z.sel = z.moff = z.soff = z.mat = 0;
  z.real = z.big = z.ssmall = z.smid = z.sbig = 0;
#pragma unroll
  for (int c = 0; c < kPlanSmallClasses; ++c) z.small[c] = 0;
  return z;
}

// one group's contribution: the same rules as the host plan
__device__ __forceinline__ PlanSums PlanOfGroup(int g, unsigned e, long long k) {
  PlanSums f = PlanZero();
  if (g < 2) return f;
  const long long gl = g;
  f.real = 1;
  f.cand = gl * (gl - 1) / 2 < gl * k ? gl * (gl - 1) / 2 : gl * k;
  f.sel = gl / 2;
  if (g <= kSmallGroup && e <= static_cast<unsigned>(kSmallStage)) {
    f.small[SmallClass(g)] = 1;
  } else {
    f.big = 1;
    f.moff = gl;
    f.soff = e > static_cast<unsigned>(kSmemEntries) || g > kSmemMaxGroup ? static_cast<long long>(e) : 0;
    f.mat = (OldCostOffset(gl * gl) + 8 * gl + 255) & ~255ll;
  }
  if (g <= kSelectSmallGroup) {
    f.ssmall = 1;
  } else if (g <= kSelectMidGroup) {
    f.smid = 1;
  } else {
    f.sbig = 1;
  }
  return f;
}

struct PlanParams {
  const int* glen;
  const unsigned* gent;
  long long G;
  long long top_k;
  PlanSums* tile_sums;
  PlanSums* tile_off;
  int tiles;
  long long* scalars;
  int* real;
  long long* cand_off;
  long long* sel_off;
  long long* mat_off;
  int* small;
  int* big;
  long long* big_moff;
  long long* soff;
  int* sel_small;
  int* sel_mid;
  int* sel_big;
};

__global__ void __launch_bounds__(kPlanThreads) PlanTileKernel(PlanParams P) {
  using Reduce = cub::BlockReduce<PlanSums, kPlanThreads>;
  __shared__ typename Reduce::TempStorage tmp;
  const long long base = static_cast<long long>(blockIdx.x) * kPlanTile + threadIdx.x * kPlanItems;
  PlanSums acc = PlanZero();
  long long max_e = 0;
  for (int j = 0; j < kPlanItems; ++j) {
    const long long gi = base + j;
    if (gi >= P.G) break;
    const PlanSums f = PlanOfGroup(P.glen[gi], P.gent[gi], P.top_k);
    acc = PlanSumOp()(acc, f);
    max_e = f.soff > max_e ? f.soff : max_e;
  }
  const PlanSums t = Reduce(tmp).Reduce(acc, PlanSumOp());
  if (threadIdx.x == 0) P.tile_sums[blockIdx.x] = t;
  if (max_e > 0) {
    atomicMax(reinterpret_cast<unsigned long long*>(P.scalars + kPlanMaxE), static_cast<unsigned long long>(max_e));
  }
}

// one CTA: exclusive offsets of the tiles, the totals, and the closing
// entries of the offset arrays
__global__ void __launch_bounds__(kPlanThreads) PlanScanKernel(PlanParams P) {
  using Scan = cub::BlockScan<PlanSums, kPlanThreads>;
  __shared__ typename Scan::TempStorage tmp;
  __shared__ PlanSums carry;
  if (threadIdx.x == 0) carry = PlanZero();
  __syncthreads();
  for (int t0 = 0; t0 < P.tiles; t0 += kPlanThreads) {
    const int t = t0 + threadIdx.x;
    const PlanSums v = t < P.tiles ? P.tile_sums[t] : PlanZero();
    PlanSums ex, total;
    Scan(tmp).ExclusiveScan(v, ex, PlanZero(), PlanSumOp(), total);
    const PlanSums c = carry;
    if (t < P.tiles) P.tile_off[t] = PlanSumOp()(c, ex);
    __syncthreads();
    if (threadIdx.x == 0) carry = PlanSumOp()(c, total);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const PlanSums T = carry;
    long long* s = P.scalars;
    s[kPlanR] = T.real;
    s[kPlanCand] = T.cand;
    s[kPlanSel] = T.sel;
    long long sb = 0;
    for (int c = 0; c < kPlanSmallClasses; ++c) {
      s[kPlanSmallBase + c] = sb;
      sb += T.small[c];
    }
    s[kPlanSmall] = sb;
    s[kPlanBig] = T.big;
    s[kPlanMembers] = T.moff;
    s[kPlanSlots] = T.soff;
    s[kPlanMat] = T.mat;
    s[kPlanSelSmall] = T.ssmall;
    s[kPlanSelMid] = T.smid;
    s[kPlanSelBig] = T.sbig;
    P.cand_off[T.real] = T.cand;
    P.sel_off[T.real] = T.sel;
    P.mat_off[T.real] = 0;
    P.big_moff[T.big] = T.moff;
    P.soff[T.big] = T.soff;
  }
}

__global__ void __launch_bounds__(kPlanThreads) PlanScatterKernel(PlanParams P) {
  using Scan = cub::BlockScan<PlanSums, kPlanThreads>;
  __shared__ typename Scan::TempStorage tmp;
  const long long base = static_cast<long long>(blockIdx.x) * kPlanTile + threadIdx.x * kPlanItems;
  int g[kPlanItems];
  unsigned e[kPlanItems];
  PlanSums acc = PlanZero();
#pragma unroll
  for (int j = 0; j < kPlanItems; ++j) {
    const long long gi = base + j;
    g[j] = gi < P.G ? P.glen[gi] : 0;
    e[j] = gi < P.G ? P.gent[gi] : 0u;
    acc = PlanSumOp()(acc, PlanOfGroup(g[j], e[j], P.top_k));
  }
  PlanSums off;
  Scan(tmp).ExclusiveScan(acc, off, P.tile_off[blockIdx.x], PlanSumOp());
#pragma unroll
  for (int j = 0; j < kPlanItems; ++j) {
    const PlanSums f = PlanOfGroup(g[j], e[j], P.top_k);
    if (f.real) {
      const int ri = off.real;
      P.real[ri] = static_cast<int>(base + j);
      P.cand_off[ri] = off.cand;
      P.sel_off[ri] = off.sel;
      P.mat_off[ri] = f.big ? off.mat : 0;
      if (!f.big) {
        const int c = SmallClass(g[j]);
        P.small[P.scalars[kPlanSmallBase + c] + off.small[c]] = ri;
      } else {
        P.big[off.big] = ri;
        P.big_moff[off.big] = off.moff;
        P.soff[off.big] = off.soff;
      }
      if (f.ssmall) {
        P.sel_small[off.ssmall] = ri;
      } else if (f.smid) {
        P.sel_mid[off.smid] = ri;
      } else {
        P.sel_big[off.sbig] = ri;
      }
    }
    off = PlanSumOp()(off, f);
  }
}

}  // namespace

void Engine::PrepareIterationBuffers() {
  const int64_t G = n_groups_;
  h_real_.clear();
  h_block_rg_.clear();
  const int64_t bs = cfg_.group_batch_size;
  const long long k = cfg_.top_k > 0 ? cfg_.top_k : 1;
  for (int64_t b0 = 0; b0 < G; b0 += bs) {
    const int64_t b1 = std::min(G, b0 + bs);
    h_block_rg_.push_back(static_cast<int>(h_real_.size()));
    for (int64_t gi = b0; gi < b1; ++gi) {
      if (h_glen_[static_cast<size_t>(gi)] >= 2) h_real_.push_back(static_cast<int>(gi));
    }
  }
  h_block_rg_.push_back(static_cast<int>(h_real_.size()));
  const size_t R = h_real_.size();
  h_cand_off_.assign(R + 1, 0);
  h_sel_off_.assign(R + 1, 0);
  h_mat_off_.assign(R + 1, 0);
  long long max_mat = 0;
  for (size_t ri = 0; ri < R; ++ri) {
    const long long g = h_glen_[static_cast<size_t>(h_real_[ri])];
    h_cand_off_[ri + 1] = h_cand_off_[ri] + std::min(g * (g - 1) / 2, g * k);
    h_sel_off_[ri + 1] = h_sel_off_[ri] + g / 2;
  }
  // groups of at most kSmallGroup members whose rows fit the staging buffer
  // go to the warp-per-group kernel; only the others need pair tables in
  // global memory
  h_small_.clear();
  h_big_.clear();
  h_big_moff_.assign(1, 0);
  h_soff_.assign(1, 0);
  h_block_small_.clear();
  h_block_big_.clear();
  std::vector<long long> block_mat;
  auto is_small = [&](int ri) {
    const size_t gid = static_cast<size_t>(h_real_[static_cast<size_t>(ri)]);
    return h_glen_[gid] <= kSmallGroup && h_gent_[gid] <= static_cast<unsigned>(kSmallStage);
  };
  for (size_t b = 0; b + 1 < h_block_rg_.size(); ++b) {
    h_block_small_.push_back(static_cast<int>(h_small_.size()));
    h_block_big_.push_back(static_cast<int>(h_big_.size()));
    // a small block with any big group sends all its groups to the big path
    // (one prepare path, fewer launches; the same candidates)
    bool all_big = false;
    if (h_block_rg_[b + 1] - h_block_rg_[b] <= kFewGroups) {
      for (int ri = h_block_rg_[b]; ri < h_block_rg_[b + 1] && !all_big; ++ri) all_big = !is_small(ri);
    }
    long long off = 0;
    for (int ri = h_block_rg_[b]; ri < h_block_rg_[b + 1]; ++ri) {
      const size_t gid = static_cast<size_t>(h_real_[static_cast<size_t>(ri)]);
      const long long g = h_glen_[gid];
      // rows counted at Divide time (rows of supernodes not merged yet only
      // shrink during an iteration, so the count is an upper bound)
      if (!all_big && is_small(ri)) {
        h_small_.push_back(ri);
        continue;
      }
      h_big_.push_back(ri);
      h_big_moff_.push_back(h_big_moff_.back() + g);
      // groups beyond the shared-memory bucket table get sort slots
      const long long e_ub = h_gent_[gid];
      h_soff_.push_back(h_soff_.back() + (e_ub > kSmemEntries || g > kSmemMaxGroup ? e_ub : 0));
      h_mat_off_[static_cast<size_t>(ri)] = off;
      off += (OldCostOffset(g * g) + 8 * g + 255) & ~255ll;  // pair tables + old costs
    }
    max_mat = std::max(max_mat, off);
    block_mat.push_back(off);
  }
  h_block_small_.push_back(static_cast<int>(h_small_.size()));
  h_block_big_.push_back(static_cast<int>(h_big_.size()));
  // selection: groups of at most kSelectSmallGroup members (at most 28
  // candidates) get one warp each, the others one CTA each
  h_sel_small_.clear();
  h_sel_mid_.clear();
  h_sel_big_.clear();
  h_block_sel_small_.clear();
  h_block_sel_mid_.clear();
  h_block_sel_big_.clear();
  for (size_t b = 0; b + 1 < h_block_rg_.size(); ++b) {
    h_block_sel_small_.push_back(static_cast<int>(h_sel_small_.size()));
    h_block_sel_mid_.push_back(static_cast<int>(h_sel_mid_.size()));
    h_block_sel_big_.push_back(static_cast<int>(h_sel_big_.size()));
    for (int ri = h_block_rg_[b]; ri < h_block_rg_[b + 1]; ++ri) {
      const int g = h_glen_[static_cast<size_t>(h_real_[static_cast<size_t>(ri)])];
      (g <= kSelectSmallGroup ? h_sel_small_ : g <= kSelectMidGroup ? h_sel_mid_ : h_sel_big_).push_back(ri);
    }
  }
  h_block_sel_small_.push_back(static_cast<int>(h_sel_small_.size()));
  h_block_sel_mid_.push_back(static_cast<int>(h_sel_mid_.size()));
  h_block_sel_big_.push_back(static_cast<int>(h_sel_big_.size()));
  d_sel_small_.ensure(h_sel_small_.size() + 1);
  d_sel_mid_.ensure(h_sel_mid_.size() + 1);
  d_sel_big_.ensure(h_sel_big_.size() + 1);
  if (!h_sel_mid_.empty()) {
    CheckCuda(cudaMemcpyAsync(d_sel_mid_.p, h_sel_mid_.data(), sizeof(int) * h_sel_mid_.size(),
                              cudaMemcpyHostToDevice, stream_), "h2d select mid list");
  }
  if (!h_sel_small_.empty()) {
    CheckCuda(cudaMemcpyAsync(d_sel_small_.p, h_sel_small_.data(), sizeof(int) * h_sel_small_.size(),
                              cudaMemcpyHostToDevice, stream_), "h2d select small list");
  }
  if (!h_sel_big_.empty()) {
    CheckCuda(cudaMemcpyAsync(d_sel_big_.p, h_sel_big_.data(), sizeof(int) * h_sel_big_.size(),
                              cudaMemcpyHostToDevice, stream_), "h2d select big list");
  }
  d_small_.ensure(h_small_.size() + 1);
  d_big_.ensure(h_big_.size() + 1);
  long long max_slots = 1;
  for (size_t b = 0; b + 1 < h_block_big_.size(); ++b) {
    max_slots = std::max(max_slots, h_soff_[static_cast<size_t>(h_block_big_[b + 1])] -
                                        h_soff_[static_cast<size_t>(h_block_big_[b])]);
  }
  d_soff_.ensure(h_soff_.size());
  CheckCuda(cudaMemcpyAsync(d_soff_.p, h_soff_.data(), sizeof(long long) * h_soff_.size(), cudaMemcpyHostToDevice,
                            stream_), "h2d soff");
  if (!h_small_.empty()) {
    CheckCuda(cudaMemcpyAsync(d_small_.p, h_small_.data(), sizeof(int) * h_small_.size(), cudaMemcpyHostToDevice,
                              stream_), "h2d small list");
  }
  d_big_moff_.ensure(h_big_moff_.size());
  if (!h_big_.empty()) {
    CheckCuda(cudaMemcpyAsync(d_big_.p, h_big_.data(), sizeof(int) * h_big_.size(), cudaMemcpyHostToDevice,
                              stream_), "h2d big list");
    CheckCuda(cudaMemcpyAsync(d_big_moff_.p, h_big_moff_.data(), sizeof(long long) * h_big_moff_.size(),
                              cudaMemcpyHostToDevice, stream_), "h2d big member offsets");
  }
  d_real_.ensure(R + 1);
  d_cand_off_.ensure(R + 1);
  d_sel_off_.ensure(R + 1);
  d_mat_off_.ensure(R + 1);
  if (R > 0) {
    CheckCuda(cudaMemcpyAsync(d_real_.p, h_real_.data(), sizeof(int) * R, cudaMemcpyHostToDevice, stream_),
              "h2d real");
    CheckCuda(cudaMemcpyAsync(d_cand_off_.p, h_cand_off_.data(), sizeof(long long) * (R + 1),
                              cudaMemcpyHostToDevice, stream_), "h2d cand_off");
    CheckCuda(cudaMemcpyAsync(d_sel_off_.p, h_sel_off_.data(), sizeof(long long) * (R + 1),
                              cudaMemcpyHostToDevice, stream_), "h2d sel_off");
    CheckCuda(cudaMemcpyAsync(d_mat_off_.p, h_mat_off_.data(), sizeof(long long) * (R + 1),
                              cudaMemcpyHostToDevice, stream_), "h2d mat_off");
  }
  SizeIterationBuffers(R, static_cast<size_t>(h_cand_off_[R]), static_cast<size_t>(h_sel_off_[R]), h_big_.size(),
                       max_mat, max_slots);
  plans_.clear();
  for (size_t b = 0; b + 1 < h_block_rg_.size(); ++b) {
    BlockPlan bp;
    bp.rg0 = h_block_rg_[b];
    bp.rg1 = h_block_rg_[b + 1];
    bp.slots = h_cand_off_[static_cast<size_t>(bp.rg1)] - h_cand_off_[static_cast<size_t>(bp.rg0)];
    bp.sel_slots = h_sel_off_[static_cast<size_t>(bp.rg1)] - h_sel_off_[static_cast<size_t>(bp.rg0)];
    bp.s0 = h_block_small_[b];
    bp.s1 = h_block_small_[b + 1];
    bp.b0 = h_block_big_[b];
    bp.b1 = h_block_big_[b + 1];
    bp.members = h_big_moff_[static_cast<size_t>(bp.b1)] - h_big_moff_[static_cast<size_t>(bp.b0)];
    bp.slot0 = h_soff_[static_cast<size_t>(bp.b0)];
    bp.nslots = h_soff_[static_cast<size_t>(bp.b1)] - bp.slot0;
    for (int i = bp.b0; i < bp.b1; ++i) {
      bp.max_e = std::max(bp.max_e, h_soff_[static_cast<size_t>(i) + 1] - h_soff_[static_cast<size_t>(i)]);
    }
    bp.mat_bytes = block_mat[b];
    bp.ss0 = h_block_sel_small_[b];
    bp.ss1 = h_block_sel_small_[b + 1];
    bp.sm0 = h_block_sel_mid_[b];
    bp.sm1 = h_block_sel_mid_[b + 1];
    bp.sb0 = h_block_sel_big_[b];
    bp.sb1 = h_block_sel_big_[b + 1];
    plans_.push_back(bp);
  }
}

// Buffers whose sizes follow from the plan's totals (either planner).
void Engine::SizeIterationBuffers(size_t R, size_t ncand, size_t nsel, size_t nbig, long long max_mat,
                                  long long max_slots) {
  d_bigdesc_.ensure(sizeof(BigDesc) * (nbig + 1));
  max_slots = std::max(max_slots, 1ll);
  for (int k = 0; k < 2; ++k) {
    d_skey_[k].ensure(static_cast<size_t>(max_slots));
    d_sval_[k].ensure(static_cast<size_t>(max_slots));
  }
  // radix-sort scratch of the deferred groups, sized once per iteration
  if (max_slots > 1) {
    size_t bytes = 0;
    CheckCuda(cub::DeviceRadixSort::SortPairs(nullptr, bytes, d_skey_[0].p, d_skey_[1].p, d_sval_[0].p,
                                              d_sval_[1].p, max_slots, 0, 64, stream_), "cub radix sort size");
    d_cub_tmp_.ensure(bytes);
  }
  d_cand_cnt_.ensure(R + 1);
  d_sel_cnt_.ensure(R + 1);
  d_cand_.ensure(ncand + 1);
  d_cand_rep_.ensure(ncand + 1);
  CheckCuda(cudaMemsetAsync(d_cand_rep_.p, 0xff, sizeof(int2) * (ncand + 1), stream_), "memset cand reps");
  d_res_.ensure(ncand + 1);
  if (cfg_.ranker) {
    d_cand_feat_.ensure(ncand + 1);
    d_rk_keep_.ensure(ncand + 1);
    d_rk_zbuf_.ensure(ncand + 1);
    for (int k = 0; k < 2; ++k) {
      d_rk_zpos_[k].ensure(static_cast<size_t>(RankerExploreCap(static_cast<long long>(ncand))));
      d_rk_zgain_[k].ensure(static_cast<size_t>(RankerExploreCap(static_cast<long long>(ncand))));
    }
  }
  rk_iter_slots_ = static_cast<long long>(ncand);
  d_sel_keep_.ensure(nsel + 1);
  d_sel_rem_.ensure(nsel + 1);
  d_sel_gain_.ensure(nsel + 1);
  d_mat_.ensure(static_cast<size_t>(max_mat) + 256);
}

// The plan of a one-block iteration, made on the device from the Divide
// output (the same lists and offsets as PrepareIterationBuffers); one small
// read-back brings the totals and the entry-pool top to the host.
void Engine::PlanOnDevice() {
  const long long G = n_groups_;
  const size_t cap = static_cast<size_t>(G) + 1;
  for (DevBuf<int>* b : {&d_real_, &d_small_, &d_big_, &d_sel_small_, &d_sel_mid_, &d_sel_big_}) b->ensure(cap);
  for (DevBuf<long long>* b : {&d_cand_off_, &d_sel_off_, &d_mat_off_, &d_big_moff_, &d_soff_}) b->ensure(cap);
  const int tiles = static_cast<int>((G + kPlanTile - 1) / kPlanTile);
  d_plan_tiles_.ensure(sizeof(PlanSums) * (2 * static_cast<size_t>(tiles) + 1));
  d_plan_scalars_.ensure(kPlanScalars);
  CheckCuda(cudaMemsetAsync(d_plan_scalars_.p, 0, sizeof(long long) * kPlanScalars, stream_), "memset plan");
  PlanParams P;
  P.glen = d_glen_.p;
  P.gent = d_gent_.p;
  P.G = G;
  P.top_k = cfg_.top_k > 0 ? cfg_.top_k : 1;
  P.tile_sums = reinterpret_cast<PlanSums*>(d_plan_tiles_.p);
  P.tile_off = P.tile_sums + tiles;
  P.tiles = tiles;
  P.scalars = d_plan_scalars_.p;
  P.real = d_real_.p;
  P.cand_off = d_cand_off_.p;
  P.sel_off = d_sel_off_.p;
  P.mat_off = d_mat_off_.p;
  P.small = d_small_.p;
  P.big = d_big_.p;
  P.big_moff = d_big_moff_.p;
  P.soff = d_soff_.p;
  P.sel_small = d_sel_small_.p;
  P.sel_mid = d_sel_mid_.p;
  P.sel_big = d_sel_big_.p;
  if (tiles > 0) {
    ++launches_;
    PlanTileKernel<<<tiles, kPlanThreads, 0, stream_>>>(P);
  }
  ++launches_;
  PlanScanKernel<<<1, kPlanThreads, 0, stream_>>>(P);
  if (tiles > 0) {
    ++launches_;
    PlanScatterKernel<<<tiles, kPlanThreads, 0, stream_>>>(P);
  }
  long long* hs = h_pin_.p + 16;
  CheckCuda(cudaMemcpyAsync(hs, d_plan_scalars_.p, sizeof(long long) * kPlanScalars, cudaMemcpyDeviceToHost,
                            stream_), "d2h plan");
  CheckCuda(cudaMemcpyAsync(hs + kPlanScalars, d_pool_top_.p, sizeof(long long), cudaMemcpyDeviceToHost, stream_),
            "d2h pool top");
  CheckCuda(cudaStreamSynchronize(stream_), "plan sync");
  CheckError();
  long long v[kPlanScalars + 1];
  std::memcpy(v, hs, sizeof(v));
  EnsurePoolRoom(static_cast<unsigned long long>(v[kPlanScalars]));
  const size_t R = static_cast<size_t>(v[kPlanR]);
  SizeIterationBuffers(R, static_cast<size_t>(v[kPlanCand]), static_cast<size_t>(v[kPlanSel]),
                       static_cast<size_t>(v[kPlanBig]), v[kPlanMat], v[kPlanSlots]);
  BlockPlan bp;
  bp.rg1 = static_cast<int>(R);
  bp.slots = v[kPlanCand];
  bp.sel_slots = v[kPlanSel];
  bp.s1 = static_cast<int>(v[kPlanSmall]);
  bp.b1 = static_cast<int>(v[kPlanBig]);
  bp.members = v[kPlanMembers];
  bp.nslots = v[kPlanSlots];
  bp.max_e = v[kPlanMaxE];
  bp.mat_bytes = v[kPlanMat];
  bp.ss1 = static_cast<int>(v[kPlanSelSmall]);
  bp.sm1 = static_cast<int>(v[kPlanSelMid]);
  bp.sb1 = static_cast<int>(v[kPlanSelBig]);
  plans_.assign(1, bp);
}

QuotientView Engine::View() {
  QuotientView Q;
  Q.ent = d_pool_[cur_pool_].p;
  Q.off = d_qoff_.p;
  Q.len = d_qlen_.p;
  Q.cap = d_qcap_.p;
  Q.size = d_qsize_.p;
  Q.internal = d_qint_.p;
  return Q;
}

void Engine::LaunchCommit(int rg0, int nrg, int64_t max_pairs, bool verify) {
  CommitParams C;
  C.Q = View();
  C.rg0 = rg0;
  C.nrg = nrg;
  C.sel_off = d_sel_off_.p;
  C.sel_keep = d_sel_keep_.p;
  C.sel_rem = d_sel_rem_.p;
  C.sel_gain = d_sel_gain_.p;
  C.sel_cnt = d_sel_cnt_.p;
  C.head = d_head_.p;
  C.next = d_next_.p;
  C.tail = d_tail_.p;
  C.fwd = d_fwd_.p;
  C.stamp = d_stamp_.p;
  C.partner = d_partner_.p;
  C.seq = d_seq_.p;
  C.claim = d_claim_.p;
  C.block_stamp = block_stamp_;
  C.pool_top = d_pool_top_.p;
  C.pool_cap = pool_cap_;
  C.scratch = d_scratch_.p;
  C.scratch_cap = d_scratch_.n;
  C.ctl = d_ctl_.p;
  C.stats = d_stats_.p;
  C.err = d_err_.p;
  C.rows_short = d_rows_short_.p;
  C.rows_long = d_rows_long_.p;
  C.ticket = d_rw_ticket_.p;
  C.sel_list = d_sel_list_.p;
  // warp-per-pair commit for short pairs, except in small blocks, where one
  // launch is cheaper than a second one
  C.warp_pairs = nrg > kFewGroups ? 1 : 0;
  if (verify) {
    const int vb = static_cast<int>(std::min<int64_t>((max_pairs + 7) / 8 + 1, 152 * 8));
    ++launches_;
    VerifyKernel<<<vb, 256, 0, stream_>>>(C);
  }
  const int grid = static_cast<int>(std::min<int64_t>(std::max<int64_t>(max_pairs, 1), kRowsGrid));
  BeginTimed(kTimeUpdate);
  ++launches_;
  // the warp kernel goes first: a pair it commits still reads as short to
  // CommitKernel (its keep row can only be short), which skips it; a long
  // pair is untouched until CommitKernel
  if (C.warp_pairs) {
    CommitShortKernel<<<static_cast<int>(std::min<int64_t>((max_pairs + 7) / 8 + 1, 152 * 8)), 256, 0, stream_>>>(C);
    ++launches_;
  }
  CommitKernel<<<grid, kRowsThreads, sizeof(RowsSmem), stream_>>>(C);
  ++launches_;
  RewriteRowsKernel<<<kRowsGrid, kRowsThreads, sizeof(RowsSmem), stream_>>>(C);
  EndTimed(kTimeUpdate);
}

// EA-proxy candidates for the small-group list entries [s0, s1) (one warp
// per group) and the big-group entries [b0, b1) (one CTA per group).
// Row sums for the scoring pass: in a large block of a one-block iteration
// (the prepare kernels write them while reading the member rows; scoring from
// them pays in a large block).
// Row sums are written by the block's own prepare kernels from its block-start
// state and read by its scoring pass only, so every block of more than
// kFewGroups groups uses them, one-block iterations or not.
bool Engine::RowSumsOn(const BlockPlan& bp) const { return bp.rg1 - bp.rg0 > kFewGroups; }

void Engine::LaunchPrepare(const BlockPlan& bp) {
  const int s0 = bp.s0, s1 = bp.s1, b0 = bp.b0, b1 = bp.b1;
  PrepareParams PP;
  PP.Q = View();
  PP.order = d_order_.p;
  PP.gstart = d_gstart_.p;
  PP.glen = d_glen_.p;
  PP.group_of = d_group_of_.p;
  PP.idx_in_group = d_idx_in_group_.p;
  PP.real = d_real_.p;
  PP.cand_off = d_cand_off_.p;
  PP.cand = d_cand_.p;
  PP.cand_cnt = d_cand_cnt_.p;
  PP.mat_off = d_mat_off_.p;
  PP.mat = d_mat_.p;
  PP.mat_zeroed = 0;
  PP.rc_before = nullptr;
  PP.rc_light = nullptr;
  PP.rc_heavy = nullptr;
  PP.rc_nheavy = nullptr;
  if (RowSumsOn(bp)) {
    d_rc_before_.ensure(static_cast<size_t>(n_));
    d_rc_light_.ensure(static_cast<size_t>(n_));
    d_rc_heavy_.ensure(static_cast<size_t>(n_));
    d_rc_nheavy_.ensure(static_cast<size_t>(n_));
    PP.rc_before = d_rc_before_.p;
    PP.rc_light = d_rc_light_.p;
    PP.rc_heavy = d_rc_heavy_.p;
    PP.rc_nheavy = d_rc_nheavy_.p;
  }
  PP.scratch = d_scratch_.p;
  PP.scratch_cap = d_scratch_.n;
  PP.ctl = d_ctl_.p;
  PP.top_k = cfg_.top_k;
  PP.stats = d_stats_.p;
  PP.err = d_err_.p;
  PP.cand_feat = cfg_.ranker ? d_cand_feat_.p : nullptr;
  PP.cand_rep = d_cand_rep_.p;
  BeginTimed(kTimePrepare);
  if (s1 > s0) {
    PP.list = d_small_.p;
    PP.list0 = s0;
    PP.nlist = s1 - s0;
    ++launches_;
    PrepareSmallKernel<<<(s1 - s0 + kSmallWarps - 1) / kSmallWarps, kSmallWarps * 32, sizeof(SmallSmem), stream_>>>(
        PP);
  }
  if (b1 > b0) {
    PP.list = d_big_.p;
    PP.list0 = b0;
    PP.nlist = b1 - b0;
    PP.moff = d_big_moff_.p;
    const long long members = bp.members;
    PP.desc = reinterpret_cast<BigDesc*>(d_bigdesc_.p);
    PP.soff = d_soff_.p;
    PP.slot0 = bp.slot0;
    PP.nslots = bp.nslots;
    if (bp.rg1 - bp.rg0 > kFewGroups && bp.mat_bytes > 0) {
      // one memset clears every pair table of a large block (a CTA clearing
      // its own group's tables is the tail of the kernel for large groups)
      CheckCuda(cudaMemsetAsync(d_mat_.p, 0, static_cast<size_t>(bp.mat_bytes), stream_), "memset pair tables");
      PP.mat_zeroed = 1;
    }
    PP.tbits = 1;
    while ((1ll << PP.tbits) < n_) ++PP.tbits;
    PP.skey = d_skey_[0].p;
    PP.sval = d_sval_[0].p;
    PP.skey_sorted = d_skey_[1].p;
    PP.sval_sorted = d_sval_[1].p;
    ++launches_;
    PrepareKernel<<<b1 - b0, kPrepThreads, sizeof(PrepSmem), stream_>>>(PP);
    if (PP.nslots > 0) {
      const long long windows = (PP.nslots + kFillWindow - 1) / kFillWindow;
      ++launches_;
      PrepareFillKernel<<<static_cast<int>(std::min(windows, 152ll * 32)), kFillThreads, 0, stream_>>>(PP);
      // key = launch-local group index << tbits | target; the group index
      // stays below 2^(bits - tbits) - 1, so no key has the padding's low bits
      int bits = PP.tbits;
      while ((1ll << (bits - PP.tbits)) <= b1 - b0) ++bits;
      size_t bytes = 0;
      CheckCuda(cub::DeviceRadixSort::SortPairs(nullptr, bytes, d_skey_[0].p, d_skey_[1].p, d_sval_[0].p,
                                                d_sval_[1].p, PP.nslots, 0, bits, stream_), "cub radix sort size");
      d_cub_tmp_.ensure(bytes);
      CheckCuda(cub::DeviceRadixSort::SortPairs(d_cub_tmp_.p, bytes, d_skey_[0].p, d_skey_[1].p, d_sval_[0].p,
                                                d_sval_[1].p, PP.nslots, 0, bits, stream_), "cub radix sort");
      const long long want = ((PP.nslots + 31) / 32 * kAccumSplit + kAccumThreads / 32 - 1) / (kAccumThreads / 32);
      ++launches_;
      PrepareAccumKernel<<<static_cast<int>(std::min<long long>(want, accum_grid_)), kAccumThreads, 0, stream_>>>(PP);
    }
    ++launches_;
    PrepareMembersKernel<<<static_cast<int>((members + 7) / 8), 256, 0, stream_>>>(PP);
    ++launches_;
    PrepareOutputKernel<<<b1 - b0, kPrepThreads, 0, stream_>>>(PP);
  }
  EndTimed(kTimePrepare);
}

void Engine::RunBlock(const BlockPlan& bp, double threshold, int iter, int total_iterations) {
  ++block_stamp_;
  ++hstats_.blocks;
  const int rg0 = bp.rg0;
  const int nrg = bp.rg1 - bp.rg0;
  const long long slots = bp.slots;
  const long long sel_slots = bp.sel_slots;
  // the block control words are zero: cleared by Merge before the first
  // block and by the previous block's rewrite kernel
  LaunchPrepare(bp);
  ScoreParams SP;
  SP.Q = View();
  SP.order = d_order_.p;
  SP.gstart = d_gstart_.p;
  SP.real = d_real_.p;
  SP.rg0 = rg0;
  SP.nrg = nrg;
  SP.cand_off = d_cand_off_.p;
  SP.cand = d_cand_.p;
  SP.cand_cnt = d_cand_cnt_.p;
  SP.cand_rep = d_cand_rep_.p;
  SP.ctl = d_ctl_.p;
  SP.res = d_res_.p;
  SP.stats = d_stats_.p;
  SP.err = d_err_.p;
  SP.threshold = threshold;
  SP.thr = SplitThreshold(threshold);
  SP.use_threshold = cfg_.ea_use_threshold ? 1 : 0;
  SP.audit = cfg_.ranker_audit ? 1 : 0;
  SP.phase = 0;
  SP.keep = d_rk_keep_.p;
  SP.zbuf = d_rk_zbuf_.p;
  SP.zpos = d_rk_zpos_[0].p;
  SP.zgain = d_rk_zgain_[0].p;
  SP.npos = d_rk_npos_.p;
  SP.zcap = 0;
  SP.cutoff = d_rk_cut_.p;
  SP.rc = RowConsts{nullptr, nullptr, nullptr, nullptr};
  if (RowSumsOn(bp)) {
    // written by this block's prepare kernels
    SP.rc = RowConsts{d_rc_before_.p, d_rc_light_.p, d_rc_heavy_.p, d_rc_nheavy_.p};
  }
  const int sgrid = static_cast<int>(
      std::min<long long>((slots + kScoreFetch * 8 - 1) / (kScoreFetch * 8), score_grid_));
  // learned ranker: trained after the logging iterations; afterwards the
  // exploration subset is scored first, then the rest above the cutoff
  const bool ranking = cfg_.ranker && rk_trained_ && iter > cfg_.ranker_train_iters;
  if (ranking) {
    RankerRank(rg0, nrg, slots, threshold, iter);
    SP.phase = 1;
    SP.zcap = static_cast<unsigned>(RankerExploreCap(slots));
    BeginTimed(kTimeScore);
    ++launches_;
    ScoreKernel<<<sgrid, kScoreThreads, 0, stream_>>>(SP);
    EndTimed(kTimeScore);
    RankerCutoff(slots);
    SP.phase = 2;
  }
  BeginTimed(kTimeScore);
  ++launches_;
  ScoreKernel<<<sgrid, kScoreThreads, 0, stream_>>>(SP);
  EndTimed(kTimeScore);
  if (cfg_.ranker && !rk_trained_ && iter <= cfg_.ranker_train_iters) {
    RankerLog(rg0, nrg, slots, iter, threshold, total_iterations);
  }
  SelectParams LP;
  LP.order = d_order_.p;
  LP.gstart = d_gstart_.p;
  LP.glen = d_glen_.p;
  LP.real = d_real_.p;
  LP.rg0 = rg0;
  LP.cand_off = d_cand_off_.p;
  LP.cand = d_cand_.p;
  LP.cand_cnt = d_cand_cnt_.p;
  LP.res = d_res_.p;
  LP.sel_off = d_sel_off_.p;
  LP.sel_keep = d_sel_keep_.p;
  LP.sel_rem = d_sel_rem_.p;
  LP.sel_gain = d_sel_gain_.p;
  LP.sel_cnt = d_sel_cnt_.p;
  LP.qlen = d_qlen_.p;
  LP.stamp = d_stamp_.p;
  LP.partner = d_partner_.p;
  LP.seq = d_seq_.p;
  LP.block_stamp = block_stamp_;
  LP.threshold = threshold;
  LP.thr = SplitThreshold(threshold);
  LP.use_threshold = cfg_.ea_use_threshold ? 1 : 0;
  LP.scratch = d_scratch_.p;
  LP.scratch_cap = d_scratch_.n;
  LP.ctl = d_ctl_.p;
  LP.stats = d_stats_.p;
  LP.err = d_err_.p;
  LP.sel_list = d_sel_list_.p;
  const int ss0 = bp.ss0, ss1 = bp.ss1;
  const int sb0 = bp.sb0, sb1 = bp.sb1;
  if (nrg <= kFewGroups) {
    // a small block: one launch, a CTA per group (same selection)
    LP.list = nullptr;
    LP.list0 = rg0;
    LP.nlist = nrg;
    ++launches_;
    SelectMatchKernel<<<nrg, kMatchThreads, 8 * kMatchSmemKeys, stream_>>>(LP);
    LaunchCommit(rg0, nrg, sel_slots, cfg_.verify_cuda_gain);
    return;
  }
  if (ss1 > ss0) {
    LP.list = d_sel_small_.p;
    LP.list0 = ss0;
    LP.nlist = ss1 - ss0;
    ++launches_;
    SelectSmallKernel<<<(ss1 - ss0 + kSelectSmallWarps - 1) / kSelectSmallWarps, kSelectSmallWarps * 32, 0,
                        stream_>>>(LP);
  }
  const int sm0 = bp.sm0, sm1 = bp.sm1;
  if (sm1 > sm0) {
    LP.list = d_sel_mid_.p;
    LP.list0 = sm0;
    LP.nlist = sm1 - sm0;
    ++launches_;
    SelectKernel<kSelectMidThreads, kSelectMidKeys><<<sm1 - sm0, kSelectMidThreads, 8 * kSelectMidKeys, stream_>>>(LP);
  }
  if (sb1 > sb0) {
    LP.list = d_sel_big_.p;
    LP.list0 = sb0;
    LP.nlist = sb1 - sb0;
    ++launches_;
    SelectMatchKernel<<<sb1 - sb0, kMatchThreads, 8 * kMatchSmemKeys, stream_>>>(LP);
  }
  LaunchCommit(rg0, nrg, sel_slots, cfg_.verify_cuda_gain);
}

void Engine::Merge(int iter, int total_iterations) {
  AllocScope alloc(stream_);
  if (n_groups_ < 0) throw std::runtime_error("Merge requires a preceding Divide");
  // ComputeMergeThreshold, reciprocal policy (src/sweg.cpp:400-406)
  const double threshold = 1.0 / static_cast<double>(iter + 1);
  if (plan_on_device_) {
    PlanOnDevice();
  } else {
    EnsurePoolRoom();
    PrepareIterationBuffers();
  }
  CheckCuda(cudaMemsetAsync(d_ctl_.p, 0, sizeof(BlockCtl), stream_), "memset ctl");
  for (const BlockPlan& bp : plans_) {
    if (bp.rg1 > bp.rg0) RunBlock(bp, threshold, iter, total_iterations);
  }
  ++launches_;
  RelabelKernel<<<(n_ + 255) / 256, 256, 0, stream_>>>(d_label_.p, d_fwd_.p, n_);
  n_groups_ = -1;  // the groups are consumed
  // accepted merges so far, read back with this synchronisation: the next
  // Divide knows the active count without a round trip of its own
  CheckCuda(cudaMemcpyAsync(h_pin_.p + 8, d_stats_.p + kStAccepted, sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, stream_), "d2h accepted");
  CheckCuda(cudaStreamSynchronize(stream_), "merge sync");
  CheckError();
  {
    unsigned long long accepted = 0;
    std::memcpy(&accepted, h_pin_.p + 8, sizeof(accepted));
    known_active_ = static_cast<int64_t>(n_) - static_cast<int64_t>(accepted);
  }
  if (cfg_.ranker && !rk_trained_ && iter == cfg_.ranker_train_iters) RankerTrain();
  if (cfg_.ranker && rk_trained_ && iter > cfg_.ranker_train_iters) RankerFinishIteration();
}

void Engine::ScorePairs(const int32_t* rep_a, const int32_t* rep_b, int64_t count, int64_t* gain,
                        int64_t* before) {
  AllocScope alloc(stream_);
  if (count <= 0) return;
  for (int64_t i = 0; i < count; ++i) {
    if (rep_a[i] < 0 || rep_a[i] >= n_ || rep_b[i] < 0 || rep_b[i] >= n_) {
      throw std::out_of_range("quotient supernode is out of range");
    }
  }
  DevBuf<int> da, db;
  DevBuf<longlong2> dr;
  da.ensure(static_cast<size_t>(count));
  db.ensure(static_cast<size_t>(count));
  dr.ensure(static_cast<size_t>(count));
  CheckCuda(cudaMemcpyAsync(da.p, rep_a, sizeof(int) * static_cast<size_t>(count), cudaMemcpyHostToDevice, stream_),
            "h2d pairs");
  CheckCuda(cudaMemcpyAsync(db.p, rep_b, sizeof(int) * static_cast<size_t>(count), cudaMemcpyHostToDevice, stream_),
            "h2d pairs");
  const int blocks = static_cast<int>(std::min<int64_t>((count + 7) / 8, 152 * 16));
  ++launches_;
  ScorePairsKernel<<<blocks, 256, 0, stream_>>>(View(), da.p, db.p, count, dr.p, d_err_.p);
  std::vector<longlong2> h(static_cast<size_t>(count));
  CheckCuda(cudaMemcpyAsync(h.data(), dr.p, sizeof(longlong2) * static_cast<size_t>(count), cudaMemcpyDeviceToHost,
                            stream_), "d2h results");
  CheckCuda(cudaStreamSynchronize(stream_), "score sync");
  da.release();
  db.release();
  dr.release();
  CheckError();
  for (int64_t i = 0; i < count; ++i) {
    gain[i] = h[static_cast<size_t>(i)].x;
    before[i] = h[static_cast<size_t>(i)].y;
  }
}

int64_t Engine::PrepareGroup(const int32_t* q, int g, int32_t* a_idx, int32_t* b_idx, int64_t cap) {
  AllocScope alloc(stream_);
  if (g < 0 || g > kMaxGroup) throw std::invalid_argument("group size out of range");
  std::vector<int> hq(q, q + g);
  for (int i = 0; i < g; ++i) {
    if (hq[static_cast<size_t>(i)] < 0 || hq[static_cast<size_t>(i)] >= n_) {
      throw std::out_of_range("quotient supernode is out of range");
    }
  }
  if (g < 2) return 0;
  // One explicit group; the Divide output is overwritten.
  n_groups_ = 1;
  h_glen_.assign(1, g);
  // the group's row entries (routing and deferred-group sort slots)
  {
    std::vector<int> lens(static_cast<size_t>(n_));
    CheckCuda(cudaMemcpyAsync(lens.data(), d_qlen_.p, sizeof(int) * static_cast<size_t>(n_), cudaMemcpyDeviceToHost,
                              stream_), "d2h row lengths");
    CheckCuda(cudaStreamSynchronize(stream_), "sync");
    unsigned e = 0;
    for (int i = 0; i < g; ++i) e += static_cast<unsigned>(lens[static_cast<size_t>(hq[static_cast<size_t>(i)])]);
    h_gent_.assign(1, e);
  }
  const int zero = 0;
  CheckCuda(cudaMemcpyAsync(d_order_.p, hq.data(), sizeof(int) * static_cast<size_t>(g), cudaMemcpyHostToDevice,
                            stream_), "h2d group");
  CheckCuda(cudaMemcpyAsync(d_gstart_.p, &zero, sizeof(int), cudaMemcpyHostToDevice, stream_), "h2d gstart");
  CheckCuda(cudaMemcpyAsync(d_glen_.p, &g, sizeof(int), cudaMemcpyHostToDevice, stream_), "h2d glen");
  std::vector<int> idx(static_cast<size_t>(g));
  for (int i = 0; i < g; ++i) idx[static_cast<size_t>(i)] = i;
  // group_of / idx_in_group for the members; every other rep must not match
  // group 0, so the array is first filled with -1.
  CheckCuda(cudaMemsetAsync(d_group_of_.p, 0xff, sizeof(int) * static_cast<size_t>(n_), stream_), "memset");
  DevBuf<int> dq, di;
  dq.ensure(static_cast<size_t>(g));
  di.ensure(static_cast<size_t>(g));
  CheckCuda(cudaMemcpyAsync(dq.p, hq.data(), sizeof(int) * static_cast<size_t>(g), cudaMemcpyHostToDevice, stream_),
            "h2d");
  CheckCuda(cudaMemcpyAsync(di.p, idx.data(), sizeof(int) * static_cast<size_t>(g), cudaMemcpyHostToDevice, stream_),
            "h2d");
  ++launches_;
  ScatterGroupKernel<<<(g + 255) / 256, 256, 0, stream_>>>(dq.p, di.p, g, d_group_of_.p, d_idx_in_group_.p);
  PrepareIterationBuffers();
  CheckCuda(cudaMemsetAsync(d_ctl_.p, 0, sizeof(BlockCtl), stream_), "memset ctl");
  LaunchPrepare(plans_.at(0));
  int cnt = 0;
  CheckCuda(cudaMemcpyAsync(&cnt, d_cand_cnt_.p, sizeof(int), cudaMemcpyDeviceToHost, stream_), "d2h");
  CheckCuda(cudaStreamSynchronize(stream_), "prepare sync");
  CheckError();
  std::vector<int2> h(static_cast<size_t>(cnt));
  if (cnt > 0) {
    CheckCuda(cudaMemcpy(h.data(), d_cand_.p, sizeof(int2) * static_cast<size_t>(cnt), cudaMemcpyDeviceToHost),
              "d2h cand");
  }
  for (int i = 0; i < cnt && i < cap; ++i) {
    a_idx[i] = h[static_cast<size_t>(i)].x;
    b_idx[i] = h[static_cast<size_t>(i)].y;
  }
  n_groups_ = -1;
  return cnt;
}

void Engine::MergePairs(const int32_t* keep, const int32_t* remove, int64_t count) {
  AllocScope alloc(stream_);
  if (count <= 0) return;
  known_active_ = -1;
  std::vector<char> seen(static_cast<size_t>(n_), 0);
  for (int64_t i = 0; i < count; ++i) {
    const int k = keep[i], r = remove[i];
    if (k < 0 || r < 0 || k >= n_ || r >= n_ || k == r) throw std::invalid_argument("invalid merge endpoints");
    if (seen[static_cast<size_t>(k)] || seen[static_cast<size_t>(r)]) {
      throw std::invalid_argument("merge batch requires endpoint-disjoint pairs");
    }
    seen[static_cast<size_t>(k)] = 1;
    seen[static_cast<size_t>(r)] = 1;
  }
  std::vector<int> hs(static_cast<size_t>(n_));
  CheckCuda(cudaMemcpy(hs.data(), d_qsize_.p, sizeof(int) * static_cast<size_t>(n_), cudaMemcpyDeviceToHost), "d2h");
  for (int64_t i = 0; i < count; ++i) {
    if (hs[static_cast<size_t>(keep[i])] <= 0 || hs[static_cast<size_t>(remove[i])] <= 0) {
      throw std::invalid_argument("quotient supernode is inactive");
    }
  }
  EnsurePoolRoom();
  // the batch is one pseudo-group's selection list
  const int cnt = static_cast<int>(count);
  h_sel_off_.assign(2, 0);
  h_sel_off_[1] = count;
  d_sel_off_.ensure(2);
  d_sel_cnt_.ensure(1);
  d_sel_keep_.ensure(static_cast<size_t>(count));
  d_sel_rem_.ensure(static_cast<size_t>(count));
  d_sel_gain_.ensure(static_cast<size_t>(count));
  CheckCuda(cudaMemcpyAsync(d_sel_off_.p, h_sel_off_.data(), 2 * sizeof(long long), cudaMemcpyHostToDevice, stream_),
            "h2d");
  CheckCuda(cudaMemcpyAsync(d_sel_cnt_.p, &cnt, sizeof(int), cudaMemcpyHostToDevice, stream_), "h2d");
  CheckCuda(cudaMemcpyAsync(d_sel_keep_.p, keep, sizeof(int) * static_cast<size_t>(count), cudaMemcpyHostToDevice,
                            stream_), "h2d");
  CheckCuda(cudaMemcpyAsync(d_sel_rem_.p, remove, sizeof(int) * static_cast<size_t>(count), cudaMemcpyHostToDevice,
                            stream_), "h2d");
  CheckCuda(cudaMemsetAsync(d_sel_gain_.p, 0, sizeof(long long) * static_cast<size_t>(count), stream_), "memset");
  ++block_stamp_;
  CheckCuda(cudaMemsetAsync(d_ctl_.p, 0, sizeof(BlockCtl), stream_), "memset ctl");
  ++launches_;
  MarkKernel<<<(cnt + 255) / 256, 256, 0, stream_>>>(d_sel_keep_.p, d_sel_rem_.p, cnt, d_stamp_.p, d_partner_.p,
                                                    d_seq_.p, block_stamp_, d_sel_list_.p, d_ctl_.p);
  LaunchCommit(0, 1, count, false);
  ++launches_;
  RelabelKernel<<<(n_ + 255) / 256, 256, 0, stream_>>>(d_label_.p, d_fwd_.p, n_);
  n_groups_ = -1;
  CheckCuda(cudaStreamSynchronize(stream_), "merge pairs sync");
  CheckError();
}

}  // namespace beam
