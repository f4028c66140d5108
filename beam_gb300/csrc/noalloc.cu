// EA-proxy candidate generation for one group that allocates no memory.
//
// Who needs it: callers that must not allocate device memory themselves or
// through this library - code running inside a memory-pool-managed host that
// forbids cudaMalloc, code that may not add an allocation's implicit
// synchronisation to a latency-critical stream, or embedders that run the
// kernel inside their own pre-sized memory budget. They own the inputs and
// outputs; the kernel's scratch (the per-group pair tables and the target
// bucket table) lives in a fixed static device array instead of the engine's
// cudaMalloc'd scratch.
//
// Limits: at most kNoAllocMaxRows members, kNoAllocMaxEntries row entries in
// total and 1 <= top_k <= kNoAllocMaxTopK; other requests are rejected
// before anything is launched. Row weights must lie in [0, 2^32) (the kernel
// stages them as 32-bit words); the kernel's validation pass rejects others.
// The array (kNoAllocScratchBytes) is held by every GPU that loads the
// library until the process exits.
//
// Semantics are those of the engine's prepare step (PrepareBatchEncodingAware-
// GroupWithWorkspace, legacy EA-proxy branch, src/sweg.cpp:1800-1999): the
// same candidate pairs, (a_idx < b_idx) in ascending order.

#include <algorithm>
#include <cstdint>
#include <mutex>
#include <string>

#include "beam_gb300.h"
#include "common.cuh"

namespace beam {
namespace {

constexpr int kNoAllocMaxRows = 256;
constexpr int kNoAllocMaxEntries = 65536;
constexpr int kNoAllocMaxTopK = 32;
constexpr int kNoAllocThreads = 512;
constexpr int kNoAllocHeads = 2 * kNoAllocMaxEntries;
// status word | pair tables (P int64, ratio double, partner int32, flag u8 per
// member pair) | bucket heads | bucket entries (target, member, count, next)
constexpr size_t kNoAllocStatusBytes = 256;
constexpr size_t kNoAllocPairBytes = 21ull * kNoAllocMaxRows * kNoAllocMaxRows;
constexpr size_t kNoAllocHeadBytes = 4ull * kNoAllocHeads;
constexpr size_t kNoAllocEntryBytes = 16ull * kNoAllocMaxEntries;
constexpr size_t kNoAllocScratchBytes = kNoAllocStatusBytes + kNoAllocPairBytes + kNoAllocHeadBytes + kNoAllocEntryBytes;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

struct FlatKey {
  double ratio;
  long long pg;
  int lo, hi, j;
};

// ranked_better (src/sweg.cpp:1926-1938)
__device__ __forceinline__ bool FlatBetter(const FlatKey& x, const FlatKey& y) {
  if (x.ratio != y.ratio) return x.ratio > y.ratio;
  if (x.pg != y.pg) return x.pg > y.pg;
  if (x.lo != y.lo) return x.lo < y.lo;
  return x.hi < y.hi;
}

struct FlatArgs {
  const int* offsets;
  const int* reps;
  const int* nb;
  const long long* wt;
  const long long* nb_size;
  const long long* row_size;
  const long long* row_internal;
  int g;
  long long entries;
  int top_k;
  int* out_a;
  int* out_b;
  int* out_count;
};

__global__ void __launch_bounds__(kNoAllocThreads) PrepareFlatKernel(FlatArgs A, unsigned char* scratch) {
  __shared__ int s_rep[kNoAllocMaxRows];
  __shared__ int s_sorted_rep[kNoAllocMaxRows];
  __shared__ int s_sorted_idx[kNoAllocMaxRows];
  __shared__ long long s_old[kNoAllocMaxRows];
  __shared__ int s_rowcnt[kNoAllocMaxRows + 1];
  __shared__ int s_bad;
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const int nwarps = kNoAllocThreads / 32;
  const int g = A.g;
  int* status = reinterpret_cast<int*>(scratch);
  long long* pmat = reinterpret_cast<long long*>(scratch + kNoAllocStatusBytes);
  const long long gg = static_cast<long long>(g) * g;
  double* rmat = reinterpret_cast<double*>(pmat + gg);
  int* cmat = reinterpret_cast<int*>(rmat + gg);
  unsigned char* fmat = reinterpret_cast<unsigned char*>(cmat + gg);
  int* heads = reinterpret_cast<int*>(scratch + kNoAllocStatusBytes + kNoAllocPairBytes);
  int* et = reinterpret_cast<int*>(scratch + kNoAllocStatusBytes + kNoAllocPairBytes + kNoAllocHeadBytes);
  int* ei = et + kNoAllocMaxEntries;
  unsigned* ee = reinterpret_cast<unsigned*>(ei + kNoAllocMaxEntries);
  int* enx = reinterpret_cast<int*>(ee + kNoAllocMaxEntries);
  const unsigned hmask = kNoAllocHeads - 1;

  // s_bad bits: 1 = offsets, 2 = repeated reps, 4 = weight out of range
  if (tid == 0) {
    s_bad = (A.offsets[0] != 0 || static_cast<long long>(A.offsets[g]) != A.entries) ? 1 : 0;
    *status = 0;
  }
  for (int i = tid; i < g; i += kNoAllocThreads) s_rep[i] = A.reps[i];
  __syncthreads();
  for (int i = tid; i < g; i += kNoAllocThreads) {
    if (A.offsets[i] > A.offsets[i + 1] || A.offsets[i + 1] > A.entries) atomicOr(&s_bad, 1);
  }
  // counts are staged as 32-bit words: a weight outside [0, 2^32) is an error,
  // never a silently truncated count
  for (long long k = tid; k < A.entries; k += kNoAllocThreads) {
    const long long c = A.wt[k];
    if (c < 0 || c > static_cast<long long>(0xffffffffu)) atomicOr(&s_bad, 4);
  }
  // clear what must start at zero: every call reuses the same array
  for (long long k = tid; k < gg; k += kNoAllocThreads) {
    pmat[k] = 0;
    fmat[k] = 0;
  }
  for (int h = tid; h < kNoAllocHeads; h += kNoAllocThreads) heads[h] = -1;
  __syncthreads();
  if (s_bad) {
    if (tid == 0) {
      *status = (s_bad & 1) ? 1 : 3;
      *A.out_count = -1;
    }
    return;
  }
  // member lookup table: members sorted by rep (ranks; reps must be distinct)
  for (int i = tid; i < g; i += kNoAllocThreads) {
    int rank = 0;
    for (int j = 0; j < g; ++j) rank += s_rep[j] < s_rep[i] || (s_rep[j] == s_rep[i] && j < i);
    s_sorted_rep[rank] = s_rep[i];
    s_sorted_idx[rank] = i;
  }
  __syncthreads();
  for (int i = tid + 1; i < g; i += kNoAllocThreads) {
    if (s_sorted_rep[i] == s_sorted_rep[i - 1]) atomicOr(&s_bad, 2);
  }
  __syncthreads();
  if (s_bad) {
    if (tid == 0) {
      *status = 2;
      *A.out_count = -1;
    }
    return;
  }
  // approximate old costs, bucket entries, direct in-group edges
  for (int i = warp; i < g; i += nwarps) {
    const int rep = s_rep[i];
    const long long si = A.row_size[i];
    const int s = A.offsets[i];
    const int e = A.offsets[i + 1];
    long long old = 0;
    for (int k = s + lane; k < e; k += 32) {
      const int t = A.nb[k];
      const long long c = A.wt[k];
      old += EncodeCostForPair(rep, si, t, A.nb_size[k], c);
      et[k] = t;
      ei[k] = i;
      ee[k] = static_cast<unsigned>(c);
      enx[k] = atomicExch(&heads[(static_cast<unsigned>(t) * 0x9E3779B1u) >> 7 & hmask], k);
      int lo = 0, hi = g;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (s_sorted_rep[mid] < t) lo = mid + 1; else hi = mid;
      }
      if (lo < g && s_sorted_rep[lo] == t) {
        const int j = s_sorted_idx[lo];
        if (i < j) atomicAdd(reinterpret_cast<unsigned long long*>(&pmat[static_cast<long long>(i) * g + j]),
                             static_cast<unsigned long long>(c));
      }
    }
    old = WarpSum(old);
    if (lane == 0) {
      const long long internal = A.row_internal[i];
      if (internal > 0) old += EncodeCostForPair(rep, si, rep, si, 2 * internal);
      s_old[i] = old;
    }
  }
  __syncthreads();
  // every two members sharing a target: proxy += max(0, old - new)
  for (long long idx = tid; idx < A.entries; idx += kNoAllocThreads) {
    const int t = et[idx];
    const int i = ei[idx];
    const long long c = ee[idx];
    // the target's size is carried per entry; every entry of t carries the same
    for (int k = enx[idx]; k != -1; k = enx[k]) {
      if (et[k] != t) continue;
      const long long st = A.nb_size[k];
      const int j = ei[k];
      const int a = i < j ? i : j;
      const int b = i < j ? j : i;
      const long long ea = a == i ? c : static_cast<long long>(ee[k]);
      const long long eb = a == i ? static_cast<long long>(ee[k]) : c;
      const long long sa = A.row_size[a];
      const long long sb = A.row_size[b];
      const long long oldc = EncodeCostForPair(s_rep[a], sa, t, st, ea) + EncodeCostForPair(s_rep[b], sb, t, st, eb);
      const long long newc = EncodeCostForPair(s_rep[a], sa + sb, t, st, ea + eb);
      if (oldc - newc > 0) {
        atomicAdd(reinterpret_cast<unsigned long long*>(&pmat[static_cast<long long>(a) * g + b]),
                  static_cast<unsigned long long>(oldc - newc));
      }
    }
  }
  __syncthreads();
  for (long long idx = tid; idx < gg; idx += kNoAllocThreads) {
    const int i = static_cast<int>(idx / g);
    const int j = static_cast<int>(idx - static_cast<long long>(i) * g);
    if (j < i) pmat[idx] = pmat[static_cast<long long>(j) * g + i];
  }
  __syncthreads();
  // per member: positive partners ranked by ratio, the top_k kept (top_k >= 1
  // is checked by the host)
  const int top_k = A.top_k < g - 1 ? A.top_k : g - 1;
  for (int i = warp; i < g; i += nwarps) {
    const long long* prow = pmat + static_cast<long long>(i) * g;
    double* rrow = rmat + static_cast<long long>(i) * g;
    int* crow = cmat + static_cast<long long>(i) * g;
    int cnt = 0;
    for (int base = 0; base < g; base += 32) {
      const int j = base + lane;
      const long long pg = (j < g && j != i) ? prow[j] : 0;
      const unsigned ball = __ballot_sync(0xffffffffu, pg > 0);
      if (pg > 0) {
        const int pos = cnt + __popc(ball & ((1u << lane) - 1u));
        long long denom = s_old[i] + s_old[j];
        if (denom < 1) denom = 1;
        rrow[pos] = static_cast<double>(pg) / static_cast<double>(denom);
        crow[pos] = j;
      }
      cnt += __popc(ball);
    }
    __syncwarp();
    const int qi = s_rep[i];
    FlatKey lst[kNoAllocMaxTopK];
    int nl = 0;
    for (int c = lane; c < cnt; c += 32) {
      FlatKey k;
      k.j = crow[c];
      k.ratio = rrow[c];
      k.pg = prow[k.j];
      const int qj = s_rep[k.j];
      k.lo = qi < qj ? qi : qj;
      k.hi = qi < qj ? qj : qi;
      if (nl == top_k && !FlatBetter(k, lst[nl - 1])) continue;
      int pos = nl < top_k ? nl : top_k - 1;
      while (pos > 0 && FlatBetter(k, lst[pos - 1])) {
        lst[pos] = lst[pos - 1];
        --pos;
      }
      lst[pos] = k;
      if (nl < top_k) ++nl;
    }
    int head = 0;
    for (int r = 0; r < top_k; ++r) {
      FlatKey best;
      bool have = head < nl;
      if (have) best = lst[head];
      int src = lane;
      for (int o = 16; o > 0; o >>= 1) {
        FlatKey other;
        other.ratio = __shfl_xor_sync(0xffffffffu, best.ratio, o);
        other.pg = __shfl_xor_sync(0xffffffffu, best.pg, o);
        other.lo = __shfl_xor_sync(0xffffffffu, best.lo, o);
        other.hi = __shfl_xor_sync(0xffffffffu, best.hi, o);
        other.j = __shfl_xor_sync(0xffffffffu, best.j, o);
        const int osrc = __shfl_xor_sync(0xffffffffu, src, o);
        const int ohave = __shfl_xor_sync(0xffffffffu, have ? 1 : 0, o);
        if (ohave && (!have || FlatBetter(other, best))) {
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
  __syncthreads();
  // union of kept pairs in (a_idx, b_idx) order
  for (int a = warp; a < g; a += nwarps) {
    int cnt = 0;
    for (int base = a + 1; base < g; base += 32) {
      const int b = base + lane;
      cnt += __popc(__ballot_sync(0xffffffffu, b < g && fmat[static_cast<long long>(a) * g + b]));
    }
    if (lane == 0) s_rowcnt[a] = cnt;
  }
  __syncthreads();
  if (tid == 0) {
    int run = 0;
    for (int a = 0; a < g; ++a) {
      const int c = s_rowcnt[a];
      s_rowcnt[a] = run;
      run += c;
    }
    s_rowcnt[g] = run;
    *A.out_count = run;
  }
  __syncthreads();
  for (int a = warp; a < g; a += nwarps) {
    int pos = s_rowcnt[a];
    for (int base = a + 1; base < g; base += 32) {
      const int b = base + lane;
      const bool f = b < g && fmat[static_cast<long long>(a) * g + b];
      const unsigned ball = __ballot_sync(0xffffffffu, f);
      if (f) {
        const int at = pos + __popc(ball & ((1u << lane) - 1u));
        A.out_a[at] = a;
        A.out_b[at] = b;
      }
      pos += __popc(ball);
    }
  }
}

thread_local std::string g_noalloc_error;

// Device address of the static scratch array, looked up once per device.
std::mutex g_symbol_mutex;
void* g_symbol_addr[64] = {};

int Fail(const std::string& msg) {
  g_noalloc_error = msg;
  return -1;
}

}  // namespace
}  // namespace beam

extern "C" {

const char* beam_prepare_flat_noalloc_last_error(void) { return beam::g_noalloc_error.c_str(); }

int beam_prepare_flat_noalloc(const int32_t* offsets, const int32_t* row_rep_ids, const int32_t* neighbors,
                              const int64_t* weights, const int64_t* neighbor_sizes, const int64_t* row_sizes,
                              const int64_t* row_internal, int32_t rows, int64_t num_entries, int32_t top_k,
                              int32_t* out_a_idx, int32_t* out_b_idx, int64_t out_capacity, int32_t* out_count,
                              void* stream) {
  using namespace beam;
  if (rows < 0 || rows > kNoAllocMaxRows) {
    return Fail("rows=" + std::to_string(rows) + " exceeds the no-allocation limit of " +
                std::to_string(kNoAllocMaxRows) + " members per group");
  }
  if (num_entries < 0 || num_entries > kNoAllocMaxEntries) {
    return Fail("num_entries=" + std::to_string(num_entries) + " exceeds the no-allocation limit of " +
                std::to_string(kNoAllocMaxEntries) + " row entries");
  }
  if (top_k > kNoAllocMaxTopK) {
    return Fail("top_k=" + std::to_string(top_k) + " exceeds the no-allocation limit of " +
                std::to_string(kNoAllocMaxTopK));
  }
  if (top_k < 1) return Fail("top_k=" + std::to_string(top_k) + " must be at least 1");
  const long long g = rows;
  const long long k = top_k;
  const long long need = g >= 2 ? std::min(g * (g - 1) / 2, g * k) : 0;
  if (out_capacity < need) {
    return Fail("out_capacity=" + std::to_string(out_capacity) + " is below min(C(rows,2), rows*top_k)=" +
                std::to_string(need));
  }
  if (!out_count || (rows > 0 && (!offsets || !row_rep_ids || !row_sizes || !row_internal)) ||
      (num_entries > 0 && (!neighbors || !weights || !neighbor_sizes)) || (need > 0 && (!out_a_idx || !out_b_idx))) {
    return Fail("null device pointer");
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  {
    // the call reads its status back and waits for the stream: not a graph node
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    const cudaError_t cst = cudaStreamIsCapturing(s, &cap);
    if (cst != cudaSuccess) return Fail(std::string("cudaStreamIsCapturing: ") + cudaGetErrorString(cst));
    if (cap != cudaStreamCaptureStatusNone) {
      return Fail("the stream is capturing: the call waits for its stream and cannot be captured in a CUDA graph");
    }
  }
  if (rows < 2) {
    cudaError_t st = cudaMemsetAsync(out_count, 0, sizeof(int32_t), s);
    if (st == cudaSuccess) st = cudaStreamSynchronize(s);
    if (st != cudaSuccess) return Fail(std::string("cuda: ") + cudaGetErrorString(st));
    return 0;
  }
  int dev = 0;
  cudaError_t st = cudaGetDevice(&dev);
  if (st != cudaSuccess || dev < 0 || dev >= 64) return Fail(std::string("cudaGetDevice: ") + cudaGetErrorString(st));
  void* scratch = nullptr;
  {
    // first call on this device: look the array's device address up (the
    // array's name in host code is only a host-side stand-in)
    std::lock_guard<std::mutex> lock(g_symbol_mutex);
    if (!g_symbol_addr[dev]) {
      void* p = nullptr;
      st = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (st != cudaSuccess) return Fail(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(st));
      g_symbol_addr[dev] = p;
    }
    scratch = g_symbol_addr[dev];
  }
  FlatArgs A{offsets, row_rep_ids, neighbors, reinterpret_cast<const long long*>(weights),
             reinterpret_cast<const long long*>(neighbor_sizes), reinterpret_cast<const long long*>(row_sizes),
             reinterpret_cast<const long long*>(row_internal), rows, num_entries, top_k, out_a_idx, out_b_idx,
             out_count};
  PrepareFlatKernel<<<1, kNoAllocThreads, 0, s>>>(A, static_cast<unsigned char*>(scratch));
  st = cudaGetLastError();
  if (st != cudaSuccess) return Fail(std::string("kernel launch: ") + cudaGetErrorString(st));
  int status = 0;
  st = cudaMemcpyAsync(&status, scratch, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (st == cudaSuccess) st = cudaStreamSynchronize(s);
  if (st != cudaSuccess) return Fail(std::string("cuda: ") + cudaGetErrorString(st));
  if (status == 1) return Fail("offsets must rise from 0 to num_entries");
  if (status == 2) return Fail("row_rep_ids must be distinct");
  if (status == 3) return Fail("weights must lie in [0, 2^32): the kernel stages counts as 32-bit words");
  return 0;
}

}  // extern "C"
