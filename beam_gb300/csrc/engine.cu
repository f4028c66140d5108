// Engine lifecycle and the C ABI (include/beam_gb300.h).
//
// Device-resident state (HBM):
//   CSR            row_ptr int64[n+1], col int32[arcs], arc source int32[arcs]
//   quotient rows  one pool of packed (neighbour, count) entries, per rep an
//                  offset / length / capacity; a second pool of the same size
//                  is the target of compaction
//   supernodes     size int32[n] (0 = inactive), internal edges int64[n]
//   partition      label[node] (rep), head/next/tail member lists, fwd[rep]
// QuotientGraph::Initialize (src/quotient_graph.cpp:72-145) is InitRowsKernel:
// each node's sorted CSR row becomes its quotient row, repeated arcs summed.

#include <cub/device/device_reduce.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "beam_gb300.h"
#include "encode_write.h"
#include "engine.h"

namespace beam {

namespace {
thread_local cudaStream_t g_alloc_stream = nullptr;
std::mutex g_pool_mutex;
std::vector<int> g_pool_ready;  // devices whose default pool keeps freed memory
}  // namespace

cudaStream_t CurrentAllocStream() { return g_alloc_stream; }

AllocScope::AllocScope(cudaStream_t s) : prev_(g_alloc_stream) { g_alloc_stream = s; }
AllocScope::~AllocScope() { g_alloc_stream = prev_; }

void* DeviceAlloc(size_t bytes, cudaStream_t s) {
  void* p = nullptr;
  if (s == nullptr) {
    CheckCuda(cudaMalloc(&p, bytes), "cudaMalloc");
    return p;
  }
  int dev = 0;
  CheckCuda(cudaGetDevice(&dev), "cudaGetDevice");
  {
    std::lock_guard<std::mutex> lock(g_pool_mutex);
    if (std::find(g_pool_ready.begin(), g_pool_ready.end(), dev) == g_pool_ready.end()) {
      cudaMemPool_t pool;
      CheckCuda(cudaDeviceGetDefaultMemPool(&pool, dev), "default mem pool");
      uint64_t keep = UINT64_MAX;
      CheckCuda(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep), "mem pool threshold");
      g_pool_ready.push_back(dev);
    }
  }
  CheckCuda(cudaMallocAsync(&p, bytes, s), "cudaMallocAsync");
  return p;
}

void DeviceFree(void* p, cudaStream_t s) {
  if (s == nullptr) {
    cudaFree(p);
  } else {
    cudaFreeAsync(p, s);
  }
}

void CheckCuda(cudaError_t status, const char* what) {
  if (status != cudaSuccess) {
    throw std::runtime_error(std::string(what) + " failed: " + cudaGetErrorString(status));
  }
}

namespace {

__global__ void InitScalarsKernel(int n, int* qsize, long long* qint, int* label, int* head, int* next, int* tail,
                                  int* fwd, int* stamp, int* partner, int* claim, int* need) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= n) return;
  qsize[u] = 1;
  qint[u] = 0;
  label[u] = u;
  head[u] = u;
  next[u] = -1;
  tail[u] = u;
  fwd[u] = u;
  stamp[u] = 0;
  partner[u] = -1;
  claim[u] = 0;
  need[u] = 0;
}

// Warp per node: the sorted CSR row, runs of equal neighbours summed.
// Also validates the input: every neighbour in [0, n) and no self-loop.
__global__ void InitRowsKernel(const long long* __restrict__ rowptr, const int* __restrict__ col, int n,
                               Entry* __restrict__ pool, long long* __restrict__ qoff, int* __restrict__ qlen,
                               int* __restrict__ qcap, int* __restrict__ arc_src, DevError* err) {
  const int lane = threadIdx.x & 31;
  const long long warp = (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const long long nw = (static_cast<long long>(gridDim.x) * blockDim.x) >> 5;
  for (long long u = warp; u < n; u += nw) {
    const long long s = rowptr[u];
    const long long e = rowptr[u + 1];
    int rank = 0;
    for (long long k0 = s; k0 < e; k0 += 32) {
      const long long k = k0 + lane;
      bool first = false;
      int id = 0;
      if (k < e) {
        id = col[k];
        arc_src[k] = static_cast<int>(u);
        first = k == s || col[k - 1] != id;
        if (id < 0 || id >= n || id == u) RaiseError(err, kErrGraph, static_cast<int>(u), id, 0);
      }
      const unsigned ball = __ballot_sync(0xffffffffu, first);
      if (first) {
        long long c = 1;
        while (k + c < e && col[k + c] == id) ++c;
        pool[s + rank + __popc(ball & ((1u << lane) - 1u))] = MakeEnt(id, c);
      }
      rank += __popc(ball);
    }
    if (lane == 0) {
      qoff[u] = s;
      qlen[u] = rank;
      qcap[u] = static_cast<int>(e - s);
    }
  }
}

__global__ void LenToLongKernel(const int* __restrict__ len, const int* __restrict__ qsize, int n,
                                long long* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = qsize[i] > 0 ? len[i] : 0;
}

__global__ void CompactRowsKernel(const Entry* __restrict__ src, Entry* __restrict__ dst,
                                  const long long* __restrict__ new_off, long long* __restrict__ qoff,
                                  int* __restrict__ qlen, int* __restrict__ qcap, const int* __restrict__ qsize,
                                  int n) {
  const int lane = threadIdx.x & 31;
  const long long warp = (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const long long nw = (static_cast<long long>(gridDim.x) * blockDim.x) >> 5;
  for (long long u = warp; u < n; u += nw) {
    const int len = qsize[u] > 0 ? qlen[u] : 0;
    const Entry* s = src + qoff[u];
    Entry* d = dst + new_off[u];
    for (int k = lane; k < len; k += 32) d[k] = s[k];
    if (lane == 0) {
      qoff[u] = new_off[u];
      qlen[u] = len;
      qcap[u] = len;
    }
  }
}

thread_local std::string g_engine_error;

}  // namespace

Engine::Engine(int n, int64_t arcs, const int64_t* row_ptr, const int32_t* col_idx, const EngineConfig& cfg)
    : n_(n), arcs_(arcs), cfg_(cfg) {
  if (n <= 0) throw std::invalid_argument("Invalid node count.");
  if (arcs < 0 || row_ptr == nullptr || (arcs > 0 && col_idx == nullptr) || row_ptr[0] != 0 || row_ptr[n] != arcs) {
    throw std::invalid_argument("invalid CSR graph shape");
  }
  if (arcs / 2 >= (int64_t{1} << 32)) throw std::invalid_argument("graph too large for 32-bit edge counts");
  if (cfg_.divide_hash_dims <= 0) cfg_.divide_hash_dims = 16;
  if (cfg_.divide_max_group <= 0) cfg_.divide_max_group = 512;
  if (cfg_.divide_max_group > kMaxGroup) {
    throw std::invalid_argument("--divide-max-group above " + std::to_string(kMaxGroup) + " is not supported");
  }
  if (cfg_.group_batch_size < 1) cfg_.group_batch_size = 1;
  // neighbour range and self-loops are checked on the device (InitRowsKernel)
  CheckCuda(cudaSetDevice(cfg_.device), "cudaSetDevice");
  CheckCuda(cudaStreamCreateWithFlags(&owned_stream_.s, cudaStreamNonBlocking), "cudaStreamCreate");
  stream_ = owned_stream_.s;
  AllocScope alloc(stream_);
  const size_t un = static_cast<size_t>(n);
  d_rowptr_.ensure(un + 1);
  d_col_.ensure(static_cast<size_t>(arcs) + 1);
  d_arc_src_.ensure(static_cast<size_t>(arcs) + 1);
  CheckCuda(cudaMemcpyAsync(d_rowptr_.p, row_ptr, sizeof(long long) * (un + 1), cudaMemcpyHostToDevice, stream_),
            "h2d row_ptr");
  if (arcs > 0) {
    CheckCuda(cudaMemcpyAsync(d_col_.p, col_idx, sizeof(int) * static_cast<size_t>(arcs), cudaMemcpyHostToDevice,
                              stream_), "h2d col_idx");
  }
  pool_cap_ = 3 * static_cast<size_t>(arcs) + 2 * un + 4096;
  d_pool_[0].ensure(pool_cap_);
  d_pool_[1].ensure(pool_cap_);
  d_pool_top_.ensure(1);
  d_qoff_.ensure(un);
  d_qlen_.ensure(un);
  d_qcap_.ensure(un);
  d_qsize_.ensure(un);
  d_qint_.ensure(un);
  for (DevBuf<int>* b : {&d_label_, &d_head_, &d_next_, &d_tail_, &d_fwd_, &d_stamp_, &d_partner_, &d_claim_, &d_seq_,
                         &d_order_, &d_head_flag_, &d_vals_, &d_vals_alt_, &d_need_, &d_seg_beg_,
                         &d_seg_end_, &d_pos_map_, &d_gstart_, &d_glen_, &d_group_of_, &d_idx_in_group_,
                         &d_perm_, &d_perm_alt_, &d_segkey_, &d_segkey_alt_, &d_rows_short_, &d_rows_long_,
                         &d_sel_list_}) {
    b->ensure(un + 1);
  }
  d_hash_.ensure(un + 1);
  d_keys_.ensure(un + 1);
  d_keys_alt_.ensure(un + 1);
  d_ctl_.ensure(1);
  d_rw_ticket_.ensure(1);
  d_stats_.ensure(kStCount);
  d_err_.ensure(1);
  d_scratch_.ensure((static_cast<size_t>(64) << 20) + 32 * (static_cast<size_t>(arcs) + un));
  h_pin_.ensure(64);
  ConfigureKernels();
  Reset();
}

Engine::~Engine() {
  for (cudaEvent_t e : ev_pool_) cudaEventDestroy(e);
  for (cudaEvent_t e : step_ev_) {
    if (e) cudaEventDestroy(e);
  }
  d_flush_.release();
  if (stream_) cudaStreamSynchronize(stream_);
  for (auto* b : {&d_pool_[0], &d_pool_[1]}) b->release();
  d_rowptr_.release();
  d_col_.release();
  d_arc_src_.release();
  d_pool_top_.release();
  d_qoff_.release();
  d_qlen_.release();
  d_qcap_.release();
  d_qsize_.release();
  d_qint_.release();
  for (DevBuf<int>* b : {&d_label_, &d_head_, &d_next_, &d_tail_, &d_fwd_, &d_stamp_, &d_partner_, &d_claim_, &d_seq_,
                         &d_order_, &d_head_flag_, &d_vals_, &d_vals_alt_, &d_need_, &d_seg_beg_,
                         &d_seg_end_, &d_pos_map_, &d_gstart_, &d_glen_, &d_group_of_, &d_idx_in_group_,
                         &d_perm_, &d_perm_alt_, &d_segkey_, &d_segkey_alt_, &d_rows_short_, &d_rows_long_, &d_counts_, &d_cand_cnt_,
                         &d_sel_keep_, &d_sel_rem_, &d_real_,
                         &d_sel_cnt_}) {
    b->release();
  }
  d_hash_.release();
  d_keys_.release();
  d_keys_alt_.release();
  d_cub_tmp_.release();
  d_cand_off_.release();
  d_sel_off_.release();
  d_mat_off_.release();
  d_cand_.release();
  d_res_.release();
  d_sel_gain_.release();
  d_mat_.release();
  d_scratch_.release();
  d_ctl_.release();
  d_stats_.release();
  d_err_.release();
  h_pin_.release();
  // the stream itself goes with owned_stream_, after every member buffer
}

void Engine::Reset() {
  AllocScope alloc(stream_);
  const int T = 256;
  cur_pool_ = 0;
  ++launches_;
  InitScalarsKernel<<<(n_ + T - 1) / T, T, 0, stream_>>>(n_, d_qsize_.p, d_qint_.p, d_label_.p, d_head_.p,
                                                          d_next_.p, d_tail_.p, d_fwd_.p, d_stamp_.p, d_partner_.p,
                                                          d_claim_.p, d_need_.p);
  CheckCuda(cudaMemsetAsync(d_err_.p, 0, sizeof(DevError), stream_), "memset err");
  CheckCuda(cudaMemsetAsync(d_ctl_.p, 0, sizeof(BlockCtl), stream_), "memset ctl");
  CheckCuda(cudaMemsetAsync(d_rw_ticket_.p, 0, sizeof(unsigned), stream_), "memset ticket");
  ++launches_;
  InitRowsKernel<<<152 * 16, 256, 0, stream_>>>(d_rowptr_.p, d_col_.p, n_, d_pool_[0].p, d_qoff_.p, d_qlen_.p,
                                                d_qcap_.p, d_arc_src_.p, d_err_.p);
  const unsigned long long top = static_cast<unsigned long long>(arcs_);
  CheckCuda(cudaMemcpyAsync(d_pool_top_.p, &top, sizeof(top), cudaMemcpyHostToDevice, stream_), "h2d pool top");
  CheckCuda(cudaMemsetAsync(d_stats_.p, 0, sizeof(unsigned long long) * kStCount, stream_), "memset stats");
  CheckCuda(cudaStreamSynchronize(stream_), "reset sync");
  CheckError();
  block_stamp_ = 0;
  need_stamp_ = 0;
  n_groups_ = -1;
  n_active_ = n_;
  known_active_ = n_;
  hstats_ = HostStats{};
  RankerReset();
}

void Engine::CheckError() {
  DevError e;
  CheckCuda(cudaMemcpy(&e, d_err_.p, sizeof(e), cudaMemcpyDeviceToHost), "d2h error");
  if (e.code == kErrNone) return;
  std::string msg;
  switch (e.code) {
    case kErrBlockCost: msg = "edge count exceeds block capacity"; break;
    case kErrAsymmetric: msg = "asymmetric quotient edge count during scoring"; break;
    case kErrGroupTooLarge: msg = "group larger than the supported maximum"; break;
    case kErrScratch: msg = "per-block scratch memory exhausted"; break;
    case kErrPool: msg = "quotient entry pool exhausted"; break;
    case kErrValidation: msg = "commit-time exact gain differs from the scored gain"; break;
    case kErrKeyRange: msg = "merge gain outside the selection key range"; break;
    case kErrInactive: msg = "quotient supernode is inactive or endpoints are equal"; break;
    case kErrSlots: msg = "group row entries exceed their prepare sort slots"; break;
    case kErrGraph:
      msg = "QuotientGraph requires a loop-free graph with valid neighbors";
      CheckCuda(cudaMemset(d_err_.p, 0, sizeof(DevError)), "memset err");
      throw std::invalid_argument(msg);
    default: msg = "device error"; break;
  }
  msg += " (" + std::to_string(e.a) + ", " + std::to_string(e.b) + ", " + std::to_string(e.c) + ")";
  throw std::runtime_error(msg);
}

void Engine::EnsurePoolRoom() {
  unsigned long long top = 0;
  CheckCuda(cudaMemcpyAsync(h_pin_.p, d_pool_top_.p, sizeof(top), cudaMemcpyDeviceToHost, stream_), "d2h pool top");
  CheckCuda(cudaStreamSynchronize(stream_), "sync");
  std::memcpy(&top, h_pin_.p, sizeof(top));
  EnsurePoolRoom(top);
}

void Engine::EnsurePoolRoom(unsigned long long top) {
  // Keep rows of one iteration allocate at most the live entries plus one per
  // merge, so this much room guarantees no exhaustion inside the iteration.
  const size_t need = static_cast<size_t>(arcs_) + 2 * static_cast<size_t>(n_) + 1024;
  if (pool_cap_ - static_cast<size_t>(top) < need) CompactPool();
}

void Engine::CompactPool() {
  const int T = 256;
  DevBuf<long long> lens, offs;
  lens.ensure(static_cast<size_t>(n_) + 1);
  offs.ensure(static_cast<size_t>(n_) + 1);
  ++launches_;
  LenToLongKernel<<<(n_ + T - 1) / T, T, 0, stream_>>>(d_qlen_.p, d_qsize_.p, n_, lens.p);
  size_t bytes = 0;
  CheckCuda(cub::DeviceScan::ExclusiveSum(nullptr, bytes, lens.p, offs.p, n_ + 1, stream_), "scan size");
  d_cub_tmp_.ensure(bytes);
  CheckCuda(cudaMemsetAsync(lens.p + n_, 0, sizeof(long long), stream_), "memset");
  CheckCuda(cub::DeviceScan::ExclusiveSum(d_cub_tmp_.p, bytes, lens.p, offs.p, n_ + 1, stream_), "scan");
  const int dst = 1 - cur_pool_;
  ++launches_;
  CompactRowsKernel<<<152 * 16, 256, 0, stream_>>>(d_pool_[cur_pool_].p, d_pool_[dst].p, offs.p, d_qoff_.p,
                                                   d_qlen_.p, d_qcap_.p, d_qsize_.p, n_);
  CheckCuda(cudaMemcpyAsync(d_pool_top_.p, offs.p + n_, sizeof(long long), cudaMemcpyDeviceToDevice, stream_),
            "pool top");
  CheckCuda(cudaStreamSynchronize(stream_), "compact sync");
  cur_pool_ = dst;
  ++hstats_.compactions;
}

void Engine::Run(int iterations) {
  AllocScope alloc(stream_);
  using Clock = std::chrono::steady_clock;
  const auto t0 = Clock::now();
  for (int iter = 1; iter <= iterations; ++iter) {
    const auto d0 = Clock::now();
    Divide(iter);
    const auto d1 = Clock::now();
    Merge(iter, iterations);
    const auto d2 = Clock::now();
    hstats_.runtime_divide_ms += std::chrono::duration<double, std::milli>(d1 - d0).count();
    hstats_.runtime_merge_ms += std::chrono::duration<double, std::milli>(d2 - d1).count();
    ++hstats_.iterations;
  }
  hstats_.runtime_run_ms += std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
}

void Engine::Synchronize() { CheckCuda(cudaStreamSynchronize(stream_), "sync"); }

void Engine::Partition(int32_t* labels, int32_t* head, int32_t* next) {
  const size_t bytes = sizeof(int) * static_cast<size_t>(n_);
  if (labels) CheckCuda(cudaMemcpyAsync(labels, d_label_.p, bytes, cudaMemcpyDeviceToHost, stream_), "d2h labels");
  if (head) CheckCuda(cudaMemcpyAsync(head, d_head_.p, bytes, cudaMemcpyDeviceToHost, stream_), "d2h head");
  if (next) CheckCuda(cudaMemcpyAsync(next, d_next_.p, bytes, cudaMemcpyDeviceToHost, stream_), "d2h next");
  CheckCuda(cudaStreamSynchronize(stream_), "partition sync");
}

void Engine::Groups(int32_t* order, int32_t* starts, int32_t* lengths) {
  if (n_groups_ < 0) throw std::runtime_error("no groups: call Divide first");
  if (order) {
    CheckCuda(cudaMemcpyAsync(order, d_order_.p, sizeof(int) * static_cast<size_t>(n_active_), cudaMemcpyDeviceToHost,
                              stream_), "d2h order");
  }
  if (starts) {
    CheckCuda(cudaMemcpyAsync(starts, d_gstart_.p, sizeof(int) * static_cast<size_t>(n_groups_),
                              cudaMemcpyDeviceToHost, stream_), "d2h starts");
  }
  if (lengths) {
    CheckCuda(cudaMemcpyAsync(lengths, d_glen_.p, sizeof(int) * static_cast<size_t>(n_groups_),
                              cudaMemcpyDeviceToHost, stream_), "d2h lengths");
  }
  CheckCuda(cudaStreamSynchronize(stream_), "groups sync");
}

int64_t Engine::ExportRow(int rep, int32_t* nb, int64_t* cnt, int64_t cap, int64_t* size, int64_t* internal) {
  if (rep < 0 || rep >= n_) throw std::out_of_range("quotient supernode is out of range");
  long long off = 0, in = 0;
  int len = 0, sz = 0;
  CheckCuda(cudaMemcpy(&off, d_qoff_.p + rep, sizeof(off), cudaMemcpyDeviceToHost), "d2h");
  CheckCuda(cudaMemcpy(&len, d_qlen_.p + rep, sizeof(len), cudaMemcpyDeviceToHost), "d2h");
  CheckCuda(cudaMemcpy(&sz, d_qsize_.p + rep, sizeof(sz), cudaMemcpyDeviceToHost), "d2h");
  CheckCuda(cudaMemcpy(&in, d_qint_.p + rep, sizeof(in), cudaMemcpyDeviceToHost), "d2h");
  if (sz <= 0) len = 0;
  if (size) *size = sz;
  if (internal) *internal = in;
  if (len > 0 && cap > 0) {
    std::vector<Entry> h(static_cast<size_t>(len));
    CheckCuda(cudaMemcpy(h.data(), d_pool_[cur_pool_].p + off, sizeof(Entry) * static_cast<size_t>(len),
                         cudaMemcpyDeviceToHost), "d2h row");
    for (int k = 0; k < len && k < cap; ++k) {
      if (nb) nb[k] = EntNb(h[static_cast<size_t>(k)]);
      if (cnt) cnt[k] = EntCnt(h[static_cast<size_t>(k)]);
    }
  }
  return len;
}

void Engine::DeviceStats(uint64_t* out, int count) {
  std::vector<unsigned long long> h(kStCount);
  CheckCuda(cudaMemcpy(h.data(), d_stats_.p, sizeof(unsigned long long) * kStCount, cudaMemcpyDeviceToHost),
            "d2h stats");
  for (int i = 0; i < count && i < kStCount; ++i) out[i] = h[static_cast<size_t>(i)];
}

int64_t Engine::QuotientNnz() {
  AllocScope alloc(stream_);
  DevBuf<long long> lens, sum;
  const int T = 256;
  lens.ensure(static_cast<size_t>(n_));
  sum.ensure(1);
  ++launches_;
  LenToLongKernel<<<(n_ + T - 1) / T, T, 0, stream_>>>(d_qlen_.p, d_qsize_.p, n_, lens.p);
  size_t bytes = 0;
  CheckCuda(cub::DeviceReduce::Sum(nullptr, bytes, lens.p, sum.p, n_, stream_), "reduce size");
  d_cub_tmp_.ensure(bytes);
  CheckCuda(cub::DeviceReduce::Sum(d_cub_tmp_.p, bytes, lens.p, sum.p, n_, stream_), "reduce");
  long long cross = 0;
  CheckCuda(cudaMemcpyAsync(&cross, sum.p, sizeof(cross), cudaMemcpyDeviceToHost, stream_), "d2h");
  CheckCuda(cudaStreamSynchronize(stream_), "sync");
  // plus one virtual internal entry per active supernode with internal edges
  std::vector<long long> internal(static_cast<size_t>(n_));
  std::vector<int> sizes(static_cast<size_t>(n_));
  CheckCuda(cudaMemcpy(internal.data(), d_qint_.p, sizeof(long long) * static_cast<size_t>(n_),
                       cudaMemcpyDeviceToHost), "d2h");
  CheckCuda(cudaMemcpy(sizes.data(), d_qsize_.p, sizeof(int) * static_cast<size_t>(n_), cudaMemcpyDeviceToHost),
            "d2h");
  long long loops = 0;
  for (int i = 0; i < n_; ++i) loops += (sizes[static_cast<size_t>(i)] > 0 && internal[static_cast<size_t>(i)] > 0);
  return cross + loops;
}

void Engine::SetTimedKernel(int which) {
  timed_kind_ = which;
  timed_ms_accum_ = 0.0;
  timed_launches_ = 0;
  ev_used_ = 0;
}

void Engine::BeginTimed(int which) {
  if (which != timed_kind_ || timed_kind_ == kTimeNone) return;
  if (ev_used_ + 2 > ev_pool_.size()) {
    for (int i = 0; i < 256; ++i) {
      cudaEvent_t e;
      CheckCuda(cudaEventCreate(&e), "cudaEventCreate");
      ev_pool_.push_back(e);
    }
  }
  CheckCuda(cudaEventRecord(ev_pool_[ev_used_], stream_), "event record");
}

void Engine::EndTimed(int which) {
  if (which != timed_kind_ || timed_kind_ == kTimeNone) return;
  CheckCuda(cudaEventRecord(ev_pool_[ev_used_ + 1], stream_), "event record");
  ev_used_ += 2;
  ++timed_launches_;
}

void Engine::StepTimerStart() {
  for (cudaEvent_t& e : step_ev_) {
    if (!e) CheckCuda(cudaEventCreate(&e), "cudaEventCreate");
  }
  CheckCuda(cudaEventRecord(step_ev_[0], stream_), "event record");
}

double Engine::StepTimerStopMs() {
  CheckCuda(cudaEventRecord(step_ev_[1], stream_), "event record");
  CheckCuda(cudaEventSynchronize(step_ev_[1]), "event sync");
  float ms = 0.f;
  CheckCuda(cudaEventElapsedTime(&ms, step_ev_[0], step_ev_[1]), "event elapsed");
  return ms;
}

void Engine::FlushL2() {
  AllocScope alloc(stream_);
  const size_t bytes = static_cast<size_t>(256) << 20;  // twice the 129 MB L2 of a GB300
  d_flush_.ensure(bytes);
  CheckCuda(cudaMemsetAsync(d_flush_.p, static_cast<int>(launches_ & 0xff), bytes, stream_), "l2 flush");
  CheckCuda(cudaStreamSynchronize(stream_), "sync");
}

double Engine::TimedKernelMs() {
  CheckCuda(cudaStreamSynchronize(stream_), "sync");
  for (size_t i = 0; i + 1 < ev_used_; i += 2) {
    float ms = 0.f;
    CheckCuda(cudaEventElapsedTime(&ms, ev_pool_[i], ev_pool_[i + 1]), "event elapsed");
    timed_ms_accum_ += ms;
  }
  ev_used_ = 0;
  return timed_ms_accum_;
}

}  // namespace beam

// ------------------------------------------------------------------ C ABI

using beam::Engine;

struct beam_engine {
  Engine* impl;
};

namespace {

int Fail(const std::exception& e) {
  beam::g_engine_error = e.what();
  return -1;
}

template <typename F>
int Guard(F&& f) {
  try {
    f();
    return 0;
  } catch (const std::exception& e) {
    return Fail(e);
  }
}

}  // namespace

extern "C" {

const char* beam_engine_last_error(void) { return beam::g_engine_error.c_str(); }

void beam_engine_default_config(beam_engine_config* cfg) {
  cfg->top_k = 16;
  cfg->group_batch_size = 64;
  cfg->divide_hash_dims = 16;
  cfg->divide_max_group = 512;
  cfg->ea_use_threshold = 1;
  cfg->device = 0;
  cfg->seed = 1;
  cfg->verify_cuda_gain = 0;
  cfg->ranker = 0;
  cfg->ranker_train_iters = 5;
  cfg->ranker_recall = 0.99f;
  cfg->ranker_audit = 0;
  cfg->ranker_max_samples = 1 << 18;
  cfg->ranker_epochs = 4;
  cfg->ranker_max_steps = 256;
  cfg->ranker_lr = 3e-3f;
}

int beam_engine_create(int32_t n, int64_t arcs, const int64_t* row_ptr, const int32_t* col_idx,
                       const beam_engine_config* cfg, beam_engine** out) {
  return Guard([&] {
    if (out == nullptr) throw std::invalid_argument("out is NULL");
    *out = nullptr;
    beam::EngineConfig c;
    if (cfg) {
      c.top_k = cfg->top_k;
      c.group_batch_size = cfg->group_batch_size;
      c.divide_hash_dims = cfg->divide_hash_dims;
      c.divide_max_group = cfg->divide_max_group;
      c.ea_use_threshold = cfg->ea_use_threshold != 0;
      c.seed = cfg->seed;
      c.device = cfg->device;
      c.verify_cuda_gain = cfg->verify_cuda_gain != 0;
      c.ranker = cfg->ranker != 0;
      c.ranker_train_iters = cfg->ranker_train_iters;
      c.ranker_recall = cfg->ranker_recall;
      c.ranker_audit = cfg->ranker_audit != 0;
      c.ranker_max_samples = cfg->ranker_max_samples;
      c.ranker_epochs = cfg->ranker_epochs;
      c.ranker_max_steps = cfg->ranker_max_steps;
      c.ranker_lr = cfg->ranker_lr;
      if (c.ranker) {
        if (c.ranker_train_iters < 1) throw std::invalid_argument("ranker_train_iters must be >= 1");
        if (!(c.ranker_recall > 0.0f && c.ranker_recall <= 1.0f)) {
          throw std::invalid_argument("ranker_recall must be in (0, 1]");
        }
        if (c.ranker_max_samples < 1024 || c.ranker_max_samples > (1 << 24)) {
          throw std::invalid_argument("ranker_max_samples must be in [1024, 2^24]");
        }
        if (c.ranker_epochs < 1 || c.ranker_max_steps < 16 || c.ranker_max_steps > 1024) {
          throw std::invalid_argument("ranker_epochs >= 1 and ranker_max_steps in [16, 1024] required");
        }
        if (!(c.ranker_lr > 0.0f)) throw std::invalid_argument("ranker_lr must be positive");
      }
    }
    auto* e = new beam_engine{new Engine(n, arcs, row_ptr, col_idx, c)};
    *out = e;
  });
}

void beam_engine_destroy(beam_engine* e) {
  if (!e) return;
  delete e->impl;
  delete e;
}

int beam_engine_reset(beam_engine* e) { return Guard([&] { e->impl->Reset(); }); }
int beam_engine_run(beam_engine* e, int32_t iterations) { return Guard([&] { e->impl->Run(iterations); }); }
int beam_engine_divide(beam_engine* e, int32_t iter) { return Guard([&] { e->impl->Divide(iter); }); }
int beam_engine_merge(beam_engine* e, int32_t iter, int32_t total) {
  return Guard([&] { e->impl->Merge(iter, total); });
}

int beam_engine_group_counts(beam_engine* e, int64_t* n_active, int64_t* n_groups) {
  return Guard([&] {
    if (n_active) *n_active = e->impl->active_count();
    if (n_groups) *n_groups = e->impl->group_count();
  });
}

int beam_engine_groups(beam_engine* e, int32_t* order, int32_t* starts, int32_t* lengths) {
  return Guard([&] { e->impl->Groups(order, starts, lengths); });
}

int beam_engine_score_pairs(beam_engine* e, const int32_t* rep_a, const int32_t* rep_b, int64_t count,
                            int64_t* gain, int64_t* before) {
  return Guard([&] { e->impl->ScorePairs(rep_a, rep_b, count, gain, before); });
}

int beam_engine_prepare_group(beam_engine* e, const int32_t* q, int32_t g, int32_t* a_idx, int32_t* b_idx,
                              int64_t cap, int64_t* count) {
  return Guard([&] {
    const int64_t c = e->impl->PrepareGroup(q, g, a_idx, b_idx, cap);
    if (count) *count = c;
  });
}

int beam_engine_merge_pairs(beam_engine* e, const int32_t* keep, const int32_t* remove, int64_t count) {
  return Guard([&] { e->impl->MergePairs(keep, remove, count); });
}

int beam_engine_partition(beam_engine* e, int32_t* labels, int32_t* head, int32_t* next) {
  return Guard([&] { e->impl->Partition(labels, head, next); });
}

int beam_engine_export_row(beam_engine* e, int32_t rep, int32_t* nb, int64_t* cnt, int64_t cap, int64_t* len,
                           int64_t* size, int64_t* internal) {
  return Guard([&] {
    const int64_t l = e->impl->ExportRow(rep, nb, cnt, cap, size, internal);
    if (len) *len = l;
  });
}

int beam_engine_get_stats(beam_engine* e, beam_engine_stats* out) {
  return Guard([&] {
    uint64_t c[beam::kStCount];
    e->impl->DeviceStats(c, beam::kStCount);
    const beam::HostStats& h = e->impl->host_stats();
    std::memset(out, 0, sizeof(*out));
    out->runtime_run_ms = h.runtime_run_ms;
    out->runtime_divide_ms = h.runtime_divide_ms;
    out->runtime_merge_ms = h.runtime_merge_ms;
    out->merge_group_count = c[beam::kStGroupCount];
    out->merge_group_max_size = c[beam::kStGroupMaxSize];
    out->merge_raw_pair_count = c[beam::kStRawPairCount];
    out->merge_candidate_pairs_after_prune = c[beam::kStCandAfterPrune];
    out->candidate_proxy_pairs_examined = c[beam::kStProxyExamined];
    out->merge_exact_gain_calls = c[beam::kStExactCalls];
    out->exact_gain_input_nnz = c[beam::kStInputNnz];
    out->exact_raw_entries_a = c[beam::kStRawA];
    out->exact_raw_entries_b = c[beam::kStRawB];
    out->exact_union_neighbors = c[beam::kStUnion];
    out->exact_overlap_neighbors = c[beam::kStOverlap];
    out->merge_positive_gain_pairs = c[beam::kStPositive];
    out->merge_rejected_by_threshold = c[beam::kStRejThreshold];
    out->merge_rejected_by_overlap = c[beam::kStRejOverlap];
    out->merge_candidate_pairs = c[beam::kStCandPairs];
    out->merge_selected_pairs = c[beam::kStSelected];
    out->merge_total_local_gain = c[beam::kStLocalGain];
    out->selected_merges_for_validation = c[beam::kStValidationCalls];
    out->validation_exact_calls = c[beam::kStValidationCalls];
    out->validation_exact_row_entry_work = c[beam::kStValidationWork];
    out->accepted_merges_after_validation = c[beam::kStAccepted];
    out->rejected_nonpositive = c[beam::kStRejNonpositive];
    out->update_touched_quotient_entries = c[beam::kStTouched];
    out->isolated_gain_sum = c[beam::kStIsolatedGain];
    out->divide_max_group_size = c[beam::kStDivideMaxGroup];
    out->divide_fallback_splits = h.divide_fallback_splits;
    out->rows_rewritten = c[beam::kStRowsRewritten];
    out->row_entries_rewritten = c[beam::kStRowEntriesRewritten];
    out->score_bytes = c[beam::kStScoreBytes];
    out->prepare_bytes = c[beam::kStPrepareBytes];
    out->update_bytes = c[beam::kStUpdateBytes];
    out->divide_bytes = c[beam::kStDivideBytes];
    out->blocks = h.blocks;
    out->iterations = h.iterations;
    out->pool_compactions = h.compactions;
    out->active_supernodes = h.active_last;
    out->groups_last = h.groups_last;
  });
}

int beam_engine_ranker_info(beam_engine* e, beam_ranker_info* out) {
  return Guard([&] {
    uint64_t c[beam::kStCount];
    e->impl->DeviceStats(c, beam::kStCount);
    const beam::RankerInfo& r = e->impl->ranker_info();
    std::memset(out, 0, sizeof(*out));
    out->samples = r.samples;
    out->positives = r.positives;
    out->train_steps = r.train_steps;
    out->ranked = c[beam::kStRkRanked];
    out->pruned = c[beam::kStRkPruned];
    out->audit_passing = c[beam::kStRkAuditPassing];
    out->audit_lost = c[beam::kStRkAuditLost];
    out->train_ms = r.train_ms;
    out->first_loss = r.first_loss;
    out->final_loss = r.final_loss;
    out->cutoff = r.cutoff;
    out->calib_recall = r.calib_recall;
    out->calib_prune = r.calib_prune;
    out->trained = r.trained ? 1 : 0;
  });
}

int beam_engine_encode(beam_engine* e, const char* out_dir, beam_encoding* out) {
  return Guard([&] {
    const int n = e->impl->n();
    std::vector<int32_t> labels(static_cast<size_t>(n)), head(static_cast<size_t>(n)), next(static_cast<size_t>(n));
    e->impl->Partition(labels.data(), head.data(), next.data());
    beam::EncodeOutput enc;
    e->impl->Encode(&enc);
    beam::FinishEncoding(n, e->impl->arcs(), head.data(), next.data(), enc, out_dir, out);
  });
}

int beam_engine_exact_partition_cost(beam_engine* e, int64_t* cost) {
  return Guard([&] { *cost = e->impl->ExactPartitionCost(); });
}

int beam_engine_validate_quotient(beam_engine* e) {
  return Guard([&] { e->impl->ValidateQuotient(); });
}

int beam_engine_quotient_nnz(beam_engine* e, int64_t* nnz) {
  return Guard([&] { *nnz = e->impl->QuotientNnz(); });
}

int beam_engine_set_timed_kernel(beam_engine* e, int32_t which) {
  return Guard([&] { e->impl->SetTimedKernel(which); });
}

int beam_engine_timed_kernel(beam_engine* e, double* ms, int64_t* launches) {
  return Guard([&] {
    const double t = e->impl->TimedKernelMs();
    if (ms) *ms = t;
    if (launches) *launches = e->impl->TimedKernelLaunches();
  });
}

int beam_engine_synchronize(beam_engine* e) { return Guard([&] { e->impl->Synchronize(); }); }

int beam_engine_step_timer_start(beam_engine* e) { return Guard([&] { e->impl->StepTimerStart(); }); }

int beam_engine_step_timer_stop(beam_engine* e, double* ms) {
  return Guard([&] { *ms = e->impl->StepTimerStopMs(); });
}

int beam_engine_flush_l2(beam_engine* e) { return Guard([&] { e->impl->FlushL2(); }); }

int beam_engine_launch_count(beam_engine* e, int64_t* launches) {
  return Guard([&] { *launches = e->impl->launches(); });
}

}  // extern "C"

// include/cuda_scoring.hpp of the reference: C++ linkage, exact signatures.
const char* CudaScoringBuildMode() { return "cuda"; }
bool CudaScoringCompiled() { return true; }
