// CostOracle::ExactPartitionCost (src/cost_oracle.cpp:112-124) on the device:
// the encoding cost of the current partition, recomputed from the resident
// input graph rather than from the quotient graph. Every undirected edge
// {u, v} becomes the key (min(label u, label v), max(...)); a radix sort and
// a run-length encode give the edge count of every supernode pair, and each
// pair contributes BlockCost(size_a, size_b, count, a == b). The reference
// builds the same counts in a hash map; the sum is the same integer.
//
// The same counts also validate the resident quotient graph against a full
// rebuild (--validate-quotient).
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_run_length_encode.cuh>

#include <algorithm>
#include <cstring>

#include "engine.h"

namespace beam {
namespace {

constexpr unsigned long long kNoKey = ~0ull;

__global__ void PairKeysKernel(const int* __restrict__ arc_src, const int* __restrict__ col,
                               const int* __restrict__ label, long long arcs,
                               unsigned long long* __restrict__ keys) {
  for (long long k = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; k < arcs;
       k += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int u = arc_src[k];
    const int v = col[k];
    if (u >= v) {
      keys[k] = kNoKey;  // each undirected edge once (u < v)
      continue;
    }
    const unsigned a = static_cast<unsigned>(label[u]);
    const unsigned b = static_cast<unsigned>(label[v]);
    keys[k] = a < b ? (static_cast<unsigned long long>(a) << 32 | b) : (static_cast<unsigned long long>(b) << 32 | a);
  }
}

__global__ void PairCostKernel(const unsigned long long* __restrict__ uniq, const int* __restrict__ counts,
                               const int* __restrict__ nruns_p, const int* __restrict__ size,
                               unsigned long long* __restrict__ total, DevError* err) {
  const int nruns = *nruns_p;
  long long acc = 0;
  int bad = 0;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nruns; r += gridDim.x * blockDim.x) {
    const unsigned long long key = uniq[r];
    if (key == kNoKey) continue;
    const int a = static_cast<int>(key >> 32);
    const int b = static_cast<int>(key & 0xffffffffu);
    acc += BlockCost(size[a], size[b], counts[r], a == b, bad);
  }
  if (bad) RaiseError(err, kErrBlockCost, 0, 0, 0);
  acc = WarpSum(acc);
  if ((threadIdx.x & 31) == 0 && acc) atomicAdd(total, static_cast<unsigned long long>(acc));
}

// QuotientGraph::ValidateAgainstOriginalGraph (src/quotient_graph.cpp:867-886)
// on the device, over the run-length-encoded supernode-pair edge counts of the
// input graph: every pair count must be the entry of both rows (or the
// internal count for a == b), and each row must hold exactly as many entries
// as the rebuild has distinct neighbours. Mismatches are recorded as the
// smallest representative they concern.
__global__ void ValidatePairsKernel(const unsigned long long* __restrict__ uniq, const int* __restrict__ counts,
                                    const int* __restrict__ nruns_p, QuotientView Q, int* __restrict__ nbr_cnt,
                                    int* __restrict__ int_seen, int* __restrict__ bad_rep) {
  const int nruns = *nruns_p;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nruns; r += gridDim.x * blockDim.x) {
    const unsigned long long key = uniq[r];
    if (key == kNoKey) continue;
    const int a = static_cast<int>(key >> 32);
    const int b = static_cast<int>(key & 0xffffffffu);
    const long long c = counts[r];
    if (a == b) {
      int_seen[a] = 1;
      if (Q.size[a] == 0 || Q.internal[a] != c) atomicMin(bad_rep, a);
      continue;
    }
    atomicAdd(&nbr_cnt[a], 1);
    atomicAdd(&nbr_cnt[b], 1);
    if (Q.size[a] == 0 || RowLookup(Q.ent + Q.off[a], Q.len[a], b) != c) atomicMin(bad_rep, a);
    if (Q.size[b] == 0 || RowLookup(Q.ent + Q.off[b], Q.len[b], a) != c) atomicMin(bad_rep, b);
  }
}

// Per rep: row lengths against the distinct neighbours, internal counts of
// reps with no internal edge, inactive reps that still carry edges, and the
// quotient graph's own exact cost (QuotientGraph::ExactCost) from its rows.
__global__ void ValidateRepsKernel(int n, QuotientView Q, const int* __restrict__ nbr_cnt,
                                   const int* __restrict__ int_seen, int* __restrict__ bad_node,
                                   int* __restrict__ bad_rep, unsigned long long* __restrict__ qcost,
                                   DevError* err) {
  long long acc = 0;
  int bad = 0;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    if (Q.size[v] > 0) {
      if (Q.len[v] != nbr_cnt[v] || (!int_seen[v] && Q.internal[v] != 0)) atomicMin(bad_rep, v);
      const long long sv = Q.size[v];
      acc += BlockCost(sv, sv, Q.internal[v], true, bad);
      const Entry* row = Q.ent + Q.off[v];
      for (int k = 0; k < Q.len[v]; ++k) {
        const int x = EntNb(row[k]);
        if (x > v) acc += BlockCost(sv, Q.size[x], EntCnt(row[k]), false, bad);
      }
    } else if (nbr_cnt[v] != 0 || int_seen[v]) {
      atomicMin(bad_node, v);
    }
  }
  if (bad) RaiseError(err, kErrBlockCost, 0, 0, 0);
  acc = WarpSum(acc);
  if ((threadIdx.x & 31) == 0 && acc) atomicAdd(qcost, static_cast<unsigned long long>(acc));
}

__global__ void LabelSizesKernel(const int* __restrict__ label, int n, int* __restrict__ size_cnt) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    atomicAdd(&size_cnt[label[v]], 1);
  }
}

__global__ void SizesMatchKernel(const int* __restrict__ size_cnt, int n, const int* __restrict__ qsize,
                                 int* __restrict__ bad_node) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    if (size_cnt[v] != qsize[v]) atomicMin(bad_node, v);
  }
}

}  // namespace

void Engine::ValidateQuotient() {
  AllocScope alloc(stream_);
  const long long arcs = arcs_;
  cudaStream_t s = stream_;
  const size_t un = static_cast<size_t>(n_);
  d_pc_keys_[0].ensure(static_cast<size_t>(arcs) + 1);
  d_pc_keys_[1].ensure(static_cast<size_t>(arcs) + 1);
  d_pc_counts_.ensure(static_cast<size_t>(arcs) + 1);
  d_pc_scalars_.ensure(4);
  DevBuf<int> cnt;  // neighbour counts | internal seen | label sizes | 2 bad markers
  cnt.ensure(3 * un + 2);
  int* nbr_cnt = cnt.p;
  int* int_seen = cnt.p + un;
  int* size_cnt = cnt.p + 2 * un;
  int* bad = cnt.p + 3 * un;  // [0] node state, [1] row
  CheckCuda(cudaMemsetAsync(d_pc_scalars_.p, 0, 4 * sizeof(unsigned long long), s), "memset");
  CheckCuda(cudaMemsetAsync(cnt.p, 0, sizeof(int) * 3 * un, s), "memset");
  CheckCuda(cudaMemsetAsync(bad, 0x7f, 2 * sizeof(int), s), "memset");
  const int grid = static_cast<int>(std::min<long long>((std::max<long long>(arcs, n_) + 255) / 256, 152 * 16));
  int* nruns = reinterpret_cast<int*>(d_pc_scalars_.p + 1);
  if (arcs > 0) {
    ++launches_;
    PairKeysKernel<<<grid, 256, 0, s>>>(d_arc_src_.p, d_col_.p, d_label_.p, arcs, d_pc_keys_[0].p);
    size_t sort_bytes = 0, rle_bytes = 0;
    CheckCuda(cub::DeviceRadixSort::SortKeys(nullptr, sort_bytes, d_pc_keys_[0].p, d_pc_keys_[1].p, arcs, 0, 64, s),
              "cub sort size");
    CheckCuda(cub::DeviceRunLengthEncode::Encode(nullptr, rle_bytes, d_pc_keys_[1].p, d_pc_keys_[0].p,
                                                 d_pc_counts_.p, nruns, arcs, s), "cub rle size");
    d_cub_tmp_.ensure(std::max(sort_bytes, rle_bytes));
    CheckCuda(cub::DeviceRadixSort::SortKeys(d_cub_tmp_.p, sort_bytes, d_pc_keys_[0].p, d_pc_keys_[1].p, arcs, 0,
                                             64, s), "cub sort");
    CheckCuda(cub::DeviceRunLengthEncode::Encode(d_cub_tmp_.p, rle_bytes, d_pc_keys_[1].p, d_pc_keys_[0].p,
                                                 d_pc_counts_.p, nruns, arcs, s), "cub rle");
    ++launches_;
    ValidatePairsKernel<<<grid, 256, 0, s>>>(d_pc_keys_[0].p, d_pc_counts_.p, nruns, View(), nbr_cnt, int_seen,
                                             bad + 1);
    ++launches_;
    PairCostKernel<<<grid, 256, 0, s>>>(d_pc_keys_[0].p, d_pc_counts_.p, nruns, d_qsize_.p, d_pc_scalars_.p,
                                        d_err_.p);
  }
  ++launches_;
  LabelSizesKernel<<<grid, 256, 0, s>>>(d_label_.p, n_, size_cnt);
  ++launches_;
  SizesMatchKernel<<<grid, 256, 0, s>>>(size_cnt, n_, d_qsize_.p, bad);
  ++launches_;
  ValidateRepsKernel<<<grid, 256, 0, s>>>(n_, View(), nbr_cnt, int_seen, bad, bad + 1, d_pc_scalars_.p + 2,
                                          d_err_.p);
  int hb[2] = {0, 0};
  unsigned long long hc[3] = {0, 0, 0};
  CheckCuda(cudaMemcpyAsync(hb, bad, sizeof(hb), cudaMemcpyDeviceToHost, s), "d2h");
  CheckCuda(cudaMemcpyAsync(hc, d_pc_scalars_.p, sizeof(hc), cudaMemcpyDeviceToHost, s), "d2h");
  CheckCuda(cudaStreamSynchronize(s), "validate sync");
  CheckError();
  if (hb[0] != 0x7f7f7f7f) throw std::runtime_error("quotient node state differs from full rebuild");
  if (hb[1] != 0x7f7f7f7f) throw std::runtime_error("quotient row differs from full rebuild at " + std::to_string(hb[1]));
  if (hc[0] != hc[2]) throw std::runtime_error("quotient cost differs from CostOracle");
}

int64_t Engine::ExactPartitionCost() {
  AllocScope alloc(stream_);
  const long long arcs = arcs_;
  cudaStream_t s = stream_;
  d_pc_keys_[0].ensure(static_cast<size_t>(arcs) + 1);
  d_pc_keys_[1].ensure(static_cast<size_t>(arcs) + 1);
  d_pc_counts_.ensure(static_cast<size_t>(arcs) + 1);
  d_pc_scalars_.ensure(4);
  CheckCuda(cudaMemsetAsync(d_pc_scalars_.p, 0, 4 * sizeof(unsigned long long), s), "memset cost");
  const int grid = static_cast<int>(std::min<long long>((arcs + 255) / 256, 152 * 16));
  if (arcs > 0) {
    ++launches_;
    PairKeysKernel<<<grid, 256, 0, s>>>(d_arc_src_.p, d_col_.p, d_label_.p, arcs, d_pc_keys_[0].p);
    size_t sort_bytes = 0, rle_bytes = 0;
    int* nruns = reinterpret_cast<int*>(d_pc_scalars_.p + 1);
    CheckCuda(cub::DeviceRadixSort::SortKeys(nullptr, sort_bytes, d_pc_keys_[0].p, d_pc_keys_[1].p, arcs, 0, 64, s),
              "cub sort size");
    CheckCuda(cub::DeviceRunLengthEncode::Encode(nullptr, rle_bytes, d_pc_keys_[1].p, d_pc_keys_[0].p,
                                                 d_pc_counts_.p, nruns, arcs, s), "cub rle size");
    d_cub_tmp_.ensure(std::max(sort_bytes, rle_bytes));
    CheckCuda(cub::DeviceRadixSort::SortKeys(d_cub_tmp_.p, sort_bytes, d_pc_keys_[0].p, d_pc_keys_[1].p, arcs, 0,
                                             64, s), "cub sort");
    CheckCuda(cub::DeviceRunLengthEncode::Encode(d_cub_tmp_.p, rle_bytes, d_pc_keys_[1].p, d_pc_keys_[0].p,
                                                 d_pc_counts_.p, nruns, arcs, s), "cub rle");
    ++launches_;
    PairCostKernel<<<grid, 256, 0, s>>>(d_pc_keys_[0].p, d_pc_counts_.p, nruns, d_qsize_.p, d_pc_scalars_.p,
                                        d_err_.p);
  }
  unsigned long long total = 0;
  CheckCuda(cudaMemcpyAsync(h_pin_.p, d_pc_scalars_.p, sizeof(total), cudaMemcpyDeviceToHost, s), "d2h cost");
  CheckCuda(cudaStreamSynchronize(s), "cost sync");
  std::memcpy(&total, h_pin_.p, sizeof(total));
  CheckError();
  return static_cast<int64_t>(total);
}

}  // namespace beam
