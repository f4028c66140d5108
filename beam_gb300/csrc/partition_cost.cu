// CostOracle::ExactPartitionCost (src/cost_oracle.cpp:112-124) on the device:
// the encoding cost of the current partition, recomputed from the resident
// input graph rather than from the quotient graph. Every undirected edge
// {u, v} becomes the key (min(label u, label v), max(...)); a radix sort and
// a run-length encode give the edge count of every supernode pair, and each
// pair contributes BlockCost(size_a, size_b, count, a == b). The reference
// builds the same counts in a hash map; the sum is the same integer.
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

}  // namespace

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
