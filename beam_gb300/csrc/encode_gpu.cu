// Sweg::Encode, mags-compatible branch (src/sweg.cpp:3017-3163), on the
// device for the engine's current partition:
//   supernode ids      active reps in ascending order (the reference's
//                      supernode numbering), node -> supernode
//   blocks             every edge {u, v} keyed by its supernode pair
//                      (smaller id first; u < v inside a supernode), a stable
//                      radix sort of the keys over the arcs in CSR order (so a
//                      block's edges stay in (u, v) order), run-length encode
//   decision           per block: corrections only (Cp: all its edges) when
//                      edges <= 1 + capacity - edges, else a superedge (P) and
//                      the block's missing member pairs (Cm)
//   Cm                 per dense block, every member pair is looked up among
//                      the block's sorted edges
// P comes out sorted; Cp and Cm are radix-sorted by (u, v). The host writes
// G.txt / P.txt / Cp.txt / Cm.txt with the same formatting as beam_encode.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_run_length_encode.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cstring>
#include <vector>

#include "encode_write.h"
#include "engine.h"

namespace beam {
namespace {

constexpr unsigned long long kNone = ~0ull;

__global__ void WidenKernel(const int* __restrict__ in, int count, long long* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) out[i] = in[i];
  if (i == count) out[i] = 0;
}

__global__ void LowHalfKernel(const unsigned long long* __restrict__ key, int count, int* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) out[i] = static_cast<int>(key[i] & 0xffffffffu);
}

__global__ void ActiveRepKernel(const int* __restrict__ size, int n, int* __restrict__ flag) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < n) flag[r] = size[r] > 0 ? 1 : 0;
}

// node -> supernode id, member keys (sid, node), sizes per supernode id
__global__ void NodeSidKernel(const int* __restrict__ label, const int* __restrict__ sid_of_rep,
                              const int* __restrict__ size, int n, int* __restrict__ nts,
                              unsigned long long* __restrict__ mkey, int* __restrict__ ssize) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  const int rep = label[v];
  const int s = sid_of_rep[rep];
  nts[v] = s;
  mkey[v] = static_cast<unsigned long long>(s) << 32 | static_cast<unsigned>(v);
  if (rep == v) ssize[s] = size[rep];
}

__global__ void ArcKeyKernel(const int* __restrict__ arc_src, const int* __restrict__ col,
                             const int* __restrict__ nts, long long arcs, unsigned long long* __restrict__ key,
                             int* __restrict__ val) {
  for (long long k = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; k < arcs;
       k += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int u = arc_src[k];
    const int v = col[k];
    const int su = nts[u];
    const int sv = nts[v];
    const bool keep = su < sv || (su == sv && u < v);
    key[k] = keep ? (static_cast<unsigned long long>(su) << 32 | static_cast<unsigned>(sv)) : kNone;
    val[k] = static_cast<int>(k);
  }
}

// per block: Cp count, Cm count, superedge flag
__global__ void BlockDecideKernel(const unsigned long long* __restrict__ uniq, const int* __restrict__ cnt,
                                  const int* __restrict__ nruns_p, const int* __restrict__ ssize,
                                  long long* __restrict__ cp_n, long long* __restrict__ cm_n,
                                  long long* __restrict__ p_n, int max_runs) {
  const int nruns = *nruns_p;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < max_runs; r += gridDim.x * blockDim.x) {
    long long cp = 0, cm = 0, p = 0;
    if (r < nruns && uniq[r] != kNone) {
      const int A = static_cast<int>(uniq[r] >> 32);
      const int B = static_cast<int>(uniq[r] & 0xffffffffu);
      const long long sa = ssize[A], sb = ssize[B];
      const long long cap = A == B ? sa * (sa - 1) / 2 : sa * sb;
      const long long real = cnt[r];
      if (real <= 1 + cap - real) {
        cp = real;
      } else {
        p = 1;
        cm = cap - real;
      }
    }
    cp_n[r] = cp;
    cm_n[r] = cm;
    p_n[r] = p;
  }
}

struct EmitParams {
  const unsigned long long* uniq;
  const int* cnt;
  const long long* run_off;  // exclusive scan of cnt
  const long long* cp_off;
  const long long* cm_off;
  const long long* p_off;
  const int* nruns;
  const int* arc_sorted;     // arc index per sorted position
  const int* arc_src;
  const int* col;
  const int* ssize;
  const long long* moff;     // member offsets per supernode id
  const int* members;        // nodes sorted by (supernode id, node)
  unsigned long long* P;     // (A << 32 | B)
  unsigned long long* Cp;    // (u << 32 | v)
  unsigned long long* Cm;
  unsigned* cm_fill;         // per dense block: pairs written
};

// one thread per sorted edge position; edges of sparse blocks go to Cp
__global__ void EmitSparseKernel(EmitParams E, long long positions) {
  const int nruns = *E.nruns;
  for (long long p = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; p < positions;
       p += static_cast<long long>(gridDim.x) * blockDim.x) {
    int lo = 0, hi = nruns;  // run of position p: last r with run_off[r] <= p
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (E.run_off[mid] <= p) lo = mid; else hi = mid;
    }
    const int r = lo;
    if (E.uniq[r] == kNone) continue;
    const long long base = E.cp_off[r];
    if (E.cp_off[r + 1] == base) continue;  // dense block
    const int k = E.arc_sorted[p];
    E.Cp[base + (p - E.run_off[r])] =
        static_cast<unsigned long long>(E.arc_src[k]) << 32 | static_cast<unsigned>(E.col[k]);
  }
}

__global__ void EmitDenseKernel(EmitParams E) {
  const int nruns = *E.nruns;
  for (int r = blockIdx.x; r < nruns; r += gridDim.x) {
    if (E.uniq[r] == kNone) continue;
    if (E.p_off[r + 1] == E.p_off[r]) continue;  // sparse block
    const int A = static_cast<int>(E.uniq[r] >> 32);
    const int B = static_cast<int>(E.uniq[r] & 0xffffffffu);
    if (threadIdx.x == 0) E.P[E.p_off[r]] = E.uniq[r];
    const long long sa = E.ssize[A], sb = E.ssize[B];
    const int* ma = E.members + E.moff[A];
    const int* mb = E.members + E.moff[B];
    const long long lo0 = E.run_off[r];
    const long long hi0 = lo0 + E.cnt[r];
    const long long cm_base = E.cm_off[r];
    for (long long t = threadIdx.x; t < sa * sb; t += blockDim.x) {
      const int u = ma[t / sb];
      const int v = mb[t % sb];
      if (A == B && u >= v) continue;
      long long lo = lo0, hi = hi0;
      while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        const int k = E.arc_sorted[mid];
        const int mu = E.arc_src[k];
        const int mv = E.col[k];
        if (mu < u || (mu == u && mv < v)) lo = mid + 1; else hi = mid;
      }
      bool present = false;
      if (lo < hi0) {
        const int k = E.arc_sorted[lo];
        present = E.arc_src[k] == u && E.col[k] == v;
      }
      if (!present) {
        const unsigned at = atomicAdd(&E.cm_fill[r], 1u);
        E.Cm[cm_base + at] = static_cast<unsigned long long>(u) << 32 | static_cast<unsigned>(v);
      }
    }
  }
}

}  // namespace

void Engine::Encode(EncodeOutput* out) {
  AllocScope alloc(stream_);
  const int n = n_;
  const long long arcs = arcs_;
  cudaStream_t s = stream_;
  const int T = 256;
  auto blocks = [&](long long items) { return static_cast<int>(std::min<long long>((items + T - 1) / T, 152 * 16)); };
  auto sort_pairs = [&](const unsigned long long* kin, unsigned long long* kout, const int* vin, int* vout,
                        long long items) {
    size_t bytes = 0;
    CheckCuda(cub::DeviceRadixSort::SortPairs(nullptr, bytes, kin, kout, vin, vout, items, 0, 64, s), "sort size");
    d_cub_tmp_.ensure(bytes);
    CheckCuda(cub::DeviceRadixSort::SortPairs(d_cub_tmp_.p, bytes, kin, kout, vin, vout, items, 0, 64, s), "sort");
  };
  auto sort_keys = [&](const unsigned long long* kin, unsigned long long* kout, long long items) {
    size_t bytes = 0;
    CheckCuda(cub::DeviceRadixSort::SortKeys(nullptr, bytes, kin, kout, items, 0, 64, s), "sort size");
    d_cub_tmp_.ensure(bytes);
    CheckCuda(cub::DeviceRadixSort::SortKeys(d_cub_tmp_.p, bytes, kin, kout, items, 0, 64, s), "sort");
  };
  auto scan_ll = [&](const long long* in, long long* outp, long long items) {
    size_t bytes = 0;
    CheckCuda(cub::DeviceScan::ExclusiveSum(nullptr, bytes, in, outp, items, s), "scan size");
    d_cub_tmp_.ensure(bytes);
    CheckCuda(cub::DeviceScan::ExclusiveSum(d_cub_tmp_.p, bytes, in, outp, items, s), "scan");
  };
  auto read_ll = [&](const long long* p) {
    CheckCuda(cudaMemcpyAsync(h_pin_.p, p, sizeof(long long), cudaMemcpyDeviceToHost, s), "d2h");
    CheckCuda(cudaStreamSynchronize(s), "sync");
    return h_pin_.p[0];
  };
  DevBuf<int> flag, sid_of_rep, nts, ssize, members, arc_val, arc_sorted, cnt;
  DevBuf<unsigned long long> mkey, mkey2, akey, akey2, uniq, P, Cp, Cp2, Cm, Cm2;
  DevBuf<long long> ll, moff, run_off, cp_n, cm_n, p_n, cp_off, cm_off, p_off;
  DevBuf<unsigned> cm_fill;
  const size_t un = static_cast<size_t>(n) + 1;
  const size_t ua = static_cast<size_t>(arcs) + 2;
  // supernode ids and member arrays
  flag.ensure(un);
  sid_of_rep.ensure(un);
  ll.ensure(un);
  ++launches_;
  ActiveRepKernel<<<(n + T - 1) / T, T, 0, s>>>(d_qsize_.p, n, flag.p);
  {
    size_t bytes = 0;
    CheckCuda(cub::DeviceScan::ExclusiveSum(nullptr, bytes, flag.p, sid_of_rep.p, n + 1, s), "scan size");
    d_cub_tmp_.ensure(bytes);
    CheckCuda(cudaMemsetAsync(flag.p + n, 0, sizeof(int), s), "memset");
    CheckCuda(cub::DeviceScan::ExclusiveSum(d_cub_tmp_.p, bytes, flag.p, sid_of_rep.p, n + 1, s), "scan");
  }
  CheckCuda(cudaMemcpyAsync(h_pin_.p, sid_of_rep.p + n, sizeof(int), cudaMemcpyDeviceToHost, s), "d2h");
  CheckCuda(cudaStreamSynchronize(s), "sync");
  int S = 0;
  std::memcpy(&S, h_pin_.p, sizeof(int));
  nts.ensure(un);
  ssize.ensure(static_cast<size_t>(S) + 1);
  mkey.ensure(un);
  mkey2.ensure(un);
  members.ensure(un);
  ++launches_;
  NodeSidKernel<<<(n + T - 1) / T, T, 0, s>>>(d_label_.p, sid_of_rep.p, d_qsize_.p, n, nts.p, mkey.p, ssize.p);
  sort_keys(mkey.p, mkey2.p, n);
  // member offsets: exclusive scan of the supernode sizes; members in
  // (supernode, node) order: the low halves of the sorted keys
  moff.ensure(static_cast<size_t>(S) + 1);
  {
    DevBuf<long long> sz64;
    sz64.ensure(static_cast<size_t>(S) + 1);
    ++launches_;
    WidenKernel<<<(S + T) / T, T, 0, s>>>(ssize.p, S, sz64.p);
    scan_ll(sz64.p, moff.p, S + 1);
  }
  ++launches_;
  LowHalfKernel<<<(n + T - 1) / T, T, 0, s>>>(mkey2.p, n, members.p);
  // blocks
  akey.ensure(ua);
  akey2.ensure(ua);
  arc_val.ensure(ua);
  arc_sorted.ensure(ua);
  uniq.ensure(ua);
  cnt.ensure(ua);
  ++launches_;
  ArcKeyKernel<<<blocks(arcs), T, 0, s>>>(d_arc_src_.p, d_col_.p, nts.p, arcs, akey.p, arc_val.p);
  sort_pairs(akey.p, akey2.p, arc_val.p, arc_sorted.p, arcs);
  int* nruns_d = reinterpret_cast<int*>(ll.p);
  {
    size_t bytes = 0;
    CheckCuda(cub::DeviceRunLengthEncode::Encode(nullptr, bytes, akey2.p, uniq.p, cnt.p, nruns_d, arcs, s),
              "rle size");
    d_cub_tmp_.ensure(bytes);
    CheckCuda(cub::DeviceRunLengthEncode::Encode(d_cub_tmp_.p, bytes, akey2.p, uniq.p, cnt.p, nruns_d, arcs, s),
              "rle");
  }
  CheckCuda(cudaMemcpyAsync(h_pin_.p, nruns_d, sizeof(int), cudaMemcpyDeviceToHost, s), "d2h");
  CheckCuda(cudaStreamSynchronize(s), "sync");
  int nruns = 0;
  std::memcpy(&nruns, h_pin_.p, sizeof(int));
  const size_t ur = static_cast<size_t>(nruns) + 1;
  run_off.ensure(ur);
  cp_n.ensure(ur);
  cm_n.ensure(ur);
  p_n.ensure(ur);
  cp_off.ensure(ur);
  cm_off.ensure(ur);
  p_off.ensure(ur);
  {
    DevBuf<long long> cnt64;
    cnt64.ensure(ur);
    ++launches_;
    WidenKernel<<<(nruns + T) / T, T, 0, s>>>(cnt.p, nruns, cnt64.p);
    scan_ll(cnt64.p, run_off.p, nruns + 1);
  }
  ++launches_;
  BlockDecideKernel<<<blocks(nruns + 1), T, 0, s>>>(uniq.p, cnt.p, nruns_d, ssize.p, cp_n.p, cm_n.p, p_n.p,
                                                    nruns + 1);
  scan_ll(cp_n.p, cp_off.p, nruns + 1);
  scan_ll(cm_n.p, cm_off.p, nruns + 1);
  scan_ll(p_n.p, p_off.p, nruns + 1);
  const long long ncp = read_ll(cp_off.p + nruns);
  const long long ncm = read_ll(cm_off.p + nruns);
  const long long np = read_ll(p_off.p + nruns);
  P.ensure(static_cast<size_t>(np) + 1);
  Cp.ensure(static_cast<size_t>(ncp) + 1);
  Cp2.ensure(static_cast<size_t>(ncp) + 1);
  Cm.ensure(static_cast<size_t>(ncm) + 1);
  Cm2.ensure(static_cast<size_t>(ncm) + 1);
  cm_fill.ensure(ur);
  CheckCuda(cudaMemsetAsync(cm_fill.p, 0, sizeof(unsigned) * ur, s), "memset");
  EmitParams E;
  E.uniq = uniq.p;
  E.cnt = cnt.p;
  E.run_off = run_off.p;
  E.cp_off = cp_off.p;
  E.cm_off = cm_off.p;
  E.p_off = p_off.p;
  E.nruns = nruns_d;
  E.arc_sorted = arc_sorted.p;
  E.arc_src = d_arc_src_.p;
  E.col = d_col_.p;
  E.ssize = ssize.p;
  E.moff = moff.p;
  E.members = members.p;
  E.P = P.p;
  E.Cp = Cp.p;
  E.Cm = Cm.p;
  E.cm_fill = cm_fill.p;
  ++launches_;
  EmitSparseKernel<<<blocks(arcs), T, 0, s>>>(E, arcs);
  ++launches_;
  EmitDenseKernel<<<152 * 8, T, 0, s>>>(E);
  if (ncp > 0) sort_keys(Cp.p, Cp2.p, ncp);
  if (ncm > 0) sort_keys(Cm.p, Cm2.p, ncm);
  out->supernodes = S;
  out->P.resize(static_cast<size_t>(np));
  out->Cp.resize(static_cast<size_t>(ncp));
  out->Cm.resize(static_cast<size_t>(ncm));
  if (np > 0) {
    CheckCuda(cudaMemcpyAsync(out->P.data(), P.p, sizeof(unsigned long long) * np, cudaMemcpyDeviceToHost, s),
              "d2h P");
  }
  if (ncp > 0) {
    CheckCuda(cudaMemcpyAsync(out->Cp.data(), Cp2.p, sizeof(unsigned long long) * ncp, cudaMemcpyDeviceToHost, s),
              "d2h Cp");
  }
  if (ncm > 0) {
    CheckCuda(cudaMemcpyAsync(out->Cm.data(), Cm2.p, sizeof(unsigned long long) * ncm, cudaMemcpyDeviceToHost, s),
              "d2h Cm");
  }
  CheckCuda(cudaStreamSynchronize(s), "encode sync");
  CheckError();
}

}  // namespace beam
