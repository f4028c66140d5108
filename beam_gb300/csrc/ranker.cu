// Learned candidate ranker: logging, training (forward, backward and Adam in
// this library's own kernels), per-iteration calibration and pruning. See
// ranker.cuh for the model and the features.
//
// Per 20-iteration run: in iterations 1..train_iters every candidate pair is
// scored exactly as in the plain method, and a hashed sample of (features,
// label) rows is logged, label = the pair would pass the loosest threshold of
// the run (exact gain > 0 and gain / before >= 1 / (iterations + 1)). The log
// is put in (iteration, slot) order and the MLP is trained on it (mini-batch
// Adam, class-weighted logistic loss, deterministic reductions). In every
// later iteration the ranker scores all candidates, a hashed exploration
// subset (1/16) is scored exactly first, and the logit cutoff is the one that
// keeps the requested recall of the subset's pairs passing the iteration's
// threshold filter, both of their number and of their exact gain (the merge
// objective: a few high-gain pairs weigh more than many marginal ones);
// candidates below it are not scored. Selection and commit only ever see
// exactly scored pairs.
#include <cuda_runtime.h>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "engine.h"
#include "ranker.cuh"

namespace beam {
namespace {

constexpr int kRkThreads = 256;    // samples per CTA of the gradient kernel
constexpr int kRkBatch = 32768;    // samples per training step
constexpr int kRkMaxEpochs = 16;
constexpr unsigned kRkExploreShift = 4;  // exploration subset: 1 / 2^4 of the candidates
constexpr int kRkNormCtas = 64;
constexpr int kRkSlotThreads = 256;
constexpr int kRkPartial = kRkParams + 1;  // gradient + loss per CTA
constexpr int kRkPad = kRkHidden + 1;      // padded rows: no bank conflicts
constexpr int kRkXPad = kRkFeat + 1;

struct RkGradSmem {
  float w[kRkParams + 3];
  float dh[kRkThreads * kRkPad];
  float hd[kRkThreads * kRkPad];
  float xs[kRkThreads * kRkXPad];
  float loss[kRkThreads];
};

struct RkGradParams {
  const float* x;        // raw features [n][16]
  const float* y;        // labels in {0, 1}
  const float* wt;       // per-sample weights (nullptr: pos_w for positives, 1 otherwise)
  long long n;           // samples available
  // sample order: position r of epoch e -> (perm_a[e] * r + perm_b[e]) mod n
  // (perm_a[e] coprime with n: a bijection per epoch); perm_a[0] == 0: identity
  unsigned long long perm_a[kRkMaxEpochs];
  unsigned long long perm_b[kRkMaxEpochs];
  long long first;       // position in the sample order of the batch's first sample
  int batch;             // samples in the batch
  float pos_w;
  const float* norm;     // mean[16] | 1/sd[16] (nullptr: features used as given)
  float* params;         // fp32 master parameters
  float* m;              // Adam moments
  float* v;
  __nv_bfloat16* wbf;    // bf16 weights (W1 | w2)
  float* partial;        // [CTAs][kRkPartial]
  unsigned* ticket;      // last-CTA counter, left at 0
  float* grad_out;       // gradient of the mean loss (nullptr: not written)
  float* loss_out;       // mean loss of the batch
  float* z_out;          // per-sample logits (nullptr: not written)
  int adam;              // 1: apply one Adam step
  float lr;
  float b1c;             // 1 - beta1^t
  float b2c;             // 1 - beta2^t
};

constexpr float kAdamB1 = 0.9f;
constexpr float kAdamB2 = 0.999f;
constexpr float kAdamEps = 1e-8f;

__device__ __forceinline__ bool RkIsWeight(int p) { return p < kRkB1 || (p >= kRkW2 && p < kRkB2); }
__device__ __forceinline__ int RkBf16Index(int p) { return p < kRkB1 ? p : kRkW1 + (p - kRkW2); }

// One mini-batch: forward, weighted logistic loss, backward per sample; the
// CTA reduces its samples' gradients in sample order, the last CTA to finish
// reduces the CTA partials in CTA order (deterministic) and applies Adam.
__global__ void __launch_bounds__(kRkThreads) RankerGradKernel(RkGradParams P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  RkGradSmem& S = *reinterpret_cast<RkGradSmem*>(smem_raw);
  __shared__ bool last;
  const int tid = threadIdx.x;
  for (int p = tid; p < kRkParams; p += kRkThreads) {
    const float v = P.params[p];
    S.w[p] = RkIsWeight(p) ? RkBf16Round(v) : v;
  }
  __syncthreads();
  const int li = blockIdx.x * kRkThreads + tid;
  const bool valid = li < P.batch;
  float x[kRkFeat];
  float y = 0.0f, wt = 0.0f;
  if (valid) {
    const long long pos = P.first + li;
    const long long r = pos % P.n;
    const int e = static_cast<int>((pos / P.n) % kRkMaxEpochs);
    const long long s = P.perm_a[0] == 0 ? r
                                         : static_cast<long long>((P.perm_a[e] * static_cast<unsigned long long>(r) +
                                                                   P.perm_b[e]) % static_cast<unsigned long long>(P.n));
#pragma unroll
    for (int f = 0; f < kRkFeat; ++f) {
      float v = P.x[s * kRkFeat + f];
      if (P.norm) v = (v - P.norm[f]) * P.norm[kRkFeat + f];
      x[f] = v;
    }
    y = P.y[s];
    wt = P.wt ? P.wt[s] : (y > 0.5f ? P.pos_w : 1.0f);
  } else {
#pragma unroll
    for (int f = 0; f < kRkFeat; ++f) x[f] = 0.0f;
  }
  float* hd = S.hd + tid * kRkPad;
  float* dh = S.dh + tid * kRkPad;
  float z = S.w[kRkB2];
  for (int j = 0; j < kRkHidden; ++j) {
    float a = S.w[kRkB1 + j];
#pragma unroll
    for (int f = 0; f < kRkFeat; ++f) a = fmaf(S.w[j * kRkFeat + f], x[f], a);
    const float h = fmaxf(a, 0.0f);
    hd[j] = h;
    z = fmaf(S.w[kRkW2 + j], h, z);
  }
  const float inv = 1.0f / static_cast<float>(P.batch);
  float loss = 0.0f, dz = 0.0f;
  if (valid) {
    const float pz = 1.0f / (1.0f + expf(-z));
    const float softplus = fmaxf(z, 0.0f) + log1pf(expf(-fabsf(z)));
    loss = wt * (softplus - y * z) * inv;
    dz = wt * (pz - y) * inv;
    if (P.z_out) P.z_out[li] = z;
  }
  for (int j = 0; j < kRkHidden; ++j) {
    const float h = hd[j];
    dh[j] = h > 0.0f ? dz * S.w[kRkW2 + j] : 0.0f;
    hd[j] = dz * h;
  }
#pragma unroll
  for (int f = 0; f < kRkFeat; ++f) S.xs[tid * kRkXPad + f] = x[f];
  S.xs[tid * kRkXPad + kRkFeat] = dz;
  S.loss[tid] = loss;
  __syncthreads();
  float* part = P.partial + static_cast<long long>(blockIdx.x) * kRkPartial;
  for (int p = tid; p < kRkPartial; p += kRkThreads) {
    float acc = 0.0f;
    if (p < kRkB1) {
      const int j = p / kRkFeat, f = p % kRkFeat;
      for (int t = 0; t < kRkThreads; ++t) acc = fmaf(S.dh[t * kRkPad + j], S.xs[t * kRkXPad + f], acc);
    } else if (p < kRkW2) {
      const int j = p - kRkB1;
      for (int t = 0; t < kRkThreads; ++t) acc += S.dh[t * kRkPad + j];
    } else if (p < kRkB2) {
      const int j = p - kRkW2;
      for (int t = 0; t < kRkThreads; ++t) acc += S.hd[t * kRkPad + j];
    } else if (p == kRkB2) {
      for (int t = 0; t < kRkThreads; ++t) acc += S.xs[t * kRkXPad + kRkFeat];
    } else {
      for (int t = 0; t < kRkThreads; ++t) acc += S.loss[t];
    }
    part[p] = acc;
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) last = atomicAdd(P.ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  for (int p = tid; p < kRkPartial; p += kRkThreads) {
    float g = 0.0f;
    for (unsigned c = 0; c < gridDim.x; ++c) g += __ldcg(P.partial + static_cast<long long>(c) * kRkPartial + p);
    if (p == kRkParams) {
      if (P.loss_out) *P.loss_out = g;
      continue;
    }
    if (P.grad_out) P.grad_out[p] = g;
    if (P.adam) {
      const float m = kAdamB1 * P.m[p] + (1.0f - kAdamB1) * g;
      const float v = kAdamB2 * P.v[p] + (1.0f - kAdamB2) * g * g;
      P.m[p] = m;
      P.v[p] = v;
      const float w = P.params[p] - P.lr * (m / P.b1c) / (sqrtf(v / P.b2c) + kAdamEps);
      P.params[p] = w;
      if (RkIsWeight(p)) P.wbf[RkBf16Index(p)] = __float2bfloat16_rn(w);
    }
  }
  if (tid == 0) *P.ticket = 0u;
}

// Feature mean and 1/sd over the log: per-thread double sums (each thread
// sees one feature), CTA partials, last CTA combines them in CTA order.
__global__ void __launch_bounds__(256) RankerNormKernel(const float* x, long long n, double* partial,
                                                        unsigned* ticket, float* norm) {
  __shared__ double s1[256], s2[256];
  __shared__ bool last;
  const int tid = threadIdx.x;
  const long long total = n * kRkFeat;
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;  // multiple of 16
  double a = 0.0, b = 0.0;
  for (long long e = static_cast<long long>(blockIdx.x) * blockDim.x + tid; e < total; e += stride) {
    const double v = x[e];
    a += v;
    b += v * v;
  }
  s1[tid] = a;
  s2[tid] = b;
  __syncthreads();
  if (tid < kRkFeat) {
    double sa = 0.0, sb = 0.0;
    for (int t = tid; t < 256; t += kRkFeat) {
      sa += s1[t];
      sb += s2[t];
    }
    partial[(static_cast<long long>(blockIdx.x) * kRkFeat + tid) * 2] = sa;
    partial[(static_cast<long long>(blockIdx.x) * kRkFeat + tid) * 2 + 1] = sb;
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  if (tid < kRkFeat) {
    double sa = 0.0, sb = 0.0;
    for (unsigned c = 0; c < gridDim.x; ++c) {
      sa += __ldcg(partial + (static_cast<long long>(c) * kRkFeat + tid) * 2);
      sb += __ldcg(partial + (static_cast<long long>(c) * kRkFeat + tid) * 2 + 1);
    }
    const double mean = n > 0 ? sa / static_cast<double>(n) : 0.0;
    double var = n > 0 ? sb / static_cast<double>(n) - mean * mean : 0.0;
    if (var < 0.0) var = 0.0;
    norm[tid] = static_cast<float>(mean);
    norm[kRkFeat + tid] = static_cast<float>(1.0 / sqrt(var + 1e-6));
  }
  if (tid == 0) *ticket = 0u;
}

__device__ __forceinline__ void RkLoadWeights(float* w, const __nv_bfloat16* wbf, const float* params) {
  for (int p = threadIdx.x; p < kRkParams; p += blockDim.x) {
    if (p < kRkB1) w[p] = __bfloat162float(wbf[p]);
    else if (p >= kRkW2 && p < kRkB2) w[p] = __bfloat162float(wbf[kRkW1 + (p - kRkW2)]);
    else w[p] = params[p];
  }
}

struct RkSlotParams {
  QuotientView Q;
  const int* order;
  const int* gstart;
  const int* glen;
  const int* real;
  int rg0;
  int nrg;
  const long long* cand_off;
  const int2* cand;
  const int* cand_cnt;
  const float2* cand_feat;  // proxy gain, proxy ratio
  float thr;
  // pruning
  const float* norm;
  const __nv_bfloat16* wbf;
  const float* params;
  unsigned char* keep;      // 0 pruned, 1 score (exploration), 2 score iff z >= *cutoff
  float* zbuf;              // per slot logit
  unsigned long long* key;  // log: sample order key (iteration, slot)
  // logging
  const longlong2* res;
  double label_thr;
  float* x_out;
  float* y_out;
  unsigned* count;          // [0] samples, [1] positives
  unsigned cap;
  unsigned rate24;  // sampling rate in 1/2^24
  unsigned long long seed;
  int iter;
  unsigned long long* stats;
};

// Shared part of the slot kernels: the pair of a candidate slot and its features.
__device__ __forceinline__ bool RkSlotFeatures(const RkSlotParams& P, long long slot, float* x) {
  const int ri = OwnerOfSlot(P.cand_off, P.rg0, P.rg0 + P.nrg, slot);
  const int p = static_cast<int>(slot - P.cand_off[ri]);
  if (p >= P.cand_cnt[ri]) return false;
  const int gid = P.real[ri];
  const int* q = P.order + P.gstart[gid];
  const int2 c = P.cand[slot];
  const float2 pf = P.cand_feat[slot];
  RankerFeatures(P.Q, q[c.x], q[c.y], P.glen[gid], pf.x, pf.y, P.thr, x);
  return true;
}

__device__ __forceinline__ unsigned long long RkSlotHash(unsigned long long seed, int iter, long long slot) {
  return SplitMix64(seed ^ (0x9e3779b97f4a7c15ull * static_cast<unsigned long long>(iter + 1)) ^
                    (0xd1b54a32d192ed03ull * static_cast<unsigned long long>(slot + 1)));
}

// Ranking iterations: the logit of every candidate slot of the block; a
// hashed 1/16 of the slots is the exploration subset, scored exactly first.
__global__ void __launch_bounds__(kRkSlotThreads) RankerRankKernel(RkSlotParams P) {
  __shared__ float w[kRkParams];
  RkLoadWeights(w, P.wbf, P.params);
  __syncthreads();
  const long long s0 = P.cand_off[P.rg0];
  const long long s1 = P.cand_off[P.rg0 + P.nrg];
  unsigned ranked = 0;
  for (long long slot = s0 + static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; slot < s1;
       slot += static_cast<long long>(gridDim.x) * blockDim.x) {
    float x[kRkFeat];
    if (!RkSlotFeatures(P, slot, x)) continue;
#pragma unroll
    for (int f = 0; f < kRkFeat; ++f) x[f] = (x[f] - P.norm[f]) * P.norm[kRkFeat + f];
    P.zbuf[slot] = RankerForward(w, x);
    const bool explore = (RkSlotHash(P.seed, P.iter, slot) >> (64 - kRkExploreShift)) == 0;
    P.keep[slot] = explore ? 1 : 2;
    ++ranked;
  }
  ranked = static_cast<unsigned>(WarpSumInt(static_cast<int>(ranked)));
  if ((threadIdx.x & 31) == 0 && ranked) atomicAdd(&P.stats[kStRkRanked], static_cast<unsigned long long>(ranked));
}

// Cutoff of the block from the exploration pairs that passed the threshold
// filter, sorted by logit with the inclusive prefix of their exact gains:
// pairs with a logit below sorted[k] are pruned, with k the largest index such
// that the pruned part holds at most (1 - recall) of the pairs AND at most
// (1 - recall) of their total gain. Too few of them: no pruning.
__global__ void RankerCutoffKernel(const float* zpos_sorted, const long long* gain_prefix, const unsigned* npos_p,
                                   unsigned cap, float recall, float* cutoff) {
  const unsigned npos = min(*npos_p, cap);
  if (npos < 8) {
    *cutoff = -3.0e38f;
    return;
  }
  const double miss = 1.0 - static_cast<double>(recall);
  unsigned k = static_cast<unsigned>(floor(miss * static_cast<double>(npos)));
  if (k >= npos) k = npos - 1;
  // largest k' <= k with gain_prefix[k' - 1] <= miss * total (prefix of no pair = 0)
  const double budget = miss * static_cast<double>(gain_prefix[npos - 1]);
  unsigned lo = 0, hi = k;
  while (lo < hi) {
    const unsigned mid = (lo + hi + 1) >> 1;
    if (static_cast<double>(gain_prefix[mid - 1]) <= budget) lo = mid; else hi = mid - 1;
  }
  *cutoff = zpos_sorted[lo];
}

// Logging iterations: a hashed sample of the block's scored slots with their
// labels, appended to the log until it is full.
__global__ void __launch_bounds__(kRkSlotThreads) RankerLogKernel(RkSlotParams P) {
  const long long s0 = P.cand_off[P.rg0];
  const long long s1 = P.cand_off[P.rg0 + P.nrg];
  for (long long slot = s0 + static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; slot < s1;
       slot += static_cast<long long>(gridDim.x) * blockDim.x) {
    if (static_cast<unsigned>(RkSlotHash(P.seed ^ 0x3c6ef372fe94f82bull, P.iter, slot) >> 40) >= P.rate24) continue;
    float x[kRkFeat];
    if (!RkSlotFeatures(P, slot, x)) continue;
    const unsigned idx = atomicAdd(P.count, 1u);
    if (idx >= P.cap) continue;
    const longlong2 r = P.res[slot];
    const bool pos = r.x > 0 && r.y > 0 && static_cast<double>(r.x) / static_cast<double>(r.y) >= P.label_thr;
#pragma unroll
    for (int f = 0; f < kRkFeat; ++f) P.x_out[static_cast<long long>(idx) * kRkFeat + f] = x[f];
    P.y_out[idx] = pos ? 1.0f : 0.0f;
    P.key[idx] = static_cast<unsigned long long>(P.iter) << 40 | static_cast<unsigned long long>(slot);
    if (pos) atomicAdd(P.count + 1, 1u);
  }
}

// The log in (iteration, slot) order: x / y gathered by the sorted index.
__global__ void RankerGatherKernel(const int* idx, long long n, const float* x, const float* y, float* xo,
                                   float* yo) {
  for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long s = idx[i];
#pragma unroll
    for (int f = 0; f < kRkFeat; ++f) xo[i * kRkFeat + f] = x[s * kRkFeat + f];
    yo[i] = y[s];
  }
}

__global__ void RankerIotaKernel(int* idx, long long n) {
  for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    idx[i] = static_cast<int>(i);
  }
}

uint64_t RkNext(uint64_t* state) {
  *state += 0x9e3779b97f4a7c15ull;
  return SplitMix64(*state - 0x9e3779b97f4a7c15ull);
}

float RkUniform(uint64_t* state) { return static_cast<float>(RkNext(state) >> 40) / 16777216.0f; }

void RkInitParams(uint64_t seed, std::vector<float>* p) {
  p->assign(kRkParams, 0.0f);
  uint64_t st = seed ^ 0x6a09e667f3bcc909ull;
  const float a1 = std::sqrt(6.0f / static_cast<float>(kRkFeat + kRkHidden));
  for (int i = 0; i < kRkW1; ++i) (*p)[static_cast<size_t>(i)] = (2.0f * RkUniform(&st) - 1.0f) * a1;
  const float a2 = std::sqrt(6.0f / static_cast<float>(kRkHidden + 1));
  for (int j = 0; j < kRkHidden; ++j) (*p)[static_cast<size_t>(kRkW2 + j)] = (2.0f * RkUniform(&st) - 1.0f) * a2;
}

size_t RkGradSmemBytes() { return sizeof(RkGradSmem); }

}  // namespace

void Engine::RankerReset() {
  rk_trained_ = false;
  rk_info_ = RankerInfo{};
  if (d_rk_count_.p) CheckCuda(cudaMemsetAsync(d_rk_count_.p, 0, 2 * sizeof(unsigned), stream_), "memset rk count");
}

void Engine::RankerEnsure() {
  if (d_rk_params_.p) return;
  const size_t cap = static_cast<size_t>(std::max(1024, cfg_.ranker_max_samples));
  d_rk_x_.ensure(cap * kRkFeat);
  d_rk_y_.ensure(cap);
  d_rk_x2_.ensure(cap * kRkFeat);
  d_rk_y2_.ensure(cap);
  d_rk_key_[0].ensure(cap);
  d_rk_key_[1].ensure(cap);
  d_rk_idx_[0].ensure(cap);
  d_rk_idx_[1].ensure(cap);
  d_rk_count_.ensure(2);
  d_rk_ticket_.ensure(2);
  d_rk_params_.ensure(kRkParams);
  d_rk_m_.ensure(kRkParams);
  d_rk_v_.ensure(kRkParams);
  d_rk_wbf_.ensure(kRkBf16);
  d_rk_norm_.ensure(2 * kRkFeat);
  d_rk_partial_.ensure(static_cast<size_t>(kRkBatch / kRkThreads) * kRkPartial);
  d_rk_npartial_.ensure(static_cast<size_t>(kRkNormCtas) * kRkFeat * 2);
  d_rk_loss_.ensure(1024);
  d_rk_npos_.ensure(1);
  d_rk_cut_.ensure(1);
  CheckCuda(cudaMemsetAsync(d_rk_count_.p, 0, 2 * sizeof(unsigned), stream_), "memset rk count");
  CheckCuda(cudaMemsetAsync(d_rk_ticket_.p, 0, 2 * sizeof(unsigned), stream_), "memset rk ticket");
  CheckCuda(cudaFuncSetAttribute(RankerGradKernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(RkGradSmemBytes())), "ranker smem attribute");
}

static RkSlotParams SlotParams(const QuotientView& Q, const int* order, const int* gstart, const int* glen,
                               const int* real, int rg0, int nrg, const long long* cand_off, const int2* cand,
                               const int* cand_cnt, const float2* cand_feat, float thr,
                               unsigned long long* stats) {
  RkSlotParams P;
  std::memset(&P, 0, sizeof(P));
  P.Q = Q;
  P.order = order;
  P.gstart = gstart;
  P.glen = glen;
  P.real = real;
  P.rg0 = rg0;
  P.nrg = nrg;
  P.cand_off = cand_off;
  P.cand = cand;
  P.cand_cnt = cand_cnt;
  P.cand_feat = cand_feat;
  P.thr = thr;
  P.stats = stats;
  return P;
}

void Engine::RankerLog(int rg0, int nrg, long long slots, int iter, double threshold, int total_iterations) {
  if (slots <= 0) return;
  RankerEnsure();
  RkSlotParams P = SlotParams(View(), d_order_.p, d_gstart_.p, d_glen_.p, d_real_.p, rg0, nrg, d_cand_off_.p,
                              d_cand_.p, d_cand_cnt_.p, d_cand_feat_.p, static_cast<float>(threshold), d_stats_.p);
  P.res = d_res_.p;
  P.label_thr = 1.0 / static_cast<double>(total_iterations + 1);
  P.x_out = d_rk_x_.p;
  P.y_out = d_rk_y_.p;
  P.key = d_rk_key_[0].p;
  P.count = d_rk_count_.p;
  P.cap = static_cast<unsigned>(cfg_.ranker_max_samples);
  // each logging iteration contributes at most about 0.9 cap / train_iters
  // samples (the slot capacity bounds the candidates), so the log does not
  // overflow and its content does not depend on the order of the appends
  const double want = 0.9 * static_cast<double>(cfg_.ranker_max_samples) / std::max(1, cfg_.ranker_train_iters);
  const double rate = std::min(1.0, want / static_cast<double>(std::max(1ll, rk_iter_slots_)));
  P.rate24 = static_cast<unsigned>(rate * 16777216.0);
  P.seed = cfg_.seed;
  P.iter = iter;
  const int grid = static_cast<int>(std::min<long long>((slots + kRkSlotThreads - 1) / kRkSlotThreads, 152 * 8));
  ++launches_;
  RankerLogKernel<<<grid, kRkSlotThreads, 0, stream_>>>(P);
}

void Engine::RankerRank(int rg0, int nrg, long long slots, double threshold, int iter) {
  RkSlotParams P = SlotParams(View(), d_order_.p, d_gstart_.p, d_glen_.p, d_real_.p, rg0, nrg, d_cand_off_.p,
                              d_cand_.p, d_cand_cnt_.p, d_cand_feat_.p, static_cast<float>(threshold), d_stats_.p);
  P.norm = d_rk_norm_.p;
  P.wbf = reinterpret_cast<const __nv_bfloat16*>(d_rk_wbf_.p);
  P.params = d_rk_params_.p;
  P.keep = d_rk_keep_.p;
  P.zbuf = d_rk_zbuf_.p;
  P.seed = cfg_.seed;
  P.iter = iter;
  const int grid = static_cast<int>(std::min<long long>((slots + kRkSlotThreads - 1) / kRkSlotThreads, 152 * 8));
  ++launches_;
  RankerRankKernel<<<grid, kRkSlotThreads, 0, stream_>>>(P);
  // exploration positives: cleared count, padding above any logit
  CheckCuda(cudaMemsetAsync(d_rk_npos_.p, 0, sizeof(unsigned), stream_), "memset npos");
  CheckCuda(cudaMemsetAsync(d_rk_zpos_[0].p, 0x7f, sizeof(float) * static_cast<size_t>(RankerExploreCap(slots)),
                            stream_), "memset zpos");
  CheckCuda(cudaMemsetAsync(d_rk_zgain_[0].p, 0, sizeof(long long) * static_cast<size_t>(RankerExploreCap(slots)),
                            stream_), "memset zgain");
}

long long Engine::RankerExploreCap(long long slots) const { return slots / 8 + 1024; }

void Engine::RankerCutoff(long long slots) {
  const long long cap = RankerExploreCap(slots);
  // logits ascending with their gains (the padding, above every logit with
  // gain 0, sorts last), then the inclusive prefix of the gains
  size_t sort_bytes = 0, scan_bytes = 0;
  CheckCuda(cub::DeviceRadixSort::SortPairs(nullptr, sort_bytes, d_rk_zpos_[0].p, d_rk_zpos_[1].p, d_rk_zgain_[0].p,
                                            d_rk_zgain_[1].p, cap, 0, 32, stream_), "cub sort size");
  CheckCuda(cub::DeviceScan::InclusiveSum(nullptr, scan_bytes, d_rk_zgain_[1].p, d_rk_zgain_[0].p, cap, stream_),
            "cub scan size");
  d_cub_tmp_.ensure(std::max(sort_bytes, scan_bytes));
  CheckCuda(cub::DeviceRadixSort::SortPairs(d_cub_tmp_.p, sort_bytes, d_rk_zpos_[0].p, d_rk_zpos_[1].p,
                                            d_rk_zgain_[0].p, d_rk_zgain_[1].p, cap, 0, 32, stream_), "cub sort");
  CheckCuda(cub::DeviceScan::InclusiveSum(d_cub_tmp_.p, scan_bytes, d_rk_zgain_[1].p, d_rk_zgain_[0].p, cap,
                                          stream_), "cub scan");
  ++launches_;
  RankerCutoffKernel<<<1, 1, 0, stream_>>>(d_rk_zpos_[1].p, d_rk_zgain_[0].p, d_rk_npos_.p, static_cast<unsigned>(cap),
                                           cfg_.ranker_recall, d_rk_cut_.p);
}

void Engine::RankerTrain() {
  RankerEnsure();
  const auto t0 = std::chrono::steady_clock::now();
  CheckCuda(cudaMemcpyAsync(h_pin_.p, d_rk_count_.p, 2 * sizeof(unsigned), cudaMemcpyDeviceToHost, stream_), "d2h");
  CheckCuda(cudaStreamSynchronize(stream_), "sync");
  unsigned counts[2];
  std::memcpy(counts, h_pin_.p, sizeof(counts));
  const long long n = std::min<long long>(counts[0], cfg_.ranker_max_samples);
  const long long npos = counts[1];
  rk_info_.samples = static_cast<uint64_t>(n);
  rk_info_.positives = static_cast<uint64_t>(npos);
  rk_trained_ = false;
  if (n < 256 || npos == 0 || npos >= n) return;
  // the log in (iteration, slot) order
  ++launches_;
  RankerIotaKernel<<<static_cast<int>(std::min<long long>((n + 255) / 256, 1024)), 256, 0, stream_>>>(
      d_rk_idx_[0].p, n);
  size_t bytes = 0;
  CheckCuda(cub::DeviceRadixSort::SortPairs(nullptr, bytes, d_rk_key_[0].p, d_rk_key_[1].p, d_rk_idx_[0].p,
                                            d_rk_idx_[1].p, n, 0, 64, stream_), "cub sort size");
  d_cub_tmp_.ensure(bytes);
  CheckCuda(cub::DeviceRadixSort::SortPairs(d_cub_tmp_.p, bytes, d_rk_key_[0].p, d_rk_key_[1].p, d_rk_idx_[0].p,
                                            d_rk_idx_[1].p, n, 0, 64, stream_), "cub sort");
  ++launches_;
  RankerGatherKernel<<<static_cast<int>(std::min<long long>((n + 255) / 256, 1024)), 256, 0, stream_>>>(
      d_rk_idx_[1].p, n, d_rk_x_.p, d_rk_y_.p, d_rk_x2_.p, d_rk_y2_.p);
  // feature standardisation
  ++launches_;
  RankerNormKernel<<<kRkNormCtas, 256, 0, stream_>>>(d_rk_x2_.p, n, d_rk_npartial_.p, d_rk_ticket_.p + 1,
                                                      d_rk_norm_.p);
  std::vector<float> p0;
  RkInitParams(cfg_.seed, &p0);
  CheckCuda(cudaMemcpyAsync(d_rk_params_.p, p0.data(), sizeof(float) * kRkParams, cudaMemcpyHostToDevice, stream_),
            "h2d params");
  CheckCuda(cudaMemsetAsync(d_rk_m_.p, 0, sizeof(float) * kRkParams, stream_), "memset m");
  CheckCuda(cudaMemsetAsync(d_rk_v_.p, 0, sizeof(float) * kRkParams, stream_), "memset v");
  std::vector<__nv_bfloat16> wb(kRkBf16);
  for (int p = 0; p < kRkW1; ++p) wb[static_cast<size_t>(p)] = __float2bfloat16_rn(p0[static_cast<size_t>(p)]);
  for (int j = 0; j < kRkHidden; ++j) {
    wb[static_cast<size_t>(kRkW1 + j)] = __float2bfloat16_rn(p0[static_cast<size_t>(kRkW2 + j)]);
  }
  CheckCuda(cudaMemcpyAsync(d_rk_wbf_.p, wb.data(), sizeof(__nv_bfloat16) * kRkBf16, cudaMemcpyHostToDevice,
                            stream_), "h2d bf16 weights");
  RkGradParams G;
  std::memset(&G, 0, sizeof(G));
  G.x = d_rk_x2_.p;
  G.y = d_rk_y2_.p;
  G.n = n;
  // per epoch an affine bijection of the sample positions (SplitMix64 stream)
  uint64_t st = cfg_.seed ^ 0xbb67ae8584caa73bull;
  for (int e = 0; e < kRkMaxEpochs; ++e) {
    uint64_t a = 1 + RkNext(&st) % static_cast<uint64_t>(n - 1);
    auto gcd = [](uint64_t u, uint64_t v) {
      while (v) {
        const uint64_t t = u % v;
        u = v;
        v = t;
      }
      return u;
    };
    while (gcd(a, static_cast<uint64_t>(n)) != 1) a = a + 1 < static_cast<uint64_t>(n) ? a + 1 : 1;
    G.perm_a[e] = a;
    G.perm_b[e] = RkNext(&st) % static_cast<uint64_t>(n);
  }
  G.batch = static_cast<int>(std::min<long long>(kRkBatch, n));
  G.pos_w = static_cast<float>(std::min(20.0, static_cast<double>(n - npos) / static_cast<double>(npos)));
  G.norm = d_rk_norm_.p;
  G.params = d_rk_params_.p;
  G.m = d_rk_m_.p;
  G.v = d_rk_v_.p;
  G.wbf = reinterpret_cast<__nv_bfloat16*>(d_rk_wbf_.p);
  G.partial = d_rk_partial_.p;
  G.ticket = d_rk_ticket_.p;
  G.adam = 1;
  G.lr = cfg_.ranker_lr;
  const long long epochs = std::min(cfg_.ranker_epochs, kRkMaxEpochs);
  const long long steps = std::max(16ll, std::min<long long>(cfg_.ranker_max_steps, (epochs * n + G.batch - 1) / G.batch));
  const int grid = (G.batch + kRkThreads - 1) / kRkThreads;
  double b1p = 1.0, b2p = 1.0;
  for (long long t = 0; t < steps; ++t) {
    b1p *= kAdamB1;
    b2p *= kAdamB2;
    G.first = t * G.batch;
    G.b1c = static_cast<float>(1.0 - b1p);
    G.b2c = static_cast<float>(1.0 - b2p);
    G.loss_out = d_rk_loss_.p + (t < 1024 ? t : 1023);
    ++launches_;
    RankerGradKernel<<<grid, kRkThreads, RkGradSmemBytes(), stream_>>>(G);
  }
  rk_info_.train_steps = static_cast<uint64_t>(steps);
  float* hl = reinterpret_cast<float*>(h_pin_.p);
  CheckCuda(cudaMemcpyAsync(hl, d_rk_loss_.p, sizeof(float), cudaMemcpyDeviceToHost, stream_), "d2h");
  CheckCuda(cudaMemcpyAsync(hl + 1, d_rk_loss_.p + std::min<long long>(steps - 1, 1023), sizeof(float),
                            cudaMemcpyDeviceToHost, stream_), "d2h");
  CheckCuda(cudaStreamSynchronize(stream_), "ranker sync");
  CheckError();
  rk_info_.first_loss = hl[0];
  rk_info_.final_loss = hl[1];
  rk_info_.train_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  rk_info_.trained = true;
  rk_trained_ = true;
}

void Engine::RankerFinishIteration() {
  if (!rk_trained_ || !d_rk_cut_.p) return;
  float* hc = reinterpret_cast<float*>(h_pin_.p);
  CheckCuda(cudaMemcpy(hc, d_rk_cut_.p, sizeof(float), cudaMemcpyDeviceToHost), "d2h cutoff");
  rk_info_.cutoff = hc[0];
}

}  // namespace beam

// ------------------------------------------------------------------ C ABI

extern "C" {

static thread_local std::string g_ranker_error;

const char* beam_ranker_last_error(void) { return g_ranker_error.c_str(); }

int beam_ranker_grad(int32_t device, const float* x, const float* y, const float* w, int64_t n, const float* params,
                     float* grad, double* loss, float* logits) {
  using namespace beam;
  try {
    if (n <= 0 || n > (1 << 20)) throw std::invalid_argument("sample count out of range (1 .. 2^20)");
    if (!x || !y || !params || !grad) throw std::invalid_argument("null argument");
    CheckCuda(cudaSetDevice(device), "cudaSetDevice");
    const size_t nn = static_cast<size_t>(n);
    DevBuf<float> dx, dy, dw, dp, dpart, dg, dl, dz;
    DevBuf<unsigned> dt;
    dx.ensure(nn * kRkFeat);
    dy.ensure(nn);
    dw.ensure(nn);
    dp.ensure(kRkParams);
    const int grid = static_cast<int>((n + kRkThreads - 1) / kRkThreads);
    dpart.ensure(static_cast<size_t>(grid) * kRkPartial);
    dg.ensure(kRkParams);
    dl.ensure(1);
    dz.ensure(nn);
    dt.ensure(1);
    CheckCuda(cudaMemcpy(dx.p, x, sizeof(float) * nn * kRkFeat, cudaMemcpyHostToDevice), "h2d x");
    CheckCuda(cudaMemcpy(dy.p, y, sizeof(float) * nn, cudaMemcpyHostToDevice), "h2d y");
    if (w) CheckCuda(cudaMemcpy(dw.p, w, sizeof(float) * nn, cudaMemcpyHostToDevice), "h2d w");
    CheckCuda(cudaMemcpy(dp.p, params, sizeof(float) * kRkParams, cudaMemcpyHostToDevice), "h2d params");
    CheckCuda(cudaMemset(dt.p, 0, sizeof(unsigned)), "memset ticket");
    CheckCuda(cudaFuncSetAttribute(RankerGradKernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(RkGradSmemBytes())), "ranker smem attribute");
    RkGradParams G;
    std::memset(&G, 0, sizeof(G));
    G.x = dx.p;
    G.y = dy.p;
    G.wt = w ? dw.p : nullptr;
    G.n = n;
    G.batch = static_cast<int>(n);
    G.pos_w = 1.0f;
    G.params = dp.p;
    G.partial = dpart.p;
    G.ticket = dt.p;
    G.grad_out = dg.p;
    G.loss_out = dl.p;
    G.z_out = dz.p;
    RankerGradKernel<<<grid, kRkThreads, RkGradSmemBytes()>>>(G);
    CheckCuda(cudaGetLastError(), "ranker gradient launch");
    CheckCuda(cudaDeviceSynchronize(), "ranker gradient");
    CheckCuda(cudaMemcpy(grad, dg.p, sizeof(float) * kRkParams, cudaMemcpyDeviceToHost), "d2h grad");
    float l = 0.0f;
    CheckCuda(cudaMemcpy(&l, dl.p, sizeof(float), cudaMemcpyDeviceToHost), "d2h loss");
    if (loss) *loss = l;
    if (logits) CheckCuda(cudaMemcpy(logits, dz.p, sizeof(float) * nn, cudaMemcpyDeviceToHost), "d2h logits");
    return 0;
  } catch (const std::exception& ex) {
    g_ranker_error = ex.what();
    return 1;
  }
}

}  // extern "C"
