// Learned candidate ranker: a 2-layer MLP (16 features -> 64 ReLU -> 1 logit,
// bf16 weights, fp32 biases and accumulation) that scores the EA-proxy
// candidate pairs of a group before exact scoring. It is trained on the GPU
// by this library's own kernels on the exact gains of the first iterations
// and then prunes candidates whose logit falls below a cutoff calibrated for
// recall; every merge is still accepted on its exact integer gain. The
// reference has no learned component: this sits beside the exact path.
#pragma once

#include <cuda_bf16.h>

#include "common.cuh"

namespace beam {

constexpr int kRkFeat = 16;
constexpr int kRkHidden = 64;
constexpr int kRkW1 = kRkHidden * kRkFeat;             // W1[h][f]
constexpr int kRkB1 = kRkW1;                           // b1[h]
constexpr int kRkW2 = kRkB1 + kRkHidden;               // w2[h]
constexpr int kRkB2 = kRkW2 + kRkHidden;               // b2
constexpr int kRkParams = kRkB2 + 1;                   // 1153
constexpr int kRkBf16 = kRkW1 + kRkHidden;             // bf16 copies: W1 | w2

__device__ __forceinline__ float RkBf16Round(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

// Pair features from the block-start state (symmetric in a, b):
//   0 log(1+sa)+log(1+sb)      1 |log(1+sa)-log(1+sb)|
//   2 log(1+la)+log(1+lb)      3 |log(1+la)-log(1+lb)|       (row lengths)
//   4 log(1+proxy gain)        5 proxy ratio (EA ranking key)
//   6 log(1+e(a,b))            7 log(1+int_a)+log(1+int_b)
//   8 threshold 1/(iter+1)     9 log(1+group size)
//  10 log(1+sa*sb)            11 e(a,b)/(sa*sb)
//  12 proxy/(1+min(la,lb))    13 log(1+min(la,lb))
//  14 log(1+max(la,lb))       15 proxy ratio / threshold
__device__ __forceinline__ void RankerFeatures(const QuotientView& Q, int a, int b, int g, float pg, float ratio,
                                               float thr, float* x) {
  const float sa = static_cast<float>(Q.size[a]);
  const float sb = static_cast<float>(Q.size[b]);
  const int la_i = Q.len[a];
  const float la = static_cast<float>(la_i);
  const float lb = static_cast<float>(Q.len[b]);
  const float e = static_cast<float>(RowLookup(Q.ent + Q.off[a], la_i, b));
  const float lsa = log1pf(sa), lsb = log1pf(sb), lla = log1pf(la), llb = log1pf(lb);
  const float cap = sa * sb;
  x[0] = lsa + lsb;
  x[1] = fabsf(lsa - lsb);
  x[2] = lla + llb;
  x[3] = fabsf(lla - llb);
  x[4] = log1pf(pg);
  x[5] = ratio;
  x[6] = log1pf(e);
  x[7] = log1pf(static_cast<float>(Q.internal[a])) + log1pf(static_cast<float>(Q.internal[b]));
  x[8] = thr;
  x[9] = log1pf(static_cast<float>(g));
  x[10] = log1pf(cap);
  x[11] = e / cap;
  x[12] = pg / (1.0f + fminf(la, lb));
  x[13] = log1pf(fminf(la, lb));
  x[14] = log1pf(fmaxf(la, lb));
  x[15] = ratio / thr;
}

// Forward pass with the weights in shared memory (as floats): returns the logit.
__device__ __forceinline__ float RankerForward(const float* w, const float* x) {
  float z = w[kRkB2];
#pragma unroll 4
  for (int j = 0; j < kRkHidden; ++j) {
    float a = w[kRkB1 + j];
#pragma unroll
    for (int f = 0; f < kRkFeat; ++f) a = fmaf(w[j * kRkFeat + f], x[f], a);
    z = fmaf(w[kRkW2 + j], fmaxf(a, 0.0f), z);
  }
  return z;
}

}  // namespace beam
