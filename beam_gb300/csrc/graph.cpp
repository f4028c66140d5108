// Graph input for the merge loop: seeded synthetic generators, the text
// edge-list loader and a binary int32 edge-list loader, all producing the
// symmetric CSR the summarizer runs on.
//
// CSR semantics follow the reference loader (src/graph_io/graph_io.cpp:12-106):
// every undirected edge "u v" becomes the two arcs u->v and v->u, n is
// max id + 1, neighbour lists are sorted ascending, duplicates are kept and
// self-loops are rejected.
//
// Generators are deterministic across machines: all randomness comes from a
// fixed xoshiro256** stream, probabilities are compared as 53-bit integers,
// and the only floating-point operations are IEEE-exact +, -, *, /, floor,
// frexp and ldexp (this file must be compiled with -ffp-contract=off), so the
// same seed yields the same edge list on x86-64 and aarch64.
//
// Large graphs are built on all host cores with the same result as one
// thread: R-MAT draws are split into fixed-size chunks whose stream positions
// are reached by jumping the xoshiro256 state (its update is linear over
// GF(2), so a jump of k draws is the k-th power of a 256x256 bit matrix), the
// edge keys are sorted by a stable parallel radix sort, and the CSR rows are
// filled in parallel and then sorted.

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <limits>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "beam_gb300.h"

namespace {

thread_local std::string g_graph_error;

int HostThreads() {
  const unsigned hc = std::thread::hardware_concurrency();
  return static_cast<int>(std::max(1u, std::min(hc, 64u)));
}

// Runs body(t) for t in [0, threads) on that many threads (t == 0 on the caller's).
template <typename F>
void ParallelRun(int threads, F&& body) {
  if (threads <= 1) {
    body(0);
    return;
  }
  std::vector<std::thread> pool;
  pool.reserve(static_cast<size_t>(threads - 1));
  for (int t = 1; t < threads; ++t) pool.emplace_back([&body, t] { body(t); });
  body(0);
  for (auto& th : pool) th.join();
}

// [begin, end) of part t when `count` items are split into `parts` contiguous parts.
inline int64_t PartBegin(int64_t count, int parts, int t) {
  return static_cast<int64_t>((static_cast<unsigned __int128>(count) * static_cast<unsigned>(t)) /
                              static_cast<unsigned>(parts));
}

struct Rng {
  uint64_t s[4];
  static uint64_t SplitMix(uint64_t& x) {
    uint64_t z = (x += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
  }
  explicit Rng(uint64_t seed) {
    uint64_t x = seed;
    for (auto& v : s) v = SplitMix(x);
  }
  static uint64_t Rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  // The state update alone (linear over GF(2)).
  static void Step(uint64_t* s) {
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = Rotl(s[3], 45);
  }
  uint64_t Next() {
    const uint64_t result = Rotl(s[1] * 5, 7) * 9;
    Step(s);
    return result;
  }
  // 53-bit uniform integer; compare with Threshold(p) for a Bernoulli draw.
  uint64_t Next53() { return Next() >> 11; }
  double Uniform() { return static_cast<double>(Next53()) * 0x1.0p-53; }
  uint64_t Below(uint64_t bound) {  // unbiased enough for bound << 2^64
    return static_cast<uint64_t>((static_cast<unsigned __int128>(Next()) * bound) >> 64);
  }
};

// 256x256 matrix over GF(2) acting on the xoshiro256 state: bit i of the
// state is bit (i % 64) of word i / 64; row i holds the coefficients of
// output bit i.
struct StateMatrix {
  uint64_t row[256][4];

  static StateMatrix Identity() {
    StateMatrix m{};
    for (int i = 0; i < 256; ++i) m.row[i][i / 64] = uint64_t{1} << (i % 64);
    return m;
  }
  // The matrix of one Rng::Step: column j is the step applied to unit state j.
  static StateMatrix OneStep() {
    StateMatrix m{};
    for (int j = 0; j < 256; ++j) {
      uint64_t s[4] = {0, 0, 0, 0};
      s[j / 64] = uint64_t{1} << (j % 64);
      Rng::Step(s);
      for (int i = 0; i < 256; ++i) {
        if ((s[i / 64] >> (i % 64)) & 1) m.row[i][j / 64] |= uint64_t{1} << (j % 64);
      }
    }
    return m;
  }
  StateMatrix operator*(const StateMatrix& b) const {
    StateMatrix c{};
    for (int i = 0; i < 256; ++i) {
      for (int k = 0; k < 256; ++k) {
        if ((row[i][k / 64] >> (k % 64)) & 1) {
          for (int w = 0; w < 4; ++w) c.row[i][w] ^= b.row[k][w];
        }
      }
    }
    return c;
  }
  void Apply(const uint64_t* x, uint64_t* y) const {
    uint64_t out[4] = {0, 0, 0, 0};
    for (int i = 0; i < 256; ++i) {
      const uint64_t dot = (row[i][0] & x[0]) ^ (row[i][1] & x[1]) ^ (row[i][2] & x[2]) ^ (row[i][3] & x[3]);
      out[i / 64] |= static_cast<uint64_t>(__builtin_parityll(dot)) << (i % 64);
    }
    std::memcpy(y, out, sizeof(out));
  }
  // The matrix that advances a stream by `steps` draws.
  static StateMatrix Jump(uint64_t steps) {
    StateMatrix result = Identity();
    StateMatrix base = OneStep();
    while (steps) {
      if (steps & 1) result = result * base;
      steps >>= 1;
      if (steps) base = base * base;
    }
    return result;
  }
};

uint64_t Threshold(double p) {
  if (!(p > 0.0)) return 0;
  if (p >= 1.0) return uint64_t{1} << 53;
  return static_cast<uint64_t>(p * 0x1.0p53);
}

// Stable LSD radix sort of the low `bits` bits of every key, on all cores.
void ParallelRadixSort(std::vector<uint64_t>& keys, int bits) {
  const int64_t count = static_cast<int64_t>(keys.size());
  if (count < (1 << 16)) {
    std::stable_sort(keys.begin(), keys.end(), [bits](uint64_t a, uint64_t b) {
      const uint64_t mask = bits >= 64 ? ~uint64_t{0} : ((uint64_t{1} << bits) - 1);
      return (a & mask) < (b & mask);
    });
    return;
  }
  const int passes = std::max(1, (bits + 11) / 12);
  const int width = (bits + passes - 1) / passes;
  const size_t buckets = size_t{1} << width;
  const int threads = HostThreads();
  std::vector<uint64_t> tmp(keys.size());
  std::vector<int64_t> hist(static_cast<size_t>(threads) * buckets);
  uint64_t* src = keys.data();
  uint64_t* dst = tmp.data();
  for (int p = 0; p < passes; ++p) {
    const int shift = p * width;
    const uint64_t mask = buckets - 1;
    std::fill(hist.begin(), hist.end(), 0);
    ParallelRun(threads, [&](int t) {
      int64_t* h = hist.data() + static_cast<size_t>(t) * buckets;
      for (int64_t i = PartBegin(count, threads, t), e = PartBegin(count, threads, t + 1); i < e; ++i) {
        ++h[(src[i] >> shift) & mask];
      }
    });
    // exclusive offsets in (digit, part) order keep the sort stable
    int64_t acc = 0;
    for (size_t d = 0; d < buckets; ++d) {
      for (int t = 0; t < threads; ++t) {
        int64_t& h = hist[static_cast<size_t>(t) * buckets + d];
        const int64_t c = h;
        h = acc;
        acc += c;
      }
    }
    ParallelRun(threads, [&](int t) {
      int64_t* h = hist.data() + static_cast<size_t>(t) * buckets;
      for (int64_t i = PartBegin(count, threads, t), e = PartBegin(count, threads, t + 1); i < e; ++i) {
        dst[h[(src[i] >> shift) & mask]++] = src[i];
      }
    });
    std::swap(src, dst);
  }
  if (src != keys.data()) keys.swap(tmp);
}

// Sorted, duplicate-free copy of the packed (lo << 32 | hi) edge keys, where
// every id is below 2^id_bits.
void SortUniqueEdges(std::vector<uint64_t>& packed, int id_bits) {
  const int64_t count = static_cast<int64_t>(packed.size());
  const int threads = HostThreads();
  // (lo << 32 | hi) -> (lo << id_bits | hi): the sort covers 2 * id_bits bits
  ParallelRun(threads, [&](int t) {
    for (int64_t i = PartBegin(count, threads, t), e = PartBegin(count, threads, t + 1); i < e; ++i) {
      packed[i] = ((packed[i] >> 32) << id_bits) | (packed[i] & 0xffffffffu);
    }
  });
  ParallelRadixSort(packed, 2 * id_bits);
  // keep the first key of each run of equal keys, restoring the (lo << 32 | hi) form
  std::vector<int64_t> kept(static_cast<size_t>(threads) + 1, 0);
  ParallelRun(threads, [&](int t) {
    int64_t c = 0;
    for (int64_t i = PartBegin(count, threads, t), e = PartBegin(count, threads, t + 1); i < e; ++i) {
      c += (i == 0 || packed[i] != packed[i - 1]) ? 1 : 0;
    }
    kept[static_cast<size_t>(t) + 1] = c;
  });
  for (int t = 0; t < threads; ++t) kept[static_cast<size_t>(t) + 1] += kept[static_cast<size_t>(t)];
  std::vector<uint64_t> out(static_cast<size_t>(kept[static_cast<size_t>(threads)]));
  const uint64_t low = (uint64_t{1} << id_bits) - 1;
  ParallelRun(threads, [&](int t) {
    int64_t o = kept[static_cast<size_t>(t)];
    for (int64_t i = PartBegin(count, threads, t), e = PartBegin(count, threads, t + 1); i < e; ++i) {
      if (i == 0 || packed[i] != packed[i - 1]) out[o++] = ((packed[i] >> id_bits) << 32) | (packed[i] & low);
    }
  });
  packed.swap(out);
}

// Deterministic natural log / exp built from IEEE-exact basic operations only.
double DetLog(double x) {
  int e = 0;
  double m = std::frexp(x, &e);  // x = m * 2^e, m in [0.5, 1)
  const double t = (m - 1.0) / (m + 1.0);
  const double t2 = t * t;
  double term = t;
  double sum = 0.0;
  for (int k = 1; k < 80; k += 2) {
    sum += term / static_cast<double>(k);
    term *= t2;
  }
  const double kLn2 = 0.6931471805599453094;
  return 2.0 * sum + static_cast<double>(e) * kLn2;
}

double DetExp(double y) {
  const double kLn2 = 0.6931471805599453094;
  const double k = std::floor(y / kLn2);
  const double r = y - k * kLn2;
  double term = 1.0;
  double sum = 1.0;
  for (int i = 1; i < 40; ++i) {
    term *= r / static_cast<double>(i);
    sum += term;
  }
  return std::ldexp(sum, static_cast<int>(k));
}

double DetPow(double x, double y) { return DetExp(y * DetLog(x)); }

struct EdgeList {
  int64_t n = 0;
  std::vector<int32_t> u;
  std::vector<int32_t> v;
};

// Keeps each undirected edge once (self-loops were never pushed). With
// relabel, the endpoints that occur are renumbered densely in ascending
// original-id order; otherwise ids are kept and n = max id + 1, as the text
// loader computes it, so isolated ids below the maximum stay as nodes.
EdgeList CanonicalEdges(std::vector<uint64_t>& packed, bool relabel) {
  uint64_t max_hi = 0;
  for (uint64_t key : packed) max_hi = std::max<uint64_t>(max_hi, key & 0xffffffffu);
  int id_bits = 1;
  while (id_bits < 32 && (max_hi >> id_bits) != 0) ++id_bits;
  SortUniqueEdges(packed, id_bits);
  if (!relabel) {
    EdgeList out;
    const int64_t count = static_cast<int64_t>(packed.size());
    out.u.resize(packed.size());
    out.v.resize(packed.size());
    const int threads = HostThreads();
    ParallelRun(threads, [&](int t) {
      for (int64_t i = PartBegin(count, threads, t), e = PartBegin(count, threads, t + 1); i < e; ++i) {
        out.u[i] = static_cast<int32_t>(packed[i] >> 32);
        out.v[i] = static_cast<int32_t>(packed[i] & 0xffffffffu);
      }
    });
    out.n = packed.empty() ? 0 : static_cast<int64_t>(max_hi) + 1;
    return out;
  }
  std::vector<uint32_t> ids;
  ids.reserve(packed.size() * 2);
  for (uint64_t key : packed) {
    ids.push_back(static_cast<uint32_t>(key >> 32));
    ids.push_back(static_cast<uint32_t>(key & 0xffffffffu));
  }
  std::sort(ids.begin(), ids.end());
  ids.erase(std::unique(ids.begin(), ids.end()), ids.end());
  EdgeList out;
  out.n = static_cast<int64_t>(ids.size());
  out.u.resize(packed.size());
  out.v.resize(packed.size());
  for (size_t i = 0; i < packed.size(); ++i) {
    const uint32_t a = static_cast<uint32_t>(packed[i] >> 32);
    const uint32_t b = static_cast<uint32_t>(packed[i] & 0xffffffffu);
    out.u[i] = static_cast<int32_t>(std::lower_bound(ids.begin(), ids.end(), a) - ids.begin());
    out.v[i] = static_cast<int32_t>(std::lower_bound(ids.begin(), ids.end(), b) - ids.begin());
  }
  return out;
}

inline void PushEdge(std::vector<uint64_t>& packed, uint64_t a, uint64_t b) {
  if (a == b) return;
  if (a > b) std::swap(a, b);
  packed.push_back((a << 32) | b);
}

// R-MAT: each edge picks one of four quadrants per level with probabilities
// (a, b, c, d), one draw of the seed's stream per level, edges in order.
// Chunks of kRmatChunk edges run in parallel from jumped stream positions;
// the key list is the one a single pass over the stream produces.
void GenRmat(std::vector<uint64_t>& packed, int scale, double edge_factor, double a, double b,
             double c, uint64_t seed) {
  if (scale < 1 || scale > 30) throw std::invalid_argument("rmat scale must be in [1, 30]");
  constexpr int64_t kRmatChunk = int64_t{1} << 16;
  const uint64_t ta = Threshold(a);
  const uint64_t tb = Threshold(a + b);
  const uint64_t tc = Threshold(a + b + c);
  const int64_t samples = static_cast<int64_t>(edge_factor * static_cast<double>(int64_t{1} << scale));
  if (samples <= 0) return;
  const int64_t chunks = (samples + kRmatChunk - 1) / kRmatChunk;
  // stream state at the start of every chunk
  std::vector<uint64_t> starts(static_cast<size_t>(chunks) * 4);
  {
    Rng rng(seed);
    const StateMatrix jump = StateMatrix::Jump(static_cast<uint64_t>(kRmatChunk) * static_cast<uint64_t>(scale));
    uint64_t s[4] = {rng.s[0], rng.s[1], rng.s[2], rng.s[3]};
    for (int64_t ch = 0; ch < chunks; ++ch) {
      std::memcpy(&starts[static_cast<size_t>(ch) * 4], s, sizeof(s));
      if (ch + 1 < chunks) jump.Apply(s, s);
    }
  }
  constexpr uint64_t kLoop = ~uint64_t{0};
  std::vector<uint64_t> keys(static_cast<size_t>(samples));
  const int threads = HostThreads();
  std::atomic<int64_t> next_chunk{0};
  ParallelRun(threads, [&](int) {
    for (int64_t ch = next_chunk++; ch < chunks; ch = next_chunk++) {
      Rng rng(0);
      std::memcpy(rng.s, &starts[static_cast<size_t>(ch) * 4], sizeof(rng.s));
      const int64_t e1 = std::min(samples, (ch + 1) * kRmatChunk);
      for (int64_t e = ch * kRmatChunk; e < e1; ++e) {
        uint64_t row = 0;
        uint64_t col = 0;
        for (int level = 0; level < scale; ++level) {
          const uint64_t r = rng.Next53();
          const uint64_t bit_row = r >= tb ? 1 : 0;
          const uint64_t bit_col = (r >= ta && r < tb) || r >= tc ? 1 : 0;
          row = (row << 1) | bit_row;
          col = (col << 1) | bit_col;
        }
        keys[static_cast<size_t>(e)] = row == col ? kLoop : (std::min(row, col) << 32) | std::max(row, col);
      }
    }
  });
  // drop the self-loops, keeping the draw order
  std::vector<int64_t> kept(static_cast<size_t>(threads) + 1, 0);
  ParallelRun(threads, [&](int t) {
    int64_t cnt = 0;
    for (int64_t i = PartBegin(samples, threads, t), e = PartBegin(samples, threads, t + 1); i < e; ++i) {
      cnt += keys[static_cast<size_t>(i)] != kLoop ? 1 : 0;
    }
    kept[static_cast<size_t>(t) + 1] = cnt;
  });
  for (int t = 0; t < threads; ++t) kept[static_cast<size_t>(t) + 1] += kept[static_cast<size_t>(t)];
  const size_t base = packed.size();
  packed.resize(base + static_cast<size_t>(kept[static_cast<size_t>(threads)]));
  ParallelRun(threads, [&](int t) {
    size_t o = base + static_cast<size_t>(kept[static_cast<size_t>(t)]);
    for (int64_t i = PartBegin(samples, threads, t), e = PartBegin(samples, threads, t + 1); i < e; ++i) {
      if (keys[static_cast<size_t>(i)] != kLoop) packed[o++] = keys[static_cast<size_t>(i)];
    }
  });
}

// Power-law weights w_i = (i + i0)^(-1/(gamma-1)), i = 0..n-1.
std::vector<double> PowerLawWeights(int64_t n, double gamma, double i0) {
  std::vector<double> w(static_cast<size_t>(n));
  const double expo = -1.0 / (gamma - 1.0);
  for (int64_t i = 0; i < n; ++i) {
    w[static_cast<size_t>(i)] = DetPow(static_cast<double>(i) + i0, expo);
  }
  return w;
}

// Chung-Lu by endpoint sampling: both endpoints of each of `samples` edges are
// drawn proportionally to the weights; repeats and loops are removed later.
void GenChungLuSampled(std::vector<uint64_t>& packed, const std::vector<double>& w,
                       uint64_t id_offset, int64_t samples, Rng& rng) {
  std::vector<double> cdf(w.size());
  double acc = 0.0;
  for (size_t i = 0; i < w.size(); ++i) {
    acc += w[i];
    cdf[i] = acc;
  }
  auto draw = [&]() -> uint64_t {
    const double x = rng.Uniform() * acc;
    size_t idx = static_cast<size_t>(std::upper_bound(cdf.begin(), cdf.end(), x) - cdf.begin());
    if (idx >= cdf.size()) idx = cdf.size() - 1;
    return id_offset + idx;
  };
  packed.reserve(packed.size() + static_cast<size_t>(samples));
  for (int64_t e = 0; e < samples; ++e) {
    const uint64_t a = draw();
    const uint64_t b = draw();
    PushEdge(packed, a, b);
  }
}

// Degree-corrected SBM: p_uv = min(1, lambda * w_u * w_v * (same block ? ratio : 1)),
// lambda chosen by bisection so the expected edge count equals target_edges.
void GenDcsbm(std::vector<uint64_t>& packed, int64_t n, int blocks, double ratio, double gamma,
              double mean_degree, uint64_t seed) {
  Rng rng(seed);
  std::vector<double> base = PowerLawWeights(n, gamma, 1.0);
  // Shuffle weights over nodes (Fisher-Yates) so block and weight are independent.
  for (int64_t i = n - 1; i > 0; --i) {
    const int64_t j = static_cast<int64_t>(rng.Below(static_cast<uint64_t>(i + 1)));
    std::swap(base[static_cast<size_t>(i)], base[static_cast<size_t>(j)]);
  }
  const double target = mean_degree * static_cast<double>(n) / 2.0;
  auto expected = [&](double lambda) {
    double sum = 0.0;
    for (int64_t u = 0; u < n; ++u) {
      for (int64_t v = u + 1; v < n; ++v) {
        const double f = (u % blocks) == (v % blocks) ? ratio : 1.0;
        double p = lambda * base[static_cast<size_t>(u)] * base[static_cast<size_t>(v)] * f;
        sum += p < 1.0 ? p : 1.0;
      }
    }
    return sum;
  };
  double lo = 0.0;
  double hi = 1.0;
  while (expected(hi) < target) hi *= 2.0;
  for (int it = 0; it < 50; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (expected(mid) < target) lo = mid; else hi = mid;
  }
  const double lambda = 0.5 * (lo + hi);
  for (int64_t u = 0; u < n; ++u) {
    for (int64_t v = u + 1; v < n; ++v) {
      const double f = (u % blocks) == (v % blocks) ? ratio : 1.0;
      const double p = lambda * base[static_cast<size_t>(u)] * base[static_cast<size_t>(v)] * f;
      if (rng.Next53() < Threshold(p)) PushEdge(packed, static_cast<uint64_t>(u), static_cast<uint64_t>(v));
    }
  }
}

// Chooses i0 so that w_0 / mean(w) == max_over_mean for w_i = (i+i0)^(-1/(gamma-1)).
double SolveOffset(int64_t n, double gamma, double max_over_mean) {
  auto ratio = [&](double i0) {
    const double expo = -1.0 / (gamma - 1.0);
    // mean via a coarse deterministic quadrature over log-spaced points
    double sum = 0.0;
    const int64_t step = std::max<int64_t>(1, n / 4096);
    int64_t count = 0;
    for (int64_t i = 0; i < n; i += step) {
      sum += DetPow(static_cast<double>(i) + i0, expo);
      ++count;
    }
    const double mean = sum / static_cast<double>(count);
    return DetPow(i0, expo) / mean;
  };
  double lo = 1e-3;
  double hi = static_cast<double>(n);
  for (int it = 0; it < 60; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (ratio(mid) > max_over_mean) lo = mid; else hi = mid;
  }
  return 0.5 * (lo + hi);
}

void GenGrid(std::vector<uint64_t>& packed, int64_t side, double delete_p, double diag_p, Rng& rng) {
  const uint64_t keep = Threshold(1.0 - delete_p);
  const uint64_t diag = Threshold(diag_p);
  for (int64_t r = 0; r < side; ++r) {
    for (int64_t c = 0; c < side; ++c) {
      const uint64_t id = static_cast<uint64_t>(r * side + c);
      if (c + 1 < side && rng.Next53() < keep) PushEdge(packed, id, id + 1);
      if (r + 1 < side && rng.Next53() < keep) PushEdge(packed, id, id + static_cast<uint64_t>(side));
      if (r + 1 < side && rng.Next53() < diag) {
        const bool right = (rng.Next() & 1) != 0;
        if (right && c + 1 < side) PushEdge(packed, id, id + static_cast<uint64_t>(side) + 1);
        if (!right && c > 0) PushEdge(packed, id, id + static_cast<uint64_t>(side) - 1);
      }
    }
  }
}

void GenPlantedTwins(std::vector<uint64_t>& packed, int64_t n, int64_t groups, Rng& rng) {
  // Disjoint twin groups from a seeded permutation of the node ids.
  std::vector<uint32_t> perm(static_cast<size_t>(n));
  for (int64_t i = 0; i < n; ++i) perm[static_cast<size_t>(i)] = static_cast<uint32_t>(i);
  for (int64_t i = n - 1; i > 0; --i) {
    const int64_t j = static_cast<int64_t>(rng.Below(static_cast<uint64_t>(i + 1)));
    std::swap(perm[static_cast<size_t>(i)], perm[static_cast<size_t>(j)]);
  }
  const uint64_t share = Threshold(0.9);
  size_t cursor = 0;
  for (int64_t g = 0; g < groups; ++g) {
    const int64_t members = 2 + static_cast<int64_t>(rng.Below(7));      // 2..8
    const int64_t nbrs = 8 + static_cast<int64_t>(rng.Below(57));        // 8..64
    if (cursor + static_cast<size_t>(members) > perm.size()) break;
    std::vector<uint64_t> set(static_cast<size_t>(nbrs));
    for (auto& s : set) s = rng.Below(static_cast<uint64_t>(n));
    for (int64_t m = 0; m < members; ++m) {
      const uint64_t node = perm[cursor + static_cast<size_t>(m)];
      for (uint64_t s : set) {
        if (rng.Next53() < share) PushEdge(packed, node, s);
      }
    }
    cursor += static_cast<size_t>(members);
  }
}

std::map<std::string, std::string> ParseSpec(const std::string& spec, std::string* kind) {
  std::map<std::string, std::string> kv;
  const size_t colon = spec.find(':');
  *kind = spec.substr(0, colon);
  if (colon == std::string::npos) return kv;
  std::stringstream ss(spec.substr(colon + 1));
  std::string item;
  while (std::getline(ss, item, ',')) {
    const size_t eq = item.find('=');
    if (eq == std::string::npos) throw std::invalid_argument("bad graph spec item: " + item);
    kv[item.substr(0, eq)] = item.substr(eq + 1);
  }
  return kv;
}

double GetD(const std::map<std::string, std::string>& kv, const char* key, double dflt) {
  auto it = kv.find(key);
  return it == kv.end() ? dflt : std::stod(it->second);
}

int64_t GetI(const std::map<std::string, std::string>& kv, const char* key, int64_t dflt) {
  auto it = kv.find(key);
  return it == kv.end() ? dflt : std::stoll(it->second);
}

EdgeList Generate(const std::string& spec) {
  std::string kind;
  const auto kv = ParseSpec(spec, &kind);
  std::vector<uint64_t> packed;
  const uint64_t seed = static_cast<uint64_t>(GetI(kv, "seed", 1));
  if (kind == "rmat") {
    GenRmat(packed, static_cast<int>(GetI(kv, "scale", 19)), GetD(kv, "ef", 2.0), GetD(kv, "a", 0.57),
            GetD(kv, "b", 0.19), GetD(kv, "c", 0.19), seed);
  } else if (kind == "dcsbm") {
    GenDcsbm(packed, GetI(kv, "n", 4096), static_cast<int>(GetI(kv, "blocks", 32)), GetD(kv, "ratio", 40.0),
             GetD(kv, "gamma", 2.5), GetD(kv, "deg", 43.0), seed);
  } else if (kind == "chunglu") {
    Rng rng(seed);
    const int64_t n = GetI(kv, "n", 100000);
    const double gamma = GetD(kv, "gamma", 2.3);
    const double deg = GetD(kv, "deg", 17.0);
    const double maxr = GetD(kv, "maxratio", 0.0);
    const double i0 = maxr > 0.0 ? SolveOffset(n, gamma, maxr) : 1.0;
    const std::vector<double> w = PowerLawWeights(n, gamma, i0);
    GenChungLuSampled(packed, w, 0, static_cast<int64_t>(deg * static_cast<double>(n) / 2.0), rng);
    const int64_t twins = GetI(kv, "twins", 0);
    if (twins > 0) GenPlantedTwins(packed, n, twins, rng);
  } else if (kind == "union") {
    // grid (side x side) + Chung-Lu component with ids after the grid
    Rng rng(seed);
    const int64_t side = GetI(kv, "side", 1400);
    GenGrid(packed, side, GetD(kv, "del", 0.10), GetD(kv, "diag", 0.02), rng);
    const int64_t n = GetI(kv, "n", 1100000);
    const double gamma = GetD(kv, "gamma", 2.1);
    const double deg = GetD(kv, "deg", 5.4);
    const double maxdeg = GetD(kv, "maxdeg", 28000.0);
    const double i0 = SolveOffset(n, gamma, maxdeg / deg);
    const std::vector<double> w = PowerLawWeights(n, gamma, i0);
    GenChungLuSampled(packed, w, static_cast<uint64_t>(side * side), static_cast<int64_t>(deg * static_cast<double>(n) / 2.0), rng);
  } else if (kind == "grid") {
    Rng rng(seed);
    GenGrid(packed, GetI(kv, "side", 64), GetD(kv, "del", 0.10), GetD(kv, "diag", 0.02), rng);
  } else if (kind == "gnm") {
    Rng rng(seed);
    const int64_t n = GetI(kv, "n", 100);
    const int64_t m = GetI(kv, "m", 300);
    for (int64_t e = 0; e < m; ++e) {
      PushEdge(packed, rng.Below(static_cast<uint64_t>(n)), rng.Below(static_cast<uint64_t>(n)));
    }
  } else {
    throw std::invalid_argument("unknown graph kind: " + kind);
  }
  return CanonicalEdges(packed, GetI(kv, "relabel", 0) != 0);
}

}  // namespace

struct beam_graph {
  int64_t n = 0;
  int64_t input_edges_raw = 0;
  std::vector<int32_t> eu;
  std::vector<int32_t> ev;
  std::vector<int64_t> row_ptr;
  std::vector<int32_t> col_idx;
};

namespace {

// Symmetric CSR with sorted neighbour lists (reference loader semantics).
// first[x] = first position i with key(i) >= x, for x in [0, n], over a
// list of `count` non-decreasing keys.
template <typename Key>
void RunStarts(int64_t count, int64_t n, Key key, int64_t* first, int threads) {
  ParallelRun(threads, [&](int t) {
    for (int64_t i = PartBegin(count, threads, t), e = PartBegin(count, threads, t + 1); i < e; ++i) {
      const int64_t lo = i == 0 ? 0 : key(i - 1) + 1;
      for (int64_t x = lo, hi = key(i); x <= hi; ++x) first[x] = i;
    }
  });
  for (int64_t x = count == 0 ? 0 : key(count - 1) + 1; x <= n; ++x) first[x] = count;
}

// CSR of a strictly increasing (u, v) edge list with u < v (the generators'
// output): row x is the u of every edge (u, x), ascending, then the v of every
// edge (x, v), ascending, with no per-row sort. The (v, u) order of the first
// part comes from a stable radix sort by v.
bool BuildCsrSorted(beam_graph* g, int threads) {
  const int64_t n = g->n;
  const int64_t edges = static_cast<int64_t>(g->eu.size());
  const int32_t* eu = g->eu.data();
  const int32_t* ev = g->ev.data();
  std::atomic<bool> sorted{true};
  ParallelRun(threads, [&](int t) {
    for (int64_t i = PartBegin(edges, threads, t), e = PartBegin(edges, threads, t + 1); i < e; ++i) {
      if (eu[i] >= ev[i] || ev[i] >= n || eu[i] < 0 ||
          (i > 0 && (eu[i - 1] > eu[i] || (eu[i - 1] == eu[i] && ev[i - 1] >= ev[i])))) {
        sorted = false;
        break;
      }
    }
  });
  if (!sorted) return false;
  int id_bits = 1;
  while (id_bits < 32 && ((n - 1) >> id_bits) != 0) ++id_bits;
  std::vector<uint64_t> tr(static_cast<size_t>(edges));
  ParallelRun(threads, [&](int t) {
    for (int64_t i = PartBegin(edges, threads, t), e = PartBegin(edges, threads, t + 1); i < e; ++i) {
      tr[i] = (static_cast<uint64_t>(eu[i]) << 32) | static_cast<uint32_t>(ev[i]);
    }
  });
  ParallelRadixSort(tr, id_bits);  // by v, u ascending within equal v (stable)
  std::vector<int64_t> fwd(static_cast<size_t>(n) + 1);
  std::vector<int64_t> bwd(static_cast<size_t>(n) + 1);
  RunStarts(edges, n, [&](int64_t i) { return static_cast<int64_t>(eu[i]); }, fwd.data(), threads);
  RunStarts(edges, n, [&](int64_t i) { return static_cast<int64_t>(tr[i] & 0xffffffffu); }, bwd.data(), threads);
  g->row_ptr.resize(static_cast<size_t>(n) + 1);
  int64_t* rp = g->row_ptr.data();
  ParallelRun(threads, [&](int t) {
    for (int64_t x = PartBegin(n + 1, threads, t), e = PartBegin(n + 1, threads, t + 1); x < e; ++x) {
      rp[x] = fwd[x] + bwd[x];
    }
  });
  g->col_idx.resize(static_cast<size_t>(2 * edges));
  int32_t* col = g->col_idx.data();
  ParallelRun(threads, [&](int t) {
    for (int64_t x = PartBegin(n, threads, t), e = PartBegin(n, threads, t + 1); x < e; ++x) {
      int64_t o = rp[x];
      for (int64_t i = bwd[x]; i < bwd[x + 1]; ++i) col[o++] = static_cast<int32_t>(tr[i] >> 32);
      for (int64_t i = fwd[x]; i < fwd[x + 1]; ++i) col[o++] = ev[i];
    }
  });
  return true;
}

// Rows are filled in parallel (arbitrary order within a row) and then sorted;
// a row's values are equal-or-distinct ids, so the sorted row is the same for
// any fill order.
void BuildCsr(beam_graph* g) {
  const int64_t n = g->n;
  const int64_t edges = static_cast<int64_t>(g->eu.size());
  const int threads = edges < (1 << 16) ? 1 : HostThreads();
  if (edges >= (1 << 16) && BuildCsrSorted(g, threads)) return;
  g->row_ptr.assign(static_cast<size_t>(n + 1), 0);
  int64_t* rp = g->row_ptr.data();
  const int32_t* eu = g->eu.data();
  const int32_t* ev = g->ev.data();
  ParallelRun(threads, [&](int t) {
    for (int64_t i = PartBegin(edges, threads, t), e = PartBegin(edges, threads, t + 1); i < e; ++i) {
      __atomic_fetch_add(&rp[eu[i] + 1], int64_t{1}, __ATOMIC_RELAXED);
      __atomic_fetch_add(&rp[ev[i] + 1], int64_t{1}, __ATOMIC_RELAXED);
    }
  });
  for (int64_t i = 0; i < n; ++i) rp[i + 1] += rp[i];
  g->col_idx.assign(static_cast<size_t>(rp[n]), 0);
  int32_t* col = g->col_idx.data();
  std::vector<int64_t> cur(g->row_ptr.begin(), g->row_ptr.end() - 1);
  int64_t* cp = cur.data();
  ParallelRun(threads, [&](int t) {
    for (int64_t i = PartBegin(edges, threads, t), e = PartBegin(edges, threads, t + 1); i < e; ++i) {
      col[__atomic_fetch_add(&cp[eu[i]], int64_t{1}, __ATOMIC_RELAXED)] = ev[i];
      col[__atomic_fetch_add(&cp[ev[i]], int64_t{1}, __ATOMIC_RELAXED)] = eu[i];
    }
  });
  std::atomic<int64_t> next_rows{0};
  constexpr int64_t kRows = 4096;
  ParallelRun(threads, [&](int) {
    for (int64_t r0 = next_rows.fetch_add(kRows); r0 < n; r0 = next_rows.fetch_add(kRows)) {
      for (int64_t v = r0, r1 = std::min(n, r0 + kRows); v < r1; ++v) {
        std::sort(col + rp[v], col + rp[v + 1]);
      }
    }
  });
}

beam_graph* FromEdges(int64_t n, std::vector<int32_t>&& u, std::vector<int32_t>&& v) {
  auto* g = new beam_graph();
  g->n = n;
  g->input_edges_raw = static_cast<int64_t>(u.size());
  g->eu = std::move(u);
  g->ev = std::move(v);
  BuildCsr(g);
  return g;
}

void SetError(const std::string& msg) { g_graph_error = msg; }

}  // namespace

extern "C" {

const char* beam_graph_last_error(void) { return g_graph_error.c_str(); }

beam_graph* beam_graph_generate(const char* spec) {
  try {
    EdgeList e = Generate(spec ? spec : "");
    return FromEdges(e.n, std::move(e.u), std::move(e.v));
  } catch (const std::exception& ex) {
    SetError(ex.what());
    return nullptr;
  }
}

beam_graph* beam_graph_from_edges(const int32_t* u, const int32_t* v, int64_t edges) {
  try {
    if (edges < 0 || (edges > 0 && (u == nullptr || v == nullptr))) {
      throw std::invalid_argument("invalid edge arrays");
    }
    int64_t max_node = -1;
    for (int64_t i = 0; i < edges; ++i) {
      if (u[i] < 0 || v[i] < 0) throw std::runtime_error("Negative node id in edge list.");
      if (u[i] == v[i]) throw std::runtime_error("Self-loop is not supported.");
      max_node = std::max<int64_t>(max_node, std::max(u[i], v[i]));
    }
    if (max_node + 1 <= 0) throw std::runtime_error("Invalid node count.");
    return FromEdges(max_node + 1, std::vector<int32_t>(u, u + edges), std::vector<int32_t>(v, v + edges));
  } catch (const std::exception& ex) {
    SetError(ex.what());
    return nullptr;
  }
}

// Text edge list with the reference loader's rules: blank lines and lines
// whose first non-blank character is '#' are skipped, each other line starts
// with two non-negative integers, self-loops are an error.
beam_graph* beam_graph_load_text(const char* path) {
  try {
    std::ifstream in(path);
    if (!in) throw std::runtime_error(std::string("Failed to open file: ") + path);
    std::vector<int32_t> u;
    std::vector<int32_t> v;
    std::string line;
    int64_t line_no = 0;
    int64_t max_node = -1;
    while (std::getline(in, line)) {
      ++line_no;
      const size_t first = line.find_first_not_of(" \t\r");
      if (first == std::string::npos || line[first] == '#') continue;
      const char* p = line.c_str() + first;
      char* end = nullptr;
      errno = 0;
      const long long a = std::strtoll(p, &end, 10);
      if (end == p || errno != 0) throw std::runtime_error("Malformed edge list line " + std::to_string(line_no) + ": expected at least two integers 'u v'.");
      p = end;
      const long long b = std::strtoll(p, &end, 10);
      if (end == p || errno != 0) throw std::runtime_error("Malformed edge list line " + std::to_string(line_no) + ": expected at least two integers 'u v'.");
      if (a < 0 || b < 0) throw std::runtime_error("Negative node id at line " + std::to_string(line_no) + ".");
      if (a > std::numeric_limits<int>::max() || b > std::numeric_limits<int>::max()) {
        throw std::runtime_error("Node id exceeds int range at line " + std::to_string(line_no) + ".");
      }
      if (a == b) throw std::runtime_error("Self-loop is not supported at line " + std::to_string(line_no) + ".");
      u.push_back(static_cast<int32_t>(a));
      v.push_back(static_cast<int32_t>(b));
      max_node = std::max<int64_t>(max_node, std::max(a, b));
    }
    if (max_node + 1 <= 0) throw std::runtime_error("Invalid node count.");
    return FromEdges(max_node + 1, std::move(u), std::move(v));
  } catch (const std::exception& ex) {
    SetError(ex.what());
    return nullptr;
  }
}

// Binary edge list: int64 edge count E followed by 2*E little-endian int32
// values u0 v0 u1 v1 ... (same rules as the text loader).
beam_graph* beam_graph_load_binary(const char* path) {
  try {
    FILE* f = std::fopen(path, "rb");
    if (!f) throw std::runtime_error(std::string("Failed to open file: ") + path);
    int64_t edges = 0;
    if (std::fread(&edges, sizeof(edges), 1, f) != 1 || edges < 0) {
      std::fclose(f);
      throw std::runtime_error("Malformed binary edge list header.");
    }
    std::vector<int32_t> buf(static_cast<size_t>(edges) * 2);
    const size_t got = buf.empty() ? 0 : std::fread(buf.data(), sizeof(int32_t), buf.size(), f);
    std::fclose(f);
    if (got != buf.size()) throw std::runtime_error("Truncated binary edge list.");
    std::vector<int32_t> u(static_cast<size_t>(edges));
    std::vector<int32_t> v(static_cast<size_t>(edges));
    for (int64_t i = 0; i < edges; ++i) {
      u[static_cast<size_t>(i)] = buf[static_cast<size_t>(2 * i)];
      v[static_cast<size_t>(i)] = buf[static_cast<size_t>(2 * i + 1)];
    }
    beam_graph* g = beam_graph_from_edges(u.data(), v.data(), edges);
    if (!g) throw std::runtime_error(g_graph_error);
    return g;
  } catch (const std::exception& ex) {
    SetError(ex.what());
    return nullptr;
  }
}

int beam_graph_write_text(const beam_graph* g, const char* path) {
  FILE* f = std::fopen(path, "w");
  if (!f) {
    SetError(std::string("Failed to open output file: ") + path);
    return -1;
  }
  for (size_t i = 0; i < g->eu.size(); ++i) std::fprintf(f, "%d %d\n", g->eu[i], g->ev[i]);
  std::fclose(f);
  return 0;
}

int beam_graph_write_binary(const beam_graph* g, const char* path) {
  FILE* f = std::fopen(path, "wb");
  if (!f) {
    SetError(std::string("Failed to open output file: ") + path);
    return -1;
  }
  const int64_t edges = static_cast<int64_t>(g->eu.size());
  std::fwrite(&edges, sizeof(edges), 1, f);
  for (size_t i = 0; i < g->eu.size(); ++i) {
    const int32_t pair[2] = {g->eu[i], g->ev[i]};
    std::fwrite(pair, sizeof(int32_t), 2, f);
  }
  std::fclose(f);
  return 0;
}

int64_t beam_graph_num_nodes(const beam_graph* g) { return g->n; }
int64_t beam_graph_num_edges(const beam_graph* g) { return g->input_edges_raw; }
int64_t beam_graph_num_arcs(const beam_graph* g) { return static_cast<int64_t>(g->col_idx.size()); }
const int64_t* beam_graph_row_ptr(const beam_graph* g) { return g->row_ptr.data(); }
const int32_t* beam_graph_col_idx(const beam_graph* g) { return g->col_idx.data(); }
const int32_t* beam_graph_edge_u(const beam_graph* g) { return g->eu.data(); }
const int32_t* beam_graph_edge_v(const beam_graph* g) { return g->ev.data(); }
void beam_graph_free(beam_graph* g) { delete g; }

}  // extern "C"
