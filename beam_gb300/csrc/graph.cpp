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

#include <algorithm>
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
#include <vector>

#include "beam_gb300.h"

namespace {

thread_local std::string g_graph_error;

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
  uint64_t Next() {
    const uint64_t result = Rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = Rotl(s[3], 45);
    return result;
  }
  // 53-bit uniform integer; compare with Threshold(p) for a Bernoulli draw.
  uint64_t Next53() { return Next() >> 11; }
  double Uniform() { return static_cast<double>(Next53()) * 0x1.0p-53; }
  uint64_t Below(uint64_t bound) {  // unbiased enough for bound << 2^64
    return static_cast<uint64_t>((static_cast<unsigned __int128>(Next()) * bound) >> 64);
  }
};

uint64_t Threshold(double p) {
  if (!(p > 0.0)) return 0;
  if (p >= 1.0) return uint64_t{1} << 53;
  return static_cast<uint64_t>(p * 0x1.0p53);
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
  std::sort(packed.begin(), packed.end());
  packed.erase(std::unique(packed.begin(), packed.end()), packed.end());
  if (!relabel) {
    EdgeList out;
    out.u.resize(packed.size());
    out.v.resize(packed.size());
    int64_t max_id = -1;
    for (size_t i = 0; i < packed.size(); ++i) {
      out.u[i] = static_cast<int32_t>(packed[i] >> 32);
      out.v[i] = static_cast<int32_t>(packed[i] & 0xffffffffu);
      max_id = std::max<int64_t>(max_id, out.v[i]);
    }
    out.n = max_id + 1;
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
// (a, b, c, d).
void GenRmat(std::vector<uint64_t>& packed, int scale, double edge_factor, double a, double b,
             double c, uint64_t seed) {
  if (scale < 1 || scale > 30) throw std::invalid_argument("rmat scale must be in [1, 30]");
  Rng rng(seed);
  const uint64_t ta = Threshold(a);
  const uint64_t tb = Threshold(a + b);
  const uint64_t tc = Threshold(a + b + c);
  const int64_t samples = static_cast<int64_t>(edge_factor * static_cast<double>(int64_t{1} << scale));
  packed.reserve(packed.size() + static_cast<size_t>(samples));
  for (int64_t e = 0; e < samples; ++e) {
    uint64_t row = 0;
    uint64_t col = 0;
    for (int level = 0; level < scale; ++level) {
      const uint64_t r = rng.Next53();
      const uint64_t bit_row = r >= tb ? 1 : 0;
      const uint64_t bit_col = (r >= ta && r < tb) || r >= tc ? 1 : 0;
      row = (row << 1) | bit_row;
      col = (col << 1) | bit_col;
    }
    PushEdge(packed, row, col);
  }
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
void BuildCsr(beam_graph* g) {
  const int64_t n = g->n;
  g->row_ptr.assign(static_cast<size_t>(n + 1), 0);
  for (size_t i = 0; i < g->eu.size(); ++i) {
    g->row_ptr[static_cast<size_t>(g->eu[i]) + 1]++;
    g->row_ptr[static_cast<size_t>(g->ev[i]) + 1]++;
  }
  for (int64_t i = 0; i < n; ++i) g->row_ptr[static_cast<size_t>(i + 1)] += g->row_ptr[static_cast<size_t>(i)];
  g->col_idx.assign(static_cast<size_t>(g->row_ptr[static_cast<size_t>(n)]), 0);
  std::vector<int64_t> cur(g->row_ptr.begin(), g->row_ptr.end() - 1);
  for (size_t i = 0; i < g->eu.size(); ++i) {
    g->col_idx[static_cast<size_t>(cur[static_cast<size_t>(g->eu[i])]++)] = g->ev[i];
    g->col_idx[static_cast<size_t>(cur[static_cast<size_t>(g->ev[i])]++)] = g->eu[i];
  }
  for (int64_t v = 0; v < n; ++v) {
    std::sort(g->col_idx.begin() + g->row_ptr[static_cast<size_t>(v)],
              g->col_idx.begin() + g->row_ptr[static_cast<size_t>(v + 1)]);
  }
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
