// Host-side summary materialisation and metrics for a partition produced on
// the GPU:
//   beam_encode                 Sweg::Encode, mags-compatible branch
//                               (src/sweg.cpp:3017-3163) + WriteOutput
//                               (src/sweg.cpp:3255-3287) + ComputeCompressionMetrics
//                               (include/compression_metrics.hpp:39-98)
//   beam_exact_partition_cost   CostOracle::ExactPartitionCost (src/cost_oracle.cpp:112-124)
//   beam_partition_hash         Sweg::PartitionHash (src/sweg.cpp:2920-2928)
// The partition arrives as member lists (head per rep, next per node) so
// that the supernode member order of G.txt is the reference's list order.

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "beam_gb300.h"
#include "encode_write.h"

namespace {

thread_local std::string g_encode_error;

struct PairArc {
  uint64_t key;
  int32_t u, v;
};

struct EdgePair {
  int32_t a, b;
  bool operator<(const EdgePair& o) const { return a != o.a ? a < o.a : b < o.b; }
};

void WritePairKeys(const std::string& path, const std::vector<unsigned long long>& v) {
  FILE* f = std::fopen(path.c_str(), "w");
  if (!f) throw std::runtime_error("Failed to open output file: " + path);
  std::string buf;
  buf.reserve(1 << 20);
  char line[32];
  for (const unsigned long long key : v) {
    const int k = std::snprintf(line, sizeof(line), "%d\t%d\n", static_cast<int32_t>(key >> 32),
                                static_cast<int32_t>(key & 0xffffffffu));
    buf.append(line, static_cast<size_t>(k));
    if (buf.size() > (1u << 20)) {
      std::fwrite(buf.data(), 1, buf.size(), f);
      buf.clear();
    }
  }
  std::fwrite(buf.data(), 1, buf.size(), f);
  std::fclose(f);
}

unsigned long long PairKey(const EdgePair& e) {
  return static_cast<unsigned long long>(static_cast<uint32_t>(e.a)) << 32 | static_cast<uint32_t>(e.b);
}

int64_t BlockCostHost(int64_t sa, int64_t sb, int64_t e, bool internal) {
  const __int128 capw = internal ? static_cast<__int128>(sa) * (sa - 1) / 2 : static_cast<__int128>(sa) * sb;
  if (sa < 0 || sb < 0 || e < 0 || capw > static_cast<__int128>(INT64_MAX) || static_cast<__int128>(e) > capw) {
    throw std::invalid_argument("edge count exceeds block capacity");
  }
  const int64_t alt = 1 + static_cast<int64_t>(capw) - e;
  return std::min(e, alt);
}

}  // namespace

namespace beam {

void FinishEncoding(int32_t n, int64_t arcs, const int32_t* head, const int32_t* next, const EncodeOutput& enc,
                    const char* out_dir, beam_encoding* out) {
  if (out_dir) {
    const std::string dir(out_dir);
    FILE* f = std::fopen((dir + "/G.txt").c_str(), "w");
    if (!f) throw std::runtime_error("Failed to open G.txt for writing.");
    int64_t sid = 0;
    for (int32_t rep = 0; rep < n; ++rep) {
      if (head[rep] == -1) continue;
      std::fprintf(f, "%lld", static_cast<long long>(sid++));
      for (int32_t v = head[rep]; v != -1; v = next[v]) std::fprintf(f, "\t%d", v);
      std::fputc('\n', f);
    }
    std::fclose(f);
    WritePairKeys(dir + "/P.txt", enc.P);
    WritePairKeys(dir + "/Cp.txt", enc.Cp);
    WritePairKeys(dir + "/Cm.txt", enc.Cm);
  }
  if (out) {
    std::memset(out, 0, sizeof(*out));
    out->supernodes = enc.supernodes;
    out->p = static_cast<int64_t>(enc.P.size());
    out->cp = static_cast<int64_t>(enc.Cp.size());
    out->cm = static_cast<int64_t>(enc.Cm.size());
    for (const unsigned long long key : enc.P) out->superedges_loop += (key >> 32) == (key & 0xffffffffu);
    out->superedges_nonloop = out->p - out->superedges_loop;
    out->encoding_cost_standard = out->p + out->cp + out->cm;
    out->encoding_cost_mags_x2 = 2 * out->encoding_cost_standard;
    const int64_t m = arcs / 2;
    out->cost_ratio_mags_compatible =
        m > 0 ? static_cast<double>(out->encoding_cost_mags_x2) / (2.0 * static_cast<double>(m)) : 0.0;
    out->cost_ratio_standard = m > 0 ? static_cast<double>(out->encoding_cost_standard) / static_cast<double>(m) : 0.0;
  }
}

}  // namespace beam

extern "C" {

const char* beam_encode_last_error(void) { return g_encode_error.c_str(); }

int beam_encode(int32_t n, int64_t arcs, const int64_t* row_ptr, const int32_t* col_idx, const int32_t* head,
                const int32_t* next, const char* out_dir, beam_encoding* out) {
  try {
    (void)arcs;
    std::vector<int32_t> nts(static_cast<size_t>(n), -1);
    std::vector<int32_t> shead;
    std::vector<int64_t> ssize;
    for (int32_t rep = 0; rep < n; ++rep) {
      if (head[rep] == -1) continue;
      const int32_t sid = static_cast<int32_t>(shead.size());
      int64_t cnt = 0;
      for (int32_t v = head[rep]; v != -1; v = next[v]) {
        if (v < 0 || v >= n || nts[static_cast<size_t>(v)] != -1) throw std::runtime_error("corrupt member lists");
        nts[static_cast<size_t>(v)] = sid;
        ++cnt;
      }
      shead.push_back(head[rep]);
      ssize.push_back(cnt);
    }
    for (int32_t v = 0; v < n; ++v) {
      if (nts[static_cast<size_t>(v)] < 0) throw std::runtime_error("Invalid node_to_supernode during encode.");
    }
    std::vector<PairArc> pa;
    pa.reserve(static_cast<size_t>(row_ptr[n] / 2 + 1));
    for (int32_t u = 0; u < n; ++u) {
      const int32_t su = nts[static_cast<size_t>(u)];
      for (int64_t k = row_ptr[u]; k < row_ptr[u + 1]; ++k) {
        const int32_t v = col_idx[k];
        const int32_t sv = nts[static_cast<size_t>(v)];
        if (su > sv || (su == sv && u >= v)) continue;
        pa.push_back(PairArc{(static_cast<uint64_t>(static_cast<uint32_t>(su)) << 32) | static_cast<uint32_t>(sv), u, v});
      }
    }
    std::sort(pa.begin(), pa.end(), [](const PairArc& x, const PairArc& y) {
      if (x.key != y.key) return x.key < y.key;
      if (x.u != y.u) return x.u < y.u;
      return x.v < y.v;
    });
    std::vector<EdgePair> P, Cp, Cm;
    for (size_t s = 0; s < pa.size();) {
      size_t e = s + 1;
      while (e < pa.size() && pa[e].key == pa[s].key) ++e;
      const int32_t A = static_cast<int32_t>(pa[s].key >> 32);
      const int32_t B = static_cast<int32_t>(pa[s].key & 0xffffffffu);
      const int64_t real = static_cast<int64_t>(e - s);
      const int64_t sa = ssize[static_cast<size_t>(A)];
      const int64_t sb = ssize[static_cast<size_t>(B)];
      const int64_t cap = A == B ? sa * (sa - 1) / 2 : sa * sb;
      if (real <= 1 + cap - real) {
        for (size_t k = s; k < e; ++k) Cp.push_back(EdgePair{pa[k].u, pa[k].v});
      } else {
        P.push_back(EdgePair{A, B});
        // missing member pairs of a dense block; the block's arcs are sorted by (u, v)
        for (int32_t u = shead[static_cast<size_t>(A)]; u != -1; u = next[u]) {
          for (int32_t v = shead[static_cast<size_t>(B)]; v != -1; v = next[v]) {
            if (A == B && u >= v) continue;
            const auto it = std::lower_bound(pa.begin() + static_cast<std::ptrdiff_t>(s),
                                             pa.begin() + static_cast<std::ptrdiff_t>(e), std::make_pair(u, v),
                                             [](const PairArc& x, const std::pair<int32_t, int32_t>& y) {
                                               return x.u != y.first ? x.u < y.first : x.v < y.second;
                                             });
            if (it == pa.begin() + static_cast<std::ptrdiff_t>(e) || it->u != u || it->v != v) {
              Cm.push_back(EdgePair{u, v});
            }
          }
        }
      }
      s = e;
    }
    std::sort(P.begin(), P.end());
    std::sort(Cp.begin(), Cp.end());
    std::sort(Cm.begin(), Cm.end());
    beam::EncodeOutput enc;
    enc.supernodes = static_cast<int64_t>(shead.size());
    enc.P.reserve(P.size());
    enc.Cp.reserve(Cp.size());
    enc.Cm.reserve(Cm.size());
    for (const EdgePair& e : P) enc.P.push_back(PairKey(e));
    for (const EdgePair& e : Cp) enc.Cp.push_back(PairKey(e));
    for (const EdgePair& e : Cm) enc.Cm.push_back(PairKey(e));
    beam::FinishEncoding(n, row_ptr[n], head, next, enc, out_dir, out);
    return 0;
  } catch (const std::exception& e) {
    g_encode_error = e.what();
    return -1;
  }
}

int beam_exact_partition_cost(int32_t n, const int64_t* row_ptr, const int32_t* col_idx, const int32_t* labels,
                              int64_t* cost) {
  try {
    std::vector<int64_t> sizes(static_cast<size_t>(n), 0);
    for (int32_t v = 0; v < n; ++v) {
      if (labels[v] < 0 || labels[v] >= n) throw std::invalid_argument("partition labels must be in [0, n)");
      sizes[static_cast<size_t>(labels[v])]++;
    }
    std::vector<uint64_t> keys;
    keys.reserve(static_cast<size_t>(row_ptr[n] / 2 + 1));
    for (int32_t u = 0; u < n; ++u) {
      for (int64_t k = row_ptr[u]; k < row_ptr[u + 1]; ++k) {
        const int32_t v = col_idx[k];
        if (u == v) throw std::invalid_argument("CostOracle does not support self-loops");
        if (u < v) {
          const uint32_t a = static_cast<uint32_t>(labels[u]);
          const uint32_t b = static_cast<uint32_t>(labels[v]);
          keys.push_back((static_cast<uint64_t>(std::min(a, b)) << 32) | std::max(a, b));
        }
      }
    }
    std::sort(keys.begin(), keys.end());
    int64_t total = 0;
    for (size_t s = 0; s < keys.size();) {
      size_t e = s + 1;
      while (e < keys.size() && keys[e] == keys[s]) ++e;
      const int32_t a = static_cast<int32_t>(keys[s] >> 32);
      const int32_t b = static_cast<int32_t>(keys[s] & 0xffffffffu);
      total += BlockCostHost(sizes[static_cast<size_t>(a)], sizes[static_cast<size_t>(b)],
                             static_cast<int64_t>(e - s), a == b);
      s = e;
    }
    *cost = total;
    return 0;
  } catch (const std::exception& e) {
    g_encode_error = e.what();
    return -1;
  }
}

uint64_t beam_partition_hash(int32_t n, const int32_t* labels) {
  uint64_t h = 1469598103934665603ULL;
  for (int32_t i = 0; i < n; ++i) {
    h ^= static_cast<uint64_t>(static_cast<uint32_t>(labels[i]));
    h *= 1099511628211ULL;
  }
  return h;
}

}  // extern "C"
