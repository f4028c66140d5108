// Writing and measuring an encoded summary (shared by the host Encode and the
// device Encode): G.txt (supernodes in ascending representative order,
// members in list order), P.txt (superedges between supernode ids), Cp.txt
// and Cm.txt (node pairs), tab-separated, one pair per line, and the
// compression metrics of include/compression_metrics.hpp:39-98.
#pragma once

#include <cstdint>
#include <vector>

#include "beam_gb300.h"

namespace beam {

struct EncodeOutput {
  int64_t supernodes = 0;
  std::vector<unsigned long long> P, Cp, Cm;  // (a << 32 | b), sorted by (a, b)
};

// Fills `out` from the encoding and writes the four files when out_dir is not
// NULL; throws std::runtime_error on I/O errors.
void FinishEncoding(int32_t n, int64_t arcs, const int32_t* head, const int32_t* next, const EncodeOutput& enc,
                    const char* out_dir, beam_encoding* out);

}  // namespace beam
