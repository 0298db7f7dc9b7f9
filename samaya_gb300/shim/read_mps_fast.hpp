// The binding a samaya maintainer adds for the first step of the PDLP drop-in path: reading the
// model. samaya::read_mps (reference src/io/mps_reader.cpp:530-541) reads it for the CLI
// (apps/cli/main.cpp:335) and the C API (samaya_read_mps, src/core/c_api.cpp:37-45); this reads
// it with the fast reader's C ABI (include/sg_mps.h). It compiles against samaya's own headers
// and is not part of libsamaya_gb300.so.
#pragma once

#include <string>

#include "samaya/model.hpp"

namespace samaya_gb300 {

// Reads an MPS file into the Model samaya::read_mps returns for it. Linear models in free or
// fixed MPS go through the fast reader; everything it declines (the quadratic sections, an
// unreadable or invalid file) goes to samaya::read_mps, which then reads the file or throws its
// own error. Threads: 0 picks them from the file's size.
samaya::Model read_mps(const std::string& path, int threads = 0);

// How many reads of this process the fast reader answered and how many went to samaya's reader.
struct ReadCounts {
  long long fast = 0;
  long long samaya = 0;
};
ReadCounts read_counts();

}  // namespace samaya_gb300
