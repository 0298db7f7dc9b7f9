// Reads each file named on standard input with the fast MPS reader (samaya_gb300/csrc/sg_mps.cpp,
// compiled into this program with AddressSanitizer and UBSan by tests/test_mps_sanitized.py) at
// 1, 3 and 7 threads, and prints per read: file, threads, status, columns, entries and a
// checksum of the arrays and names. Any memory error or undefined behaviour ends the program.
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <iterator>
#include <string>

#include "sg_mps.h"

namespace {

uint64_t fnv(uint64_t h, const void* p, size_t n) {
  const unsigned char* c = static_cast<const unsigned char*>(p);
  for (size_t i = 0; i < n; ++i) h = (h ^ c[i]) * 1099511628211ull;
  return h;
}

template <class V>
uint64_t mix(uint64_t h, const V& v) {
  return fnv(h, v.data(), v.size() * sizeof(v[0]));
}

}  // namespace

int main() {
  std::string path;
  while (std::getline(std::cin, path)) {
    std::ifstream in(path, std::ios::binary);
    const std::string text((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    for (int threads : {1, 3, 7}) {
      sg::MpsModel m;
      sg::MpsError e;
      const sg::MpsStatus st = sg::read_mps_text(text.data(), text.size(), threads, &m, &e);
      uint64_t h = 1469598103934665603ull;
      h = mix(mix(mix(mix(h, m.colptr), m.rowidx), m.vals), m.obj);
      h = mix(mix(mix(mix(h, m.col_lower), m.col_upper), m.row_lower), m.row_upper);
      h = mix(mix(mix(h, m.col_integer), m.row_names), m.col_names);
      std::printf("%s %d %d %d %zu %016llx %lld\n", path.c_str(), threads, static_cast<int>(st),
                  m.n, m.vals.size(), static_cast<unsigned long long>(h), e.line);
    }
  }
  return 0;
}
