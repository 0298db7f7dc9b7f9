// Fast reader of free-format MPS files (the work of samaya::read_mps, reference
// src/io/mps_reader.cpp, for linear models), spread over host threads. Host code only.
#pragma once

#include <cstddef>
#include <cstdint>
#include <memory>
#include <new>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

namespace sg {

// An allocator whose value-less construct leaves trivial elements uninitialised: large arrays are
// then first touched (and their pages faulted in) by the threads that fill them.
template <class T>
struct DefaultInit : std::allocator<T> {
  template <class U>
  struct rebind {
    using other = DefaultInit<U>;
  };
  DefaultInit() = default;
  template <class U>
  DefaultInit(const DefaultInit<U>&) noexcept {}
  template <class U>
  void construct(U* p) noexcept(std::is_nothrow_default_constructible<U>::value) {
    ::new (static_cast<void*>(p)) U;
  }
  template <class U, class... A>
  void construct(U* p, A&&... a) {
    ::new (static_cast<void*>(p)) U(std::forward<A>(a)...);
  }
};

template <class T>
using Buffer = std::vector<T, DefaultInit<T>>;

// A linear model read from MPS, laid out as samaya::Model (reference include/samaya/model.hpp:
// 44-60): A in CSC form (int64 column starts, int32 row indices sorted within each column, no
// explicit zeros), infinite bounds as +-inf, names as one character buffer per kind with
// count + 1 offsets.
struct MpsModel {
  std::string name;
  bool maximize = false;
  double obj_offset = 0.0;
  int32_t m = 0;
  int32_t n = 0;
  Buffer<double> obj, col_lower, col_upper;
  Buffer<uint8_t> col_integer;
  Buffer<double> row_lower, row_upper;
  Buffer<int64_t> colptr;
  Buffer<int32_t> rowidx;
  Buffer<double> vals;
  Buffer<char> row_names, col_names;
  Buffer<int64_t> row_name_start, col_name_start;
};

enum class MpsStatus {
  kOk = 0,
  kParseError,   // not valid free MPS (read_mps would go on to try fixed MPS)
  kUnsupported,  // valid input outside what this reader reads (the quadratic sections)
  kIoError,      // the file cannot be opened or read
  kTooLarge,     // more than 2^31 - 1 rows, columns or entries in one section range
  kOutOfMemory,
};

struct MpsError {
  long long line = 0;  // 1-based line of the error, 0 when it concerns the whole model
  std::string message;
};

// threads: 0 picks the number of host threads from the input's size (at most the hardware's
// and 64); N > 0 cuts every section into exactly N line-aligned byte ranges, one thread each.
MpsStatus read_mps_text(const char* text, size_t len, int threads, MpsModel* out,
                        MpsError* err);
MpsStatus read_mps_file(const char* path, int threads, MpsModel* out, MpsError* err);

}  // namespace sg
