// samaya::read_mps on the fast reader (see read_mps_fast.hpp).
#include "read_mps_fast.hpp"

#include <atomic>
#include <cstdint>
#include <utility>
#include <vector>

#include "samaya/io.hpp"
#include "samaya/sparse_matrix.hpp"
#include "sg_mps.h"

namespace samaya_gb300 {
namespace {

std::atomic<long long> g_fast{0};
std::atomic<long long> g_samaya{0};

std::vector<std::string> split_names(const std::vector<char>& chars,
                                     const std::vector<int64_t>& start) {
  std::vector<std::string> names(start.size() - 1);
  for (size_t i = 0; i + 1 < start.size(); ++i) {
    names[i].assign(chars.data() + start[i], static_cast<size_t>(start[i + 1] - start[i]));
  }
  return names;
}

// The Model of a successful read (the handle is freed by the caller).
samaya::Model take(const sg_mps* h) {
  sg_mps_info info;
  sg_mps_get_info(h, &info);
  const size_t m = static_cast<size_t>(info.m), n = static_cast<size_t>(info.n);
  const size_t nnz = static_cast<size_t>(info.nnz);
  samaya::Model model;
  model.obj.resize(n);
  model.col_lower.resize(n);
  model.col_upper.resize(n);
  model.row_lower.resize(m);
  model.row_upper.resize(m);
  std::vector<int64_t> colptr(n + 1);
  std::vector<int32_t> rowidx(nnz);
  std::vector<double> vals(nnz);
  std::vector<uint8_t> integer(n);
  sg_mps_get_model(h, colptr.data(), rowidx.data(), vals.data(), model.obj.data(),
                   model.col_lower.data(), model.col_upper.data(), integer.data(),
                   model.row_lower.data(), model.row_upper.data());
  std::vector<char> name(static_cast<size_t>(info.name_bytes));
  std::vector<char> rows(static_cast<size_t>(info.row_name_bytes));
  std::vector<char> cols(static_cast<size_t>(info.col_name_bytes));
  std::vector<int64_t> row_start(m + 1), col_start(n + 1);
  sg_mps_get_names(h, name.data(), rows.data(), row_start.data(), cols.data(), col_start.data());
  model.name.assign(name.begin(), name.end());
  model.sense = info.maximize ? samaya::ObjSense::kMaximize : samaya::ObjSense::kMinimize;
  model.obj_offset = info.obj_offset;
  model.col_type.resize(n);
  for (size_t j = 0; j < n; ++j) {
    model.col_type[j] = integer[j] ? samaya::VarType::kInteger : samaya::VarType::kContinuous;
  }
  model.row_names = split_names(rows, row_start);
  model.col_names = split_names(cols, col_start);
  // samaya's SparseMatrix has one public builder, from_triplets; the columns arrive sorted by
  // row, merged and without zeros, so it keeps every entry as it is.
  std::vector<samaya::Triplet> triplets(nnz);
  for (size_t j = 0; j < n; ++j) {
    for (int64_t p = colptr[j]; p < colptr[j + 1]; ++p) {
      triplets[static_cast<size_t>(p)] = {rowidx[p], static_cast<samaya::Index>(j), vals[p]};
    }
  }
  model.A = samaya::SparseMatrix::from_triplets(static_cast<samaya::Index>(m),
                                                static_cast<samaya::Index>(n),
                                                std::move(triplets));
  return model;
}

}  // namespace

samaya::Model read_mps(const std::string& path, int threads) {
  sg_mps* h = nullptr;
  if (sg_mps_read(path.c_str(), threads, &h) != SG_OK) {
    ++g_samaya;
    return samaya::read_mps(path);
  }
  try {
    samaya::Model model = take(h);
    sg_mps_free(h);
    ++g_fast;
    return model;
  } catch (...) {
    sg_mps_free(h);
    throw;
  }
}

ReadCounts read_counts() { return ReadCounts{g_fast.load(), g_samaya.load()}; }

}  // namespace samaya_gb300
