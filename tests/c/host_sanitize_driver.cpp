// The engine's host-side model code under AddressSanitizer and UBSan: sg_scale_model
// (samaya_gb300/csrc/sg_model.cpp) and the threaded checks and transpose of sg_pdlp_create
// (samaya_gb300/csrc/sg_transpose.cpp), compiled into this program by
// tests/test_host_sanitized.py. Each file named on standard input holds a model (int64 m, n,
// maximize, nnz; colptr n + 1 int64; rowidx nnz int32; vals nnz, obj n, col_lower n,
// col_upper n, row_lower m, row_upper m as float64). For each, <file>.out receives: the status
// of sg_scale_model and, when 0, its LpProblem (colptr, rowidx, vals, cost, lower, upper,
// col_scale, row_scale); the statuses of check_nonzeros and check_columns at 1 and 4 threads;
// and, when the checks pass, the CSR of csc_to_csr at 1 and 4 threads.
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "sg_pdlp.h"
#include "sg_transpose.h"

namespace {

template <class T>
bool get(std::ifstream& in, std::vector<T>& v, size_t n) {
  v.resize(n);
  return n == 0 || static_cast<bool>(in.read(reinterpret_cast<char*>(v.data()),
                                             static_cast<std::streamsize>(n * sizeof(T))));
}

template <class T>
void put(std::ofstream& out, const std::vector<T>& v) {
  if (!v.empty()) {
    out.write(reinterpret_cast<const char*>(v.data()),
              static_cast<std::streamsize>(v.size() * sizeof(T)));
  }
}

void put_int(std::ofstream& out, int64_t x) { out.write(reinterpret_cast<const char*>(&x), 8); }

}  // namespace

int main() {
  std::string path;
  while (std::getline(std::cin, path)) {
    std::ifstream in(path, std::ios::binary);
    int64_t head[4];
    if (!in.read(reinterpret_cast<char*>(head), sizeof(head))) return 2;
    const int m = static_cast<int>(head[0]), n = static_cast<int>(head[1]);
    const int maximize = static_cast<int>(head[2]);
    const size_t nnz = static_cast<size_t>(head[3]);
    std::vector<int64_t> colptr;
    std::vector<int32_t> rowidx;
    std::vector<double> vals, obj, cl, cu, rl, ru;
    if (!get(in, colptr, n + 1) || !get(in, rowidx, nnz) || !get(in, vals, nnz) ||
        !get(in, obj, n) || !get(in, cl, n) || !get(in, cu, n) || !get(in, rl, m) ||
        !get(in, ru, m)) {
      return 2;
    }
    std::ofstream out(path + ".out", std::ios::binary);
    std::vector<int64_t> lp_colptr(n + 1);
    std::vector<int32_t> lp_rowidx(nnz);
    std::vector<double> lp_val(nnz), cost(n + m), lower(n + m), upper(n + m), cs(n), rs(m);
    int64_t lp_nnz = 0;
    const int st = sg_scale_model(m, n, colptr.data(), rowidx.data(), vals.data(), obj.data(),
                                  cl.data(), cu.data(), rl.data(), ru.data(), maximize,
                                  lp_colptr.data(), lp_rowidx.data(), lp_val.data(), cost.data(),
                                  lower.data(), upper.data(), cs.data(), rs.data(), &lp_nnz);
    put_int(out, st);
    if (st == 0) {
      lp_rowidx.resize(static_cast<size_t>(lp_nnz));
      lp_val.resize(static_cast<size_t>(lp_nnz));
      put(out, lp_colptr);
      put(out, lp_rowidx);
      put(out, lp_val);
      put(out, cost);
      put(out, lower);
      put(out, upper);
      put(out, cs);
      put(out, rs);
    }
    // The checks of sg_pdlp_create, on the model's own columns (cost and bounds of n + m).
    std::vector<double> c2(obj), lo2(cl), up2(cu);
    c2.resize(n + m, 0.0);
    lo2.insert(lo2.end(), rl.begin(), rl.end());
    up2.insert(up2.end(), ru.begin(), ru.end());
    bool ok = true;
    for (int threads : {1, 4}) {
      const char* why = nullptr;
      const int a = sg::check_nonzeros(m, static_cast<long long>(nnz), rowidx.data(),
                                       vals.data(), threads, &why);
      std::vector<int> tptr(n + 1);
      bool shared = false;
      const int b = sg::check_columns(m, n, colptr.data(), c2.data(), lo2.data(), up2.data(),
                                      tptr.data(), &shared, threads, &why);
      put_int(out, a);
      put_int(out, b);
      ok = ok && a == 0 && b == 0;
    }
    if (ok) {
      for (int threads : {1, 4}) {
        std::vector<int> kptr(m + 1), kidx(nnz);
        std::vector<double> kval(nnz);
        const char* why = nullptr;
        const int c = sg::csc_to_csr(m, n, colptr.data(), rowidx.data(), vals.data(),
                                     kptr.data(), kidx.data(), kval.data(), threads, &why);
        put_int(out, c);
        put(out, kptr);
        put(out, kidx);
        put(out, kval);
      }
    }
  }
  return 0;
}
