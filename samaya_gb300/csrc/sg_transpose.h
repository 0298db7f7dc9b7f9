// Host CSC -> CSR of the constraint matrix (see sg_transpose.cpp).
#pragma once

#include <cstdint>

namespace sg {

// Rows of A from its CSC form (colptr n + 1 with colptr[0] = 0 and non-decreasing, rowidx and
// val colptr[n] long): kptr (m + 1), kidx and kval (colptr[n]), each row's columns in
// increasing order. Checks every row index and value; returns 0, or 1 with `why` set when one is
// out of range or not finite. Uses up to max_threads host threads.
int csc_to_csr(int m, int n, const int64_t* colptr, const int32_t* rowidx, const double* val,
               int* kptr, int* kidx, double* kval, int max_threads, const char** why);

// Column starts non-decreasing (and copied to int32 `tptr`, n + 1), every cost finite and no
// bound NaN (n + m entries): returns 0, or 1 with `why` set; *shared is set when every
// structural column has the first column's bounds. Uses up to max_threads host threads.
int check_columns(int m, int n, const int64_t* colptr, const double* cost, const double* lower,
                  const double* upper, int* tptr, bool* shared, int max_threads,
                  const char** why);

// Every row index in [0, m) and every value finite: returns 0, or 1 with `why` set. Uses up to
// max_threads host threads.
int check_nonzeros(int m, long long nnz, const int32_t* rowidx, const double* val,
                   int max_threads, const char** why);

}  // namespace sg
