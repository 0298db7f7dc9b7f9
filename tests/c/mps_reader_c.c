/* A plain C99 caller of the engine library's C ABI (include/sg_mps.h, include/sg_pdlp.h): reads
 * an MPS file with the fast reader and prints its sizes, objective sense and offset, the sum of
 * its entries and its first row and column names; then asks for a GPU. Built and run by
 * tests/test_cabi.py on a machine without one. */
#include <stdio.h>
#include <stdlib.h>

#include "sg_mps.h"
#include "sg_pdlp.h"

int main(int argc, char** argv) {
  if (argc != 2) {
    fprintf(stderr, "usage: %s model.mps\n", argv[0]);
    return 2;
  }
  sg_mps* h = NULL;
  int rc = sg_mps_read(argv[1], 0, &h);
  if (rc != SG_OK) {
    printf("error %d %s: %s\n", rc, sg_pdlp_error_string(rc), sg_pdlp_last_error());
    return 0;
  }
  sg_mps_info info;
  sg_mps_get_info(h, &info);
  int64_t* colptr = malloc(sizeof(int64_t) * (size_t)(info.n + 1));
  int32_t* rowidx = malloc(sizeof(int32_t) * (size_t)(info.nnz > 0 ? info.nnz : 1));
  double* vals = malloc(sizeof(double) * (size_t)(info.nnz > 0 ? info.nnz : 1));
  char* rows = malloc((size_t)info.row_name_bytes + 1);
  char* cols = malloc((size_t)info.col_name_bytes + 1);
  int64_t* rs = malloc(sizeof(int64_t) * (size_t)(info.m + 1));
  int64_t* cs = malloc(sizeof(int64_t) * (size_t)(info.n + 1));
  sg_mps_get_model(h, colptr, rowidx, vals, NULL, NULL, NULL, NULL, NULL, NULL);
  sg_mps_get_names(h, NULL, rows, rs, cols, cs);
  double sum = 0.0;
  for (int64_t k = 0; k < info.nnz; ++k) sum += vals[k];
  printf("read %d %d %lld %d %d %.17g %.17g %.*s %.*s\n", info.m, info.n, (long long)info.nnz,
         info.maximize, info.num_integers, info.obj_offset, sum, (int)(rs[1] - rs[0]), rows,
         (int)(cs[1] - cs[0]), cols);
  sg_mps_free(h);
  free(colptr);
  free(rowidx);
  free(vals);
  free(rows);
  free(cols);
  free(rs);
  free(cs);
  int major = 0, minor = 0;
  char name[64];
  printf("available %d\n", sg_pdlp_available(&major, &minor, name, sizeof(name)));
  return 0;
}
