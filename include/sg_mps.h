/* C ABI of the fast MPS reader (samaya_gb300).
 *
 * Reads an MPS file (free format, and fixed format where free MPS fails, as samaya's reader
 * does) into the arrays of samaya::Model (reference
 * include/samaya/model.hpp:44-60) on several host threads: the drop-in for samaya::read_mps
 * (reference src/io/mps_reader.cpp:530-541, declared in include/samaya/io.hpp:27-28) and its C
 * form samaya_read_mps (src/core/c_api.cpp:37-45) on linear models, which the CLI's
 * `--lp-method pdlp --gpu model.mps` path reads first (apps/cli/main.cpp:335).
 *
 * The model is the one read_mps builds, value for value: same number conversion
 * (std::from_chars, one leading '+' allowed, |v| >= 1e30 infinite), same defaults and bound
 * rules, A summed as SparseMatrix::from_triplets sums it (rows sorted within a column, duplicate
 * entries added, exact zeros dropped) and checked as Model::validate checks it. Where three or
 * more entries share a (row, column), they are added in file order (read_mps leaves that order
 * to its sort).
 *
 * What the reader does not read it declines, and the caller then calls samaya::read_mps:
 * SG_ERR_UNSUPPORTED for the quadratic sections (QUADOBJ, QMATRIX, QSECTION, QCMATRIX),
 * SG_ERR_PARSE for input that neither free nor fixed MPS reads (with the free reading's
 * message and line, as read_mps reports it), SG_ERR_IO when the file cannot be read. The message and line are in
 * sg_pdlp_last_error(). Host only: no GPU is used or needed.
 */
#ifndef SG_MPS_H
#define SG_MPS_H

#include <stddef.h>
#include <stdint.h>

#include "sg_pdlp.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sg_mps sg_mps;

/* Sizes of a model that was read. */
typedef struct sg_mps_info {
  int32_t m;                /* rows (E, L and G rows; N rows are the objective or dropped) */
  int32_t n;                /* columns */
  int64_t nnz;              /* entries of A */
  int32_t maximize;         /* 1 for OBJSENSE MAX / MAXIMIZE */
  int32_t num_integers;     /* columns marked integer (markers, BV, LI, UI) */
  double obj_offset;        /* minus the RHS entry of the objective row */
  int64_t name_bytes;       /* length of the NAME field (no terminating zero) */
  int64_t row_name_bytes;   /* total length of the row names */
  int64_t col_name_bytes;   /* total length of the column names */
} sg_mps_info;

/* Reads the MPS file at path (free MPS; where that fails, fixed MPS). threads: 0 picks the number of host threads from the file's size
 * (at most the hardware's and 64); N > 0 cuts every section into N line-aligned ranges. */
int sg_mps_read(const char* path, int threads, sg_mps** out);

/* The same for text held in memory (len bytes; need not end with a zero). */
int sg_mps_read_text(const char* text, size_t len, int threads, sg_mps** out);

int sg_mps_get_info(const sg_mps* h, sg_mps_info* info);

/* Copies the model into caller buffers; any pointer may be NULL to skip that array.
 * colptr n + 1, rowidx / vals nnz, obj / col_lower / col_upper / col_integer n,
 * row_lower / row_upper m. Infinite bounds are +-INFINITY. */
int sg_mps_get_model(const sg_mps* h, int64_t* colptr, int32_t* rowidx, double* vals,
                     double* obj, double* col_lower, double* col_upper, uint8_t* col_integer,
                     double* row_lower, double* row_upper);

/* Copies the names: name (name_bytes), the row names concatenated (row_name_bytes) with m + 1
 * starts, the column names (col_name_bytes) with n + 1 starts. Any pointer may be NULL. */
int sg_mps_get_names(const sg_mps* h, char* name, char* row_names, int64_t* row_starts,
                     char* col_names, int64_t* col_starts);

void sg_mps_free(sg_mps* h);

#ifdef __cplusplus
}
#endif

#endif /* SG_MPS_H */
