/*
 * oracle.h -- CPU restatement of the LeSpMV conversion and SpMV algorithms.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU library
 * (tests, the smoke check and the CPU-baseline leg of the benchmark).  The
 * product path never links or calls it.
 *
 * Every function restates one reference routine; the file:line of the routine
 * it follows (paths inside the LeSpMV project) is given beside each
 * declaration.  Index type is int32 (the reference's `int` instantiation),
 * value type is double (`_f64`) or float (`_f32`).
 *
 * Sliced formats (S-ELL, SELL-c-sigma, SELL-c-R) are returned "flattened":
 * the reference keeps one allocation per chunk (T** col_index/values); here the
 * chunks are concatenated in chunk order, each chunk row-major exactly as the
 * reference lays it out, so byte comparison of the flat arrays is comparison
 * of the reference's logical content.
 *
 * Parity pin: the outputs of these functions are checked against fixtures
 * produced by the reference's own code (compiled from its sources by
 * oracle/Makefile, target `ref`) in tests/test_oracle_golden.py.
 */
#ifndef SSPMV_ORACLE_H
#define SSPMV_ORACLE_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------- structural (index-only) steps ---------------- */

/* ELL width = max row nnz (include/sparse_conversion.h:197-203). */
int32_t oracle_ell_width(int32_t m, const int32_t *rowptr);

/* S-ELL per-chunk width, aligned up (include/sparse_conversion.h:272-296).
 * Writes row_width[ceil(m/C)], returns total slots sum(C*row_width). */
int64_t oracle_sell_row_width(int32_t m, const int32_t *rowptr, int32_t C,
                              int32_t align, int32_t *row_width);

/* SELL-c-sigma reorder: per sigma-slice sort of (nnz,row) pairs with
 * std::greater, i.e. nnz descending, ties -> larger row first
 * (include/sparse_conversion.h:366-400).  sigma <= 0 means one slice of all
 * rows (SELL-c-R, include/sparse_conversion.h:501-523).  Returns 0, or -1 when
 * sigma % C != 0 (the reference exits, :357-361). */
int oracle_sell_cs_reorder(int32_t m, const int32_t *rowptr, int32_t sigma,
                           int32_t C, int32_t *reorder);

/* chunk_len over reordered rows, aligned up (include/sparse_conversion.h:405-433).
 * Writes chunk_len[ceil(m/C)], returns total slots sum(C*chunk_len). */
int64_t oracle_sell_cs_chunk_len(int32_t m, const int32_t *rowptr,
                                 const int32_t *reorder, int32_t C,
                                 int32_t align, int32_t *chunk_len);

/* DIA diagonal map in first-encounter order of a row-major scan
 * (include/sparse_conversion.h:626-649).  diag_map has m+n entries
 * (index = m - i + j), -1 where unoccupied.  Returns complete_ndiags. */
int32_t oracle_dia_map(int32_t m, int32_t n, const int32_t *rowptr,
                       const int32_t *col, int32_t *diag_map);

/* BSR block-row pointer (include/sparse_conversion.h:817-848).  Returns nnzb.
 * row_ptr has mb+1 entries. */
int32_t oracle_bsr_row_ptr(int32_t m, int32_t n, const int32_t *rowptr,
                           const int32_t *col, int32_t r, int32_t c,
                           int32_t *row_ptr);
/* BSR block column indices, ascending per block row
 * (include/sparse_conversion.h:861-888). */
void oracle_bsr_colindex(int32_t m, int32_t n, const int32_t *rowptr,
                         const int32_t *col, int32_t r, int32_t c,
                         const int32_t *row_ptr, int32_t *colindex);

/* CSR5 descriptor geometry (include/sparse_conversion.h:958-996). */
typedef struct {
    int32_t sigma, omega;
    int32_t bit_y_offset, bit_scansum_offset, num_packets;
    int32_t p;                     /* number of tiles (_p) */
    int32_t num_offsets;
    int32_t tail_partition_start;
} oracle_csr5_geom;

/* Geometry only.  Returns 0, or -1 when the bit fields do not fit. */
int oracle_csr5_geometry(int32_t nnz, int32_t sigma, int32_t omega,
                         oracle_csr5_geom *g);
/* tile_ptr (p+1), tile_desc (p*omega*num_packets), tile_desc_offset_ptr (p+1);
 * fills g->num_offsets and g->tail_partition_start
 * (include/sparse_conversion.h:1024-1252). */
void oracle_csr5_descriptors(int32_t m, const int32_t *rowptr,
                             oracle_csr5_geom *g, uint32_t *tile_ptr,
                             uint32_t *tile_desc,
                             int32_t *tile_desc_offset_ptr);
/* tile_desc_offset (num_offsets) (include/sparse_conversion.h:1254-1358). */
void oracle_csr5_offsets(int32_t m, const int32_t *rowptr,
                         const oracle_csr5_geom *g, const uint32_t *tile_ptr,
                         const uint32_t *tile_desc,
                         const int32_t *tile_desc_offset_ptr,
                         int32_t *tile_desc_offset);
/* In-place per-tile transpose of an array of elem_size-byte items
 * (include/csr5_utils.h:11-87, R2C direction). */
void oracle_csr5_transpose(int32_t nnz, const oracle_csr5_geom *g,
                           const uint32_t *tile_ptr, void *data,
                           int32_t elem_size);

/* ---------------- value-typed steps ---------------- */
#define ORACLE_DECLARE(V, S)                                                   \
  /* stable counting sort, duplicates kept (include/sparse_conversion.h:30-91) */ \
  void oracle_coo_to_csr_##S(int32_t m, int32_t nnz, const int32_t *ri,        \
                             const int32_t *ci, const V *v, int32_t *rowptr,   \
                             int32_t *col, V *val);                            \
  /* include/sparse_conversion.h:145-168 */                                    \
  void oracle_csr_to_coo_##S(int32_t m, const int32_t *rowptr,                 \
                             const int32_t *col, const V *val, int32_t *ri,    \
                             int32_t *ci, V *v);                               \
  /* ld: 0 RowMajor, 1 ColMajor (include/sparse_conversion.h:205-246) */       \
  void oracle_csr_to_ell_##S(int32_t m, const int32_t *rowptr,                 \
                             const int32_t *col, const V *val, int32_t width,  \
                             int32_t ld, int32_t *ell_col, V *ell_val);        \
  /* include/sparse_conversion.h:298-333 (flattened chunks) */                 \
  void oracle_csr_to_sell_##S(int32_t m, const int32_t *rowptr,                \
                              const int32_t *col, const V *val, int32_t C,     \
                              const int32_t *row_width, int32_t *col_flat,     \
                              V *val_flat);                                    \
  /* include/sparse_conversion.h:435-476 and :571-595 (flattened chunks) */    \
  void oracle_csr_to_sell_cs_##S(int32_t m, const int32_t *rowptr,             \
                                 const int32_t *col, const V *val,             \
                                 const int32_t *reorder, int32_t C,            \
                                 const int32_t *chunk_len, int32_t *col_flat,  \
                                 V *val_flat);                                 \
  /* include/sparse_conversion.h:739-762; data has ndiags*stride entries */    \
  void oracle_csr_to_dia_##S(int32_t m, int32_t n, const int32_t *rowptr,      \
                             const int32_t *col, const V *val,                 \
                             const int32_t *diag_map, int32_t ndiags,          \
                             int32_t stride, int64_t *offsets, V *data);       \
  /* include/sparse_conversion.h:784-923 (r=c=1 copies CSR) */                 \
  void oracle_csr_to_bsr_##S(int32_t m, int32_t n, const int32_t *rowptr,      \
                             const int32_t *col, const V *val, int32_t r,      \
                             int32_t c, const int32_t *row_ptr,                \
                             const int32_t *colindex, V *data);                \
  /* ---- SpMV  y = alpha*A*x + beta*y ---- */                                 \
  /* src/spmv_csr.cpp:34-62,138-162 (nnz-balanced row partition) */            \
  void oracle_spmv_csr_##S(int32_t m, const int32_t *rowptr,                   \
                           const int32_t *col, const V *val, V alpha,          \
                           const V *x, V beta, V *y, int nthreads);            \
  /* src/spmv_coo.cpp:38-78 (atomic scatter) */                                \
  void oracle_spmv_coo_##S(int32_t m, int32_t nnz, const int32_t *ri,          \
                           const int32_t *ci, const V *v, V alpha, const V *x, \
                           V beta, V *y, int nthreads);                        \
  /* src/spmv_ell.cpp:17-68,128-222 */                                         \
  void oracle_spmv_ell_##S(int32_t m, int32_t width, int32_t ld,               \
                           const int32_t *ell_col, const V *ell_val, V alpha,  \
                           const V *x, V beta, V *y, int nthreads);            \
  /* src/spmv_s_ell.cpp:121-200 */                                             \
  void oracle_spmv_sell_##S(int32_t m, int32_t C, const int32_t *row_width,    \
                            const int32_t *col_flat, const V *val_flat,        \
                            V alpha, const V *x, V beta, V *y, int nthreads);  \
  /* src/spmv_sell_c_sigma.cpp:104-188; src/spmv_sell_c_R.cpp (same) */        \
  void oracle_spmv_sell_cs_##S(int32_t m, int32_t C, const int32_t *reorder,   \
                               const int32_t *chunk_len,                       \
                               const int32_t *col_flat, const V *val_flat,     \
                               V alpha, const V *x, V beta, V *y,              \
                               int nthreads);                                  \
  /* src/spmv_dia.cpp:16-44 (row-parallel restatement) */                      \
  void oracle_spmv_dia_##S(int32_t m, int32_t n, int32_t ndiags,               \
                           int32_t stride, const int64_t *offsets,             \
                           const V *data, V alpha, const V *x, V beta, V *y,   \
                           int nthreads);                                      \
  /* src/spmv_bsr.cpp:121-213 */                                               \
  void oracle_spmv_bsr_##S(int32_t m, int32_t r, int32_t c, int32_t mb,        \
                           const int32_t *row_ptr, const int32_t *colindex,    \
                           const V *data, V alpha, const V *x, V beta, V *y,   \
                           int nthreads);                                      \
  /* FP64 CSR result on V inputs plus per-row sum|a_ij x_j| (the tolerance    \
   * scale) for k right-hand sides, X[col*ldx+r], Y[row*ldy+r]                 \
   * (src/spmv_csr.cpp:65-91 in double). y_out/absum are m*k, ld k. */         \
  void oracle_spmm_ref_##S(int32_t m, const int32_t *rowptr,                   \
                           const int32_t *col, const V *val, int32_t k,        \
                           const V *x, int64_t ldx, double alpha,              \
                           double beta, const V *y0, int64_t ldy,              \
                           double *y_out, double *absum, int nthreads);        \
  /* include/sparse_operation.h:76-94 */                                       \
  V oracle_max_rel_error_##S(const V *a, const V *b, int64_t n);

ORACLE_DECLARE(double, f64)
ORACLE_DECLARE(float, f32)

int oracle_max_threads(void);

/* Matrix features (class MTX, src/sparse_features.cpp:122-968) of a general
 * CSR matrix with T x T tiles: F receives the 62 values in the library's
 * feature order; nnz_by_tiles / uniq_rb / uniq_cb (T*T each, may be NULL)
 * receive the per-tile counts. */
void oracle_features(int32_t m, int32_t n, const int32_t *rowptr, const int32_t *col, const double *val,
                     int32_t T, double *F, int32_t *nnz_by_tiles, int32_t *uniq_rb, int32_t *uniq_cb);

/* GrX tile-group features (CalculateTilesExtraFeatures under BSR_ANA and
 * AnalyzeTile_Group, src/sparse_features.cpp:884-1065), restated with the
 * reference's literal loops over dense BestDimForBSR-sized tiles: out[0..3] =
 * GrX_uniqR, GrX_uniqC, GrX_potReuseR, GrX_potReuseC (-1 where the tile is
 * smaller than X).  The reference's own code for these is not built (its
 * BSR_ANA block does not compile), so this restatement is not pinned to
 * reference output. */
void oracle_grx(int32_t m, int32_t n, const int32_t *rowptr, const int32_t *col, const double *val, int32_t T,
                int32_t X, double *out);

#ifdef __cplusplus
}
#endif
#endif
