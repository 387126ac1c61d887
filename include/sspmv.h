/*
 * sspmv.h -- C ABI of the GB300-native sparse SpMV library (libsspmv.so).
 *
 * Drop-in boundary for LeSpMV's per-format SpMV path.  The reference exposes
 * C++ templates over <IndexType, ValueType>; this ABI exposes one plain-C
 * entry point per reference routine with the value type carried at run time
 * in the matrix struct (SSPMV_F32 / SSPMV_F64, int32 indices).
 *
 *   reference (LeSpMV project paths)                  this ABI
 *   ------------------------------------------------  ---------------------------
 *   struct <Fmt>_Matrix (include/sparse_format.h)     sspmv_<fmt> (device arrays)
 *   coo_to_csr / csr_to_<fmt>                         sspmv_coo_to_csr /
 *     (include/sparse_conversion.h)                     sspmv_csr_to_<fmt>
 *   LeSpMV_<fmt>(alpha, A, x, beta, y)                sspmv_LeSpMV_<fmt>
 *     (src/spmv_<fmt>.cpp)                            (+ sspmv_spmm_<fmt>, k RHS)
 *   delete_host_matrix (include/sparse_format.h)      sspmv_delete_<fmt>
 *   read_csr_matrix (utils/sparse_io.cpp)             sspmv_read_mtx
 *
 * Conventions
 *  - All matrix arrays and x / y live in device memory (HBM).  Matrices made
 *    by this library own their arrays; free them with sspmv_delete_<fmt>.
 *  - Every call is ordered on the given CUDA stream.  SpMV / SpMM calls do not
 *    synchronize; converters synchronize their stream (they size outputs).
 *  - Errors are returned as sspmv_status; nothing exits or throws.  The text
 *    of the last error of the calling thread is sspmv_last_error().
 *  - Parameters passed as 0 take the reference's shipped defaults:
 *    chunk width C = 4, sigma = 16384, alignment = 64 / sizeof(value),
 *    BSR block = 16 x (64 / sizeof(value)), max_diags = 10240,
 *    CSR5 sigma = 16, omega = 64 / sizeof(value)
 *    (include/general_config.h:17-26, include/plat_config.h:20-25).
 *  - y = alpha*A*x + beta*y for every row, including rows without nonzeros.
 *    beta == 0 never reads y.
 *  - SpMM: k right-hand sides, X is row-major num_cols x k with leading
 *    dimension ldx >= k (X[col*ldx + r]); Y likewise with ldy.
 */
#ifndef SSPMV_H
#define SSPMV_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *sspmv_stream_t; /* == cudaStream_t */

typedef enum {
    SSPMV_OK = 0,
    SSPMV_INVALID_ARG = 1,
    SSPMV_INFEASIBLE = 2,       /* e.g. DIA over max_diags (reference exits) */
    SSPMV_OUT_OF_MEMORY = 3,
    SSPMV_BUDGET_EXCEEDED = 4,
    SSPMV_DEVICE_TIMEOUT = 5,
    SSPMV_CUDA_ERROR = 6,
    SSPMV_NOT_SUPPORTED = 7
} sspmv_status;

typedef enum { SSPMV_F32 = 0, SSPMV_F64 = 1 } sspmv_value_type;
typedef enum { SSPMV_ROW_MAJOR = 0, SSPMV_COL_MAJOR = 1 } sspmv_leading_dimension;

/* Matrix_Features (include/sparse_format.h:50-68).  `partition` of the
 * reference (CPU thread split) is replaced by `priv`: library-private device
 * state (cached schedules, carry buffers), created on first use. */
typedef struct {
    int64_t num_rows;
    int64_t num_cols;
    int64_t num_nnzs;
    double sparsity;
    double time, gflops, gbytes;
    int32_t tag;
    int32_t kernel_flag; /* 0 = library default kernel; see each format */
    int32_t value_type;  /* sspmv_value_type */
    int32_t owns;        /* 1: arrays allocated by the library */
    void *priv;
} sspmv_features;

/* COO_Matrix (include/sparse_format.h:77-86) */
typedef struct {
    sspmv_features f;
    int32_t *row_index;
    int32_t *col_index;
    void *values;
    int32_t row_sorted; /* 1 when row_index is non-decreasing */
} sspmv_coo;

/* CSR_Matrix (include/sparse_format.h:96-104) */
typedef struct {
    sspmv_features f;
    int32_t *row_offset;
    int32_t *col_index;
    void *values;
} sspmv_csr;

/* ELL_Matrix (include/sparse_format.h:192-205).  Device storage is always
 * column-major (slot k of row i at k*num_rows + i, padding col -1 / value 0);
 * `ld` records the layout the reference would hold, used by the export. */
typedef struct {
    sspmv_features f;
    int32_t ld;
    int32_t max_row_width;
    int32_t min_row_width;
    int32_t *col_index;
    void *values;
} sspmv_ell;

/* S_ELL_Matrix (include/sparse_format.h:214-238).  The reference keeps one
 * allocation per chunk (T**); here all chunks share one slab and chunk c
 * starts at slot chunk_ptr[c].  Inside a chunk storage is slot-major (slot k
 * of the chunk's row r at chunk_ptr[c] + k*sliceWidth + r), so C consecutive
 * rows are read together; the export returns the reference's row-major
 * chunks. */
typedef struct {
    sspmv_features f;
    int32_t sliceWidth; /* C rows per chunk */
    int32_t chunk_num;
    int32_t alignment;
    int32_t *row_width; /* [chunk_num], multiples of alignment */
    int64_t *chunk_ptr; /* [chunk_num + 1] */
    int64_t total_slots;
    int32_t *col_index;
    void *values;
} sspmv_s_ell;

/* SELL_C_Sigma_Matrix (include/sparse_format.h:245-270); chunk storage as
 * sspmv_s_ell.  reorder[i] is the original row stored at position i. */
typedef struct {
    sspmv_features f;
    int32_t sliceWidth_Sigma;
    int32_t chunkWidth_C;
    int32_t sliceNum;
    int32_t chunkNum;
    int32_t validchunkNum;
    int32_t chunk_num_per_slice;
    int32_t alignment;
    int32_t *reorder;   /* [num_rows] */
    int32_t *chunk_len; /* [validchunkNum] */
    int64_t *chunk_ptr; /* [validchunkNum + 1] */
    int64_t total_slots;
    int32_t *col_index;
    void *values;
} sspmv_sell_c_sigma;

/* SELL_C_R_Matrix (include/sparse_format.h:275-295): SELL-c-sigma with one
 * slice holding every row. */
typedef struct {
    sspmv_features f;
    int32_t chunkWidth_C;
    int32_t validchunkNum;
    int32_t alignment;
    int32_t *reorder;
    int32_t *chunk_len;
    int64_t *chunk_ptr;
    int64_t total_slots;
    int32_t *col_index;
    void *values;
} sspmv_sell_c_R;

/* DIA_Matrix (include/sparse_format.h:173-185): diagonal d (offset
 * diag_offsets[d]) stored at diag_data[d*stride + row], zero filled. */
typedef struct {
    sspmv_features f;
    int32_t stride;
    int32_t complete_ndiags;
    int64_t *diag_offsets;
    void *diag_data;
} sspmv_dia;

/* BSR_Matrix (include/sparse_format.h:113-130): blockDim_r x blockDim_c
 * blocks, row-major inside a block, block columns ascending per block row. */
typedef struct {
    sspmv_features f;
    int64_t blockDim_r;
    int64_t blockDim_c;
    int64_t blockNNZ;
    int64_t mb;
    int64_t nb;
    int64_t nnzb;
    int32_t *row_ptr;        /* [mb + 1] */
    int32_t *block_colindex; /* [nnzb] */
    void *block_data;        /* [nnzb * blockNNZ] */
} sspmv_bsr;

/* CSR5_Matrix (include/sparse_format.h:141-166): the CSR arrays (col_index /
 * values transposed tile by tile) plus the tile pointer and descriptors. */
typedef struct {
    sspmv_features f;
    int32_t *row_offset;
    int32_t *col_index;
    void *values;
    int32_t sigma;
    int32_t omega;
    int32_t bit_y_offset;
    int32_t bit_scansum_offset;
    int32_t num_packets;
    int32_t num_offsets;
    int32_t _p;
    int32_t tail_partition_start;
    uint32_t *tile_ptr;             /* [_p + 1] */
    uint32_t *tile_desc;            /* [_p * omega * num_packets] */
    int32_t *tile_desc_offset_ptr;  /* [_p + 1] */
    int32_t *tile_desc_offset;      /* [num_offsets] */
} sspmv_csr5;

/* ---------------- status / memory ---------------- */
const char *sspmv_status_string(sspmv_status s);
const char *sspmv_last_error(void);
const char *sspmv_version(void);
/* Number of kernels this library has launched in the process so far. */
int64_t sspmv_launch_count(void);
/* Frees the plan of a matrix (pass &A->f): the per-matrix schedule and carry
 * buffers the first SpMV builds, which sspmv_delete_<fmt> otherwise frees.
 * The frees are ordered on `stream` (work queued there before may still use
 * the plan) and nothing waits for the device; the next SpMV builds a new
 * plan.  The kernel choice (kernel_flag and the sspmv_set_kernel parameter)
 * is kept; a nonzero parameter is kept in a host-side record that
 * sspmv_delete_<fmt> frees.  For callers that wrap arrays per call (sspmv_csr_wrap) and must not
 * keep state between calls.  No reference counterpart. */
sspmv_status sspmv_release_plan(sspmv_features *f, sspmv_stream_t stream);
/* Selects the SpMV kernel of a matrix (pass &A->f): kernel_flag as in each
 * format's LeSpMV entry, param a kernel parameter (0 lets the library
 * choose): CSR vector kernel: lanes per row 1..32; CSR row-block kernel:
 * nonzeros per block window (512, 1024, 2048, 4096); S-ELL, SELL-c-sigma,
 * SELL-c-R: the slots a row's thread reads before the rest of the row moves
 * to the overflow CSR pass (default: a cost model over the row lengths).
 * Used by the autotuner. */
sspmv_status sspmv_set_kernel(sspmv_features *f, int32_t kernel_flag, int32_t param);

/* Number of bounded device-side waits (a kernel waiting for its own bulk
 * copies into shared memory: the CSR row-block and the staged DIA kernels)
 * that gave up since the library was loaded, on
 * the current device.  A wait that gives up leaves its kernel's output
 * incomplete; 0 in every correct run.  No reference counterpart (the
 * reference has no device code).  Synchronizes the device. */
sspmv_status sspmv_wait_timeouts(int64_t *count);

/* ---------------- CSR creation ---------------- */
/* Device CSR from arrays.  from_host != 0: copies host arrays to library-
 * owned device memory.  from_host == 0: copies device arrays. */
sspmv_status sspmv_csr_create(sspmv_csr *out, int32_t value_type, int64_t num_rows, int64_t num_cols,
                              int64_t num_nnzs, const int32_t *row_offset, const int32_t *col_index,
                              const void *values, int32_t from_host, sspmv_stream_t stream);
/* Wrap caller-owned device arrays (nothing copied, nothing freed). */
sspmv_status sspmv_csr_wrap(sspmv_csr *out, int32_t value_type, int64_t num_rows, int64_t num_cols,
                            int64_t num_nnzs, int32_t *row_offset, int32_t *col_index, void *values);
/* Copy the CSR arrays to host buffers (row_offset: num_rows+1, col_index and
 * values: num_nnzs). */
sspmv_status sspmv_csr_export(const sspmv_csr *A, int32_t *row_offset, int32_t *col_index, void *values,
                              sspmv_stream_t stream);
sspmv_status sspmv_delete_csr(sspmv_csr *A);

/* ---------------- SpMV / SpMM ---------------- */
/* LeSpMV_csr (src/spmv_csr.cpp:165-185).  kernel_flag 0 (default):
 * nonzero-split stream kernel (256 nonzeros per warp; matrices with runs of
 * more than 256 empty rows use merge-path); 2: nnz-balanced merge-path
 * kernel; 1: vector-per-row kernel (param: lanes per row, 1..32); 3: row-block
 * kernel for matrices whose rows all have at most 64 nonzeros (one CTA per
 * block of whole rows, param: nonzeros per block window, 512..4096; one
 * right-hand side; other matrices and k > 1 run the default kernel); 4:
 * software-pipelined row kernel (each lane keeps three rows' loads in
 * flight; param bit 0 set: values loaded one row ahead with the columns,
 * else with the x gathers; param bits 1-2: log2 of the lanes per row, 1 to
 * 8; param bit 3 set: CTAs of 1024 threads instead of 256 where the
 * register budget allows; rows of at most 12 nonzeros with one lane per row,
 * 8 per lane with more; one right-hand side; other matrices and k > 1 run
 * the default kernel). */
sspmv_status sspmv_LeSpMV_csr(double alpha, const sspmv_csr *A, const void *x, double beta, void *y,
                              sspmv_stream_t stream);
sspmv_status sspmv_spmm_csr(double alpha, const sspmv_csr *A, int32_t k, const void *X, int64_t ldx,
                            double beta, void *Y, int64_t ldy, sspmv_stream_t stream);
/* Allocation-free CSR SpMV (no counterpart in the reference).  Same result as
 * sspmv_LeSpMV_csr's merge-path kernel, for callers that cannot allocate
 * device memory at SpMV time: a solver or serving loop whose device heap is
 * owned by its own pool allocator, a latency-bound loop that cannot take
 * cudaMalloc's implicit device synchronisation, a component held to a device
 * memory budget enforced elsewhere.  Its scratch (tile split points and
 * carries) lives in one fixed 16 MiB device array that every GPU loading this
 * library keeps until exit; no per-matrix plan is built and nothing is
 * allocated.  Limit: num_rows + num_nnzs <= 238,594,048 (116,501 tiles of
 * 2048 merge items); larger matrices return SSPMV_INVALID_ARG.  The first call
 * on a device (and the first after a cudaDeviceReset of it) looks up the
 * array's address with that device current: make it before any stream
 * capture.  All calls share the array: calls that overlap on
 * the GPU race and must be serialised by the caller.  Nothing in the array
 * needs clearing between calls (each call writes every entry it reads). */
sspmv_status sspmv_LeSpMV_csr_noalloc(double alpha, const sspmv_csr *A, const void *x, double beta, void *y,
                                      sspmv_stream_t stream);

/* ---------------- ELL ---------------- */
/* csr_to_ell (include/sparse_conversion.h:187-248) */
sspmv_status sspmv_csr_to_ell(const sspmv_csr *csr, int32_t ld, sspmv_ell *out, sspmv_stream_t stream);
/* coo_to_ell (include/sparse_conversion.h:94-142): each row's entries in COO
 * order; ld is ignored and the result is RowMajor, as in the reference. */
sspmv_status sspmv_coo_to_ell(const sspmv_coo *coo, int32_t ld, sspmv_ell *out, sspmv_stream_t stream);
/* LeSpMV_ell (src/spmv_ell.cpp:225-247): one thread per row over the
 * column-major slots, stopping at the row's first padding slot. */
sspmv_status sspmv_LeSpMV_ell(double alpha, const sspmv_ell *A, const void *x, double beta, void *y,
                              sspmv_stream_t stream);
sspmv_status sspmv_spmm_ell(double alpha, const sspmv_ell *A, int32_t k, const void *X, int64_t ldx,
                            double beta, void *Y, int64_t ldy, sspmv_stream_t stream);
/* col_index / values: num_rows*max_row_width each, in A->ld layout. */
sspmv_status sspmv_ell_export(const sspmv_ell *A, int32_t *col_index, void *values, sspmv_stream_t stream);
sspmv_status sspmv_delete_ell(sspmv_ell *A);

/* ---------------- S-ELL ---------------- */
/* csr_to_sell (include/sparse_conversion.h:258-334); chunkwidth / alignment
 * 0 = reference defaults (4, 64/sizeof(value)). */
sspmv_status sspmv_csr_to_sell(const sspmv_csr *csr, int32_t chunkwidth, int32_t alignment, sspmv_s_ell *out,
                               sspmv_stream_t stream);
/* LeSpMV_sell (src/spmv_s_ell.cpp:203-224) */
sspmv_status sspmv_LeSpMV_sell(double alpha, const sspmv_s_ell *A, const void *x, double beta, void *y,
                               sspmv_stream_t stream);
sspmv_status sspmv_spmm_sell(double alpha, const sspmv_s_ell *A, int32_t k, const void *X, int64_t ldx,
                             double beta, void *Y, int64_t ldy, sspmv_stream_t stream);
/* row_width: chunk_num; col_index / values: total_slots, chunks in order,
 * row-major inside a chunk (the reference's layout). */
sspmv_status sspmv_sell_export(const sspmv_s_ell *A, int32_t *row_width, int32_t *col_index, void *values,
                               sspmv_stream_t stream);
sspmv_status sspmv_delete_sell(sspmv_s_ell *A);

/* ---------------- SELL-c-sigma ---------------- */
/* csr_to_sell_c_sigma (include/sparse_conversion.h:337-479): rows sorted by
 * nonzero count, descending, inside each sigma-slice (ties: larger row
 * first).  slicewidth % chunkwidth != 0 -> SSPMV_INVALID_ARG (the reference
 * exits).  0 = defaults (16384, 4, 64/sizeof(value)). */
sspmv_status sspmv_csr_to_sell_c_sigma(const sspmv_csr *csr, int32_t slicewidth, int32_t chunkwidth,
                                       int32_t alignment, sspmv_sell_c_sigma *out, sspmv_stream_t stream);
/* LeSpMV_sell_c_sigma (src/spmv_sell_c_sigma.cpp:190-211) */
sspmv_status sspmv_LeSpMV_sell_c_sigma(double alpha, const sspmv_sell_c_sigma *A, const void *x, double beta,
                                       void *y, sspmv_stream_t stream);
sspmv_status sspmv_spmm_sell_c_sigma(double alpha, const sspmv_sell_c_sigma *A, int32_t k, const void *X,
                                     int64_t ldx, double beta, void *Y, int64_t ldy, sspmv_stream_t stream);
sspmv_status sspmv_sell_c_sigma_export(const sspmv_sell_c_sigma *A, int32_t *reorder, int32_t *chunk_len,
                                       int32_t *col_index, void *values, sspmv_stream_t stream);
sspmv_status sspmv_delete_sell_c_sigma(sspmv_sell_c_sigma *A);

/* ---------------- SELL-c-R ---------------- */
/* csr_to_sell_c_R (include/sparse_conversion.h:483-598) */
sspmv_status sspmv_csr_to_sell_c_R(const sspmv_csr *csr, int32_t chunkwidth, int32_t alignment,
                                   sspmv_sell_c_R *out, sspmv_stream_t stream);
/* LeSpMV_sell_c_R (src/spmv_sell_c_R.cpp:190-211) */
sspmv_status sspmv_LeSpMV_sell_c_R(double alpha, const sspmv_sell_c_R *A, const void *x, double beta, void *y,
                                   sspmv_stream_t stream);
sspmv_status sspmv_spmm_sell_c_R(double alpha, const sspmv_sell_c_R *A, int32_t k, const void *X, int64_t ldx,
                                 double beta, void *Y, int64_t ldy, sspmv_stream_t stream);
sspmv_status sspmv_sell_c_R_export(const sspmv_sell_c_R *A, int32_t *reorder, int32_t *chunk_len,
                                   int32_t *col_index, void *values, sspmv_stream_t stream);
sspmv_status sspmv_delete_sell_c_R(sspmv_sell_c_R *A);

/* ---------------- COO ---------------- */
/* Device COO from arrays (from_host as sspmv_csr_create); row_sorted is set
 * when the host rows are non-decreasing (device input: 0). */
sspmv_status sspmv_coo_create(sspmv_coo *out, int32_t value_type, int64_t num_rows, int64_t num_cols,
                              int64_t num_nnzs, const int32_t *row_index, const int32_t *col_index,
                              const void *values, int32_t from_host, sspmv_stream_t stream);
/* csr_to_coo (include/sparse_conversion.h:145-168) */
sspmv_status sspmv_csr_to_coo(const sspmv_csr *csr, sspmv_coo *out, sspmv_stream_t stream);
/* coo_to_csr (include/sparse_conversion.h:30-91, compact = false) */
sspmv_status sspmv_coo_to_csr(const sspmv_coo *coo, sspmv_csr *out, sspmv_stream_t stream);
/* LeSpMV_coo (src/spmv_coo.cpp:161-182) */
sspmv_status sspmv_LeSpMV_coo(double alpha, const sspmv_coo *A, const void *x, double beta, void *y,
                              sspmv_stream_t stream);
sspmv_status sspmv_spmm_coo(double alpha, const sspmv_coo *A, int32_t k, const void *X, int64_t ldx,
                            double beta, void *Y, int64_t ldy, sspmv_stream_t stream);
sspmv_status sspmv_coo_export(const sspmv_coo *A, int32_t *row_index, int32_t *col_index, void *values,
                              sspmv_stream_t stream);
sspmv_status sspmv_delete_coo(sspmv_coo *A);

/* ---------------- DIA ---------------- */
/* csr_to_dia (include/sparse_conversion.h:612-766); max_diags / alignment 0
 * = defaults (10240, 64/sizeof(value)); more diagonals -> SSPMV_INFEASIBLE. */
sspmv_status sspmv_csr_to_dia(const sspmv_csr *csr, int32_t max_diags, int32_t alignment, sspmv_dia *out,
                              sspmv_stream_t stream);
/* LeSpMV_dia (src/spmv_dia.cpp:177-197).  kernel_flag 0 (default): a thread
 * per row over the diagonals; 1 (one right-hand side, at most 16 diagonals):
 * the rows' values and each diagonal's x window staged in shared memory by
 * bulk copies, a tile ahead of the threads. */
sspmv_status sspmv_LeSpMV_dia(double alpha, const sspmv_dia *A, const void *x, double beta, void *y,
                              sspmv_stream_t stream);
sspmv_status sspmv_spmm_dia(double alpha, const sspmv_dia *A, int32_t k, const void *X, int64_t ldx,
                            double beta, void *Y, int64_t ldy, sspmv_stream_t stream);
/* diag_offsets: complete_ndiags; diag_data: complete_ndiags*stride */
sspmv_status sspmv_dia_export(const sspmv_dia *A, int64_t *diag_offsets, void *diag_data, sspmv_stream_t stream);
sspmv_status sspmv_delete_dia(sspmv_dia *A);

/* ---------------- BSR ---------------- */
/* csr_to_bsr (include/sparse_conversion.h:769-926); 0 = defaults
 * (16 x 64/sizeof(value)). */
sspmv_status sspmv_csr_to_bsr(const sspmv_csr *csr, int32_t blockDimRow, int32_t blockDimCol, sspmv_bsr *out,
                              sspmv_stream_t stream);
/* Number of distinct r x c blocks csr_to_bsr would make (no block data is
 * allocated): lets a caller bound the fill before converting. */
sspmv_status sspmv_csr_count_blocks(const sspmv_csr *csr, int32_t blockDimRow, int32_t blockDimCol, int64_t *nnzb,
                                    sspmv_stream_t stream);
/* LeSpMV_bsr (src/spmv_bsr.cpp:215-233).  kernel_flag 0 (default): for
 * SpMV with r a power of two <= 32 and c in {1,2,4,8,16}, the block-stream
 * kernel (all lanes on blocks, segmented scan per step) when the thread-per-
 * row kernel would leave more than half its lane slots idle (uneven block
 * rows), else the thread-per-row kernel; 1: thread-per-row (the reference's
 * flag 1, rows in parallel); 2: block-stream where the shape allows (its flag
 * 2, balanced over blocks).  SpMM (k > 1) runs thread-per-row. */
sspmv_status sspmv_LeSpMV_bsr(double alpha, const sspmv_bsr *A, const void *x, double beta, void *y,
                              sspmv_stream_t stream);
sspmv_status sspmv_spmm_bsr(double alpha, const sspmv_bsr *A, int32_t k, const void *X, int64_t ldx,
                            double beta, void *Y, int64_t ldy, sspmv_stream_t stream);
/* row_ptr: mb+1 (num_rows+1 for 1x1 blocks); block_colindex: nnzb;
 * block_data: nnzb*blockNNZ */
sspmv_status sspmv_bsr_export(const sspmv_bsr *A, int32_t *row_ptr, int32_t *block_colindex, void *block_data,
                              sspmv_stream_t stream);
sspmv_status sspmv_delete_bsr(sspmv_bsr *A);

/* ---------------- CSR5 ---------------- */
/* csr_to_csr5 (include/sparse_conversion.h:939-1379); sigma / omega 0 =
 * reference defaults (16, 64/sizeof(value)); the SpMV kernel accepts omega in
 * {4, 8, 16, 32}. */
sspmv_status sspmv_csr_to_csr5(const sspmv_csr *csr, int32_t sigma, int32_t omega, sspmv_csr5 *out,
                               sspmv_stream_t stream);
/* LeSpMV_csr5 (src/spmv_csr5.cpp:439-457) */
sspmv_status sspmv_LeSpMV_csr5(double alpha, const sspmv_csr5 *A, const void *x, double beta, void *y,
                               sspmv_stream_t stream);
sspmv_status sspmv_spmm_csr5(double alpha, const sspmv_csr5 *A, int32_t k, const void *X, int64_t ldx,
                             double beta, void *Y, int64_t ldy, sspmv_stream_t stream);
/* Sizes from the struct fields; col_index / values are the transposed copies. */
sspmv_status sspmv_csr5_export(const sspmv_csr5 *A, uint32_t *tile_ptr, uint32_t *tile_desc,
                               int32_t *tile_desc_offset_ptr, int32_t *tile_desc_offset, int32_t *col_index,
                               void *values, sspmv_stream_t stream);
sspmv_status sspmv_delete_csr5(sspmv_csr5 *A);

/* Algorithmic bytes of one SpMV with k right-hand sides: structural bytes of
 * the format (padding excluded) + x once + y once (twice when beta != 0). */
double sspmv_algorithmic_bytes_csr(const sspmv_csr *A, int32_t k, int32_t beta_nonzero);
double sspmv_algorithmic_bytes_csr5(const sspmv_csr5 *A, int32_t k, int32_t beta_nonzero);
double sspmv_algorithmic_bytes_coo(const sspmv_coo *A, int32_t k, int32_t beta_nonzero);
double sspmv_algorithmic_bytes_dia(const sspmv_dia *A, int32_t k, int32_t beta_nonzero);
double sspmv_algorithmic_bytes_bsr(const sspmv_bsr *A, int32_t k, int32_t beta_nonzero);
double sspmv_algorithmic_bytes_ell(const sspmv_ell *A, int32_t k, int32_t beta_nonzero);
double sspmv_algorithmic_bytes_sell(const sspmv_s_ell *A, int32_t k, int32_t beta_nonzero);
double sspmv_algorithmic_bytes_sell_c_sigma(const sspmv_sell_c_sigma *A, int32_t k, int32_t beta_nonzero);
double sspmv_algorithmic_bytes_sell_c_R(const sspmv_sell_c_R *A, int32_t k, int32_t beta_nonzero);

/* The reference benchmark's bytes per SpMV, bytes_per_spmv
 * (include/spmv_benchmark.h:26-150), the numerator of the GB/s its benchmark
 * programs print (src/spmv_benchmark.cpp:68): x charged per nonzero, y twice
 * per row, padded slots for ELL and the sliced formats (their values at 4
 * bytes, as the reference counts them), y of occupied rows only for COO.
 * From the struct fields, except COO, which counts its occupied rows on the
 * device (synchronous).  -1 on a null or malformed matrix. */
double sspmv_reference_bytes_csr(const sspmv_csr *A);
double sspmv_reference_bytes_csr5(const sspmv_csr5 *A);
double sspmv_reference_bytes_coo(const sspmv_coo *A);
double sspmv_reference_bytes_dia(const sspmv_dia *A);
double sspmv_reference_bytes_bsr(const sspmv_bsr *A);
double sspmv_reference_bytes_ell(const sspmv_ell *A);
double sspmv_reference_bytes_sell(const sspmv_s_ell *A);
double sspmv_reference_bytes_sell_c_sigma(const sspmv_sell_c_sigma *A);
double sspmv_reference_bytes_sell_c_R(const sspmv_sell_c_R *A);

/* ---------------- matrix features ---------------- */
/* The reference's MTX feature extractor (src/sparse_features.cpp:122-968) on
 * a device CSR matrix: features[0..39] are the 40 values of its .features
 * file in file order (FeaturesWrite, :1347-1400), features[40..61] the other
 * statistics it computes (triangle and diagonal counts, minima, dominance,
 * value ranges, symmetry, variances, GrX = -1 as the reference leaves them).
 * tile_blocks: T for the T x T tile grid (0 = 256, the shipped
 * MAT_TILE_SIZE).  nnz_by_tiles / uniq_rb / uniq_cb: optional host arrays of
 * T*T counts (nonzeros, distinct rows, distinct columns per tile). */
#define SSPMV_NUM_FEATURES 62
sspmv_status sspmv_csr_features(const sspmv_csr *A, int32_t tile_blocks, double *features, int32_t *nnz_by_tiles,
                                int32_t *uniq_rb, int32_t *uniq_cb, sspmv_stream_t stream);
const char *sspmv_feature_name(int32_t i);
/* The GrX tile-group features the reference specifies but leaves at -1
 * (CalculateTilesExtraFeatures under BSR_ANA and AnalyzeTile_Group,
 * src/sparse_features.cpp:884-1065, README "GrX_uniqR and GrX_uniqC"):
 * out[0..3] = GrX_uniqR, GrX_uniqC, GrX_potReuseR, GrX_potReuseC over
 * BestDimForBSR-sized tiles of a T x T grid (tile_blocks: T, 0 = 256) with
 * groups of X = group rows / columns (0 = 64 / sizeof(value), the
 * reference's CACHE_LINE / sizeof(ValueType)).  Entries with value 0 count as
 * absent; a feature stays -1 when the tile is smaller than X. */
sspmv_status sspmv_csr_grx_features(const sspmv_csr *A, int32_t tile_blocks, int32_t group, double *out,
                                    sspmv_stream_t stream);

/* ---------------- host utilities ---------------- */
/* Matrix Market reader (utils/sparse_io.cpp:27-204: coordinate format,
 * general/symmetric, real/integer/pattern; symmetric entries mirrored,
 * duplicates kept, CSR built by a stable counting sort).  Two calls: first
 * with NULL arrays to get sizes, then with buffers of those sizes. */
sspmv_status sspmv_read_mtx(const char *path, int32_t value_type, int64_t *num_rows, int64_t *num_cols,
                            int64_t *num_nnzs, int32_t *row_offset, int32_t *col_index, void *values);
/* read_coo_matrix (utils/sparse_io.cpp:27-163): the triplets in file order
 * (0-based; symmetric files: each off-diagonal entry followed by its
 * mirror; pattern values 1.0), into host arrays of num_nnzs entries.  Call
 * with row_index == NULL to get the sizes first. */
sspmv_status sspmv_read_mtx_coo(const char *path, int32_t value_type, int64_t *num_rows, int64_t *num_cols,
                                int64_t *num_nnzs, int32_t *row_index, int32_t *col_index, void *values);
/* sum_csr_duplicates (include/sparse_operation.h:22-73), the compact step of
 * coo_to_csr / read_csr_matrix(path, compact = true): in place on host CSR
 * arrays; per row equal columns summed, columns in reverse order of first
 * appearance, zero sums dropped; row_offset rewritten, *num_nnzs set. */
sspmv_status sspmv_sum_csr_duplicates(int32_t value_type, int64_t num_rows, int64_t num_cols, int32_t *row_offset,
                                      int32_t *col_index, void *values, int64_t *num_nnzs);

/* Writes a CSR matrix as "matrix coordinate real general" (1-based, %.17g),
 * a file the reference's read_csr_matrix reads back bit-exactly. */
sspmv_status sspmv_write_mtx(const char *path, int64_t num_rows, int64_t num_cols, const int32_t *row_offset,
                             const int32_t *col_index, const double *values);

typedef enum {
    SSPMV_SYNTH_LAPLACIAN2D = 0,
    SSPMV_SYNTH_BANDED = 1,
    SSPMV_SYNTH_POWERLAW = 2,
    SSPMV_SYNTH_BLOCK = 3,
    SSPMV_SYNTH_UNIFORM = 4
} sspmv_synth_family;

typedef struct {
    int32_t family;        /* sspmv_synth_family */
    int32_t num_offsets;   /* BANDED */
    int64_t num_rows;      /* all but LAPLACIAN2D */
    int64_t num_cols;      /* 0: square */
    int64_t grid;          /* LAPLACIAN2D: g (num_rows = g*g) */
    int64_t offsets[32];   /* BANDED */
    double alpha;          /* POWERLAW Zipf exponent */
    double mean;           /* POWERLAW target mean row length (<=0: unscaled) */
    int64_t cap;           /* POWERLAW maximum row length */
    int64_t block_dim;     /* BLOCK: b */
    int64_t num_blocks;    /* BLOCK: distinct dense blocks */
    int64_t per_row;       /* UNIFORM */
    double empty_row_frac; /* POWERLAW / UNIFORM: fraction of empty rows */
} sspmv_synth_params;

/* Seeded synthetic CSR: row offsets first (returns nnz, or -1 if it does not
 * fit int32), then columns and values (FP32 values are the FP64 draws
 * rounded). */
int64_t sspmv_synth_row_offsets(const sspmv_synth_params *p, uint64_t seed, int32_t *row_offset);
int sspmv_synth_fill_f64(const sspmv_synth_params *p, uint64_t seed, const int32_t *row_offset,
                         int32_t *col_index, double *values);
int sspmv_synth_fill_f32(const sspmv_synth_params *p, uint64_t seed, const int32_t *row_offset,
                         int32_t *col_index, float *values);
/* x_i ~ U[-1,1) from (seed, i). */
void sspmv_synth_vector_f64(int64_t n, uint64_t seed, double *out);
void sspmv_synth_vector_f32(int64_t n, uint64_t seed, float *out);

/* ---------------- selector network (FP32) ---------------- */
/* Kernels of the format selector's multilayer perceptron; no counterpart in
 * the reference's C++ (its selector is a Keras model,
 * SmartAdpter/models/SpMV_Adapter.py).  Row-major, device pointers, leading
 * dimensions in elements.  W of a layer is out x in. */
/* y = x W^T + b (b may be NULL), ReLU when relu != 0. */
sspmv_status sspmv_nn_linear_forward(int32_t batch, int32_t in, int32_t out, const float *x, int32_t ldx,
                                     const float *W, const float *b, int32_t relu, float *y, int32_t ldy,
                                     sspmv_stream_t stream);
/* Gradients of a layer from dy (masked in place by y > 0 when relu != 0,
 * which needs ldy == out): dW = dy^T x, db = column sums of dy, dx = dy W
 * (dx may be NULL). */
sspmv_status sspmv_nn_linear_backward(int32_t batch, int32_t in, int32_t out, const float *x, int32_t ldx,
                                      const float *W, const float *y, int32_t relu, float *dy, int32_t ldy,
                                      float *dx, int32_t lddx, float *dW, float *db, sspmv_stream_t stream);
/* Softmax cross-entropy of C logits per row: loss_rows[b] = -log p[label]
 * (0 when label < 0), dlogits = (p - onehot) / batch. */
sspmv_status sspmv_nn_softmax_xent(int32_t batch, int32_t C, const float *logits, int32_t ld, const int32_t *labels,
                                   float *dlogits, int32_t ldd, float *loss_rows, sspmv_stream_t stream);
/* Masked squared error: loss_rows[b] = sum_c mask (pred - target)^2 / count,
 * dpred = weight * 2 (pred - target) mask / count; target and mask are
 * batch x C dense. */
sspmv_status sspmv_nn_masked_mse(int32_t batch, int32_t C, const float *pred, int32_t ld, const float *target,
                                 const float *mask, float weight, float count, float *dpred, int32_t ldd,
                                 float *loss_rows, sspmv_stream_t stream);
/* Adam (bias-corrected, step >= 1); weight_decay * w is added to the
 * gradient (L2 regularisation). */
sspmv_status sspmv_nn_adam(int64_t n, float *w, const float *g, float *m, float *v, float lr, float beta1,
                           float beta2, float eps, int32_t step, float weight_decay, sspmv_stream_t stream);

/* ---------------- request server ---------------- */
/* No counterpart in the reference (its benchmark_spmv_<fmt> programs run one
 * matrix per process).  A server keeps registered matrices resident in HBM in
 * the format each was registered with (loaded from the caller's host arrays
 * on first use, least-recently-used eviction under a byte budget) and serves
 * requests y = alpha * A * X + beta * Y (k right-hand sides, row-major X/Y
 * with leading dimensions, HOST buffers) with continuous batching: while
 * batches are on the GPU, the requests that arrive are gathered into the
 * next one.  CSR requests with k in {1, 2, 4, 8} of a batch run in one
 * persistent stream-kernel launch per (value type, k) group, replayed from a
 * CUDA graph; other requests get their format's own launch in the same
 * batch.  A request's result is bit-identical whatever else is batched with
 * it.  Mode SSPMV_SERVE_PER_REQUEST serves one request at a time through
 * sspmv_spmm_<fmt> (the plain per-request launch path, for comparison). */
typedef enum {
    SSPMV_FMT_CSR = 0,
    SSPMV_FMT_COO = 1,
    SSPMV_FMT_ELL = 2,
    SSPMV_FMT_SELL = 3,
    SSPMV_FMT_SELL_C_SIGMA = 4,
    SSPMV_FMT_SELL_C_R = 5,
    SSPMV_FMT_DIA = 6,
    SSPMV_FMT_BSR = 7,
    SSPMV_FMT_CSR5 = 8
} sspmv_format;

typedef enum { SSPMV_SERVE_BATCHED = 0, SSPMV_SERVE_PER_REQUEST = 1 } sspmv_serve_mode;

typedef struct {
    int32_t mode;               /* sspmv_serve_mode */
    int32_t max_batch_requests; /* 0: 1024 */
    int64_t max_batch_tiles;    /* 256-nonzero chunks (carry slots) per batch; 0: 1 << 20 */
    int64_t arena_bytes;        /* per batch in flight, device staging for X and for Y each; 0: 512 MiB */
    int64_t stage_limit_bytes;  /* X / Y up to this size are packed through pinned staging; 0: 1 MiB */
    int64_t hbm_budget_bytes;   /* resident matrices; 0: 120e9 */
    int32_t num_inflight;       /* batches in flight, one stream each; 0: 2 */
    int32_t use_graphs;         /* batched launches replayed from CUDA graphs */
} sspmv_server_config;

#define SSPMV_REQ_DEVICE_BUFFERS 1 /* x and y are device pointers: no copies */

typedef struct {
    int32_t matrix_id;
    int32_t k;                  /* right-hand sides (>= 1) */
    double alpha, beta;
    const void *x;              /* num_cols rows of ldx values (host unless SSPMV_REQ_DEVICE_BUFFERS) */
    int64_t ldx;
    void *y;                    /* num_rows rows of ldy values (read when beta != 0) */
    int64_t ldy;
    int32_t flags;              /* SSPMV_REQ_DEVICE_BUFFERS or 0 */
    int32_t reserved;
} sspmv_request;

typedef struct {
    int32_t status;             /* sspmv_status of the request */
    int32_t batch_size;         /* requests in its batch */
    int64_t batch_id;
    int64_t arrival_ns;         /* submit time (replay: the scheduled arrival), steady clock */
    int64_t launch_ns;          /* its batch was issued to the GPU */
    int64_t done_ns;            /* result in the caller's y */
} sspmv_request_info;

typedef struct {
    int64_t requests_done, requests_failed, batches, batched_requests, batched_tiles, graph_launches;
    int64_t loads, evictions, resident_matrices, resident_bytes;
} sspmv_server_stats;

typedef struct sspmv_server sspmv_server;

sspmv_status sspmv_server_create(const sspmv_server_config *cfg, sspmv_server **out);
/* Serves what is queued, then stops and frees everything the server holds. */
sspmv_status sspmv_server_destroy(sspmv_server *srv);
/* Registers matrix `id` from host CSR arrays that must stay valid while it is
 * registered.  format: sspmv_format; params: the converter's integer
 * arguments in declaration order (ELL: ld; SELL: chunkwidth, alignment;
 * SELL-c-sigma: slicewidth, chunkwidth, alignment; SELL-c-R: chunkwidth,
 * alignment; DIA: max_diags, alignment; BSR: blockDimRow, blockDimCol; CSR5:
 * sigma, omega), NULL for the defaults. */
sspmv_status sspmv_server_add_matrix(sspmv_server *srv, int32_t id, int32_t value_type, int64_t num_rows,
                                     int64_t num_cols, int64_t num_nnzs, const int32_t *row_offset,
                                     const int32_t *col_index, const void *values, int32_t format,
                                     const int32_t *params);
/* Loads matrix `id` into HBM now (otherwise its first request does). */
sspmv_status sspmv_server_preload(sspmv_server *srv, int32_t id);
/* Queues one request; x and y must stay valid until it completes. */
sspmv_status sspmv_server_submit(sspmv_server *srv, const sspmv_request *req, int64_t *ticket);
/* Waits (timeout_s < 0: forever) for a submitted request and forgets it;
 * SSPMV_DEVICE_TIMEOUT if it has not completed in time. */
sspmv_status sspmv_server_wait(sspmv_server *srv, int64_t ticket, double timeout_s, sspmv_request_info *info);
/* Open-loop load: submits request i at arrival_ns[i] nanoseconds after the
 * call starts (ascending), then waits for all of them and fills infos[i]. */
sspmv_status sspmv_server_replay(sspmv_server *srv, int64_t n, const sspmv_request *reqs, const int64_t *arrival_ns,
                                 sspmv_request_info *infos);
sspmv_status sspmv_server_get_stats(const sspmv_server *srv, sspmv_server_stats *stats);

#ifdef __cplusplus
}
#endif
#endif /* SSPMV_H */
