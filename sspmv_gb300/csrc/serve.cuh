// serve.cuh -- device-side batch description shared by the request server
// (server.cu) and the batched stream CSR kernels (spmv_csr.cu).
//
// A batch holds many independent requests y = alpha*A*X + beta*Y on CSR
// matrices of any size.  Requests are grouped by (value type, k); group g =
// 4 * (value_type == F64) + log2(k) for k in {1, 2, 4, 8}.  Within a group the
// 256-nonzero chunks of all requests are numbered consecutively (item i owns
// global chunks [chunk_begin, chunk_begin + num_chunks)), and one persistent
// kernel per group walks the global chunks.  Each request is cut into exactly
// the chunks the single-matrix stream kernel uses (the matrix's own
// row_start), so a request's result does not depend on what else is in the
// batch.
#pragma once

#include "common.cuh"

namespace sspmv {

constexpr int kBatchGroups = 8;

inline int batch_group(int32_t value_type, int32_t k) {
    const int lk = k == 8 ? 3 : k == 4 ? 2 : k == 2 ? 1 : 0;
    return (value_type == SSPMV_F64 ? 4 : 0) + lk;
}

struct BatchItem {
    const int32_t *row_offset;
    const int32_t *col_index;
    const void *values;
    const int32_t *row_start;  // num_chunks + 1 rows holding each chunk's first nonzero
    const void *x;
    void *y;
    int64_t ldx, ldy;
    double alpha, beta;
    int64_t chunk_begin;  // first global chunk of this item in its group
    int64_t nnz;
    int32_t m;
    int32_t num_chunks;
    int32_t vec;          // 16-byte aligned col_index / values: vector loads
    int32_t xvec;         // X rows aligned for vector loads (xrow_vec)
};

struct BatchHeader {
    int32_t item_begin[kBatchGroups];    // first item of each group (items are stored group by group)
    int32_t n_items[kBatchGroups];
    int64_t total_chunks[kBatchGroups];
    int64_t carry_base[kBatchGroups];    // first carry slot of each group
};

// Carry slots of one batch workspace (one per chunk): a row index, an end
// flag and kMaxK carry and head values of up to 8 bytes.
constexpr size_t kBatchSlotBytes = 4 + 4 + 2 * 8 * 8;

// The stream kernel's plan of a matrix (built once): row of each chunk's first
// nonzero, chunk count, longest run of empty rows.
sspmv_status csr_stream_plan(const sspmv_csr *A, const int32_t **row_start, int64_t *num_chunks, int32_t *max_gap,
                             sspmv_stream_t s);
// Whether the stream kernel (and so the batched kernel) takes the matrix.
bool csr_stream_takes(int64_t num_nnzs, int32_t max_gap);

// Persistent grid size of group g (SMs x resident CTAs of its batch kernel).
unsigned csr_batch_grid(int g);

// Launches group g's batched stream kernel and its fix-up kernel on stream s.
// Header and items are read from device memory when the kernels run, so the
// launches can be captured once and replayed for every batch.
sspmv_status launch_csr_batch_group(int g, const BatchHeader *d_hdr, const BatchItem *d_items, void *carry,
                                    int64_t carry_slots, sspmv_stream_t s);

}  // namespace sspmv
