// serve.cuh -- device-side batch description shared by the request server
// (server.cu) and the batched merge-path CSR kernels (spmv_csr.cu).
//
// A batch holds many independent requests y = alpha*A*X + beta*Y on CSR
// matrices of any size.  Requests are grouped by (value type, k); group g =
// 4 * (value_type == F64) + log2(k) for k in {1, 2, 4, 8}.  Within a group the
// merge-path tiles of all requests are numbered consecutively (item i owns
// global tiles [tile_begin, tile_begin + num_tiles)), and one persistent
// kernel per group walks the global tiles.  Each request is cut into exactly
// the tiles the single-matrix kernel uses (the matrix's own merge split
// points), so a request's result does not depend on what else is in the batch.
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
    const int2 *coords;   // num_tiles + 1 merge split points of the matrix
    const void *x;
    void *y;
    int64_t ldx, ldy;
    double alpha, beta;
    int64_t tile_begin;   // first global tile of this item in its group
    int32_t m;
    int32_t num_tiles;
};

struct BatchHeader {
    int32_t item_begin[kBatchGroups];   // first item of each group (items are stored group by group)
    int32_t n_items[kBatchGroups];
    int64_t total_tiles[kBatchGroups];
    int64_t carry_base[kBatchGroups];   // first carry slot of each group
};

// Carry slots of one batch workspace: per slot a row index, an end flag and
// kMaxK carry and head values of up to 8 bytes.
constexpr size_t kBatchSlotBytes = 4 + 4 + 2 * 8 * 8;

// Merge items per tile for k right-hand sides (2048 for k <= 4, 1024 for k = 8).
int csr_merge_tile_items(int32_t k);

// Builds the matrix's merge split points for k right-hand sides (once) and
// returns them.
sspmv_status csr_merge_coords(const sspmv_csr *A, int32_t k, const int2 **coords, int64_t *num_tiles,
                              sspmv_stream_t s);

// Persistent grid size of group g (SMs x resident CTAs of its merge kernel).
unsigned csr_batch_grid(int g);

// Launches group g's batched merge kernel and its fix-up kernel on stream s.
// Header and items are read from device memory when the kernels run, so the
// launches can be captured once and replayed for every batch.
sspmv_status launch_csr_batch_group(int g, const BatchHeader *d_hdr, const BatchItem *d_items, void *carry,
                                    int64_t carry_slots, sspmv_stream_t s);

}  // namespace sspmv
