// plan.cuh -- library-private per-matrix state hung off sspmv_features.priv.
//
// A plan caches what depends only on the sparsity structure (merge-path tile
// coordinates, per-tile carry buffers, chosen launch shapes).  It is built on
// the first SpMV of a matrix (or by the converter that made the matrix) and
// freed by sspmv_delete_<fmt>.  Carry buffers are shared by all calls on one
// matrix: calls on the same matrix must be ordered (one stream, or events).
#pragma once

#include "common.cuh"
#include <mutex>

namespace sspmv {

// Merge-path schedule over (row ends, nonzeros) for CSR-like kernels.
struct MergePlan {
    int tile_items = 0;       // merge items per CTA tile
    int64_t num_tiles = 0;
    int2 *coords = nullptr;   // num_tiles + 1 split points (row, nnz)
    int32_t *carry_row = nullptr;
    int32_t *has_end = nullptr;
    void *carry_val = nullptr;  // num_tiles * kMaxK values
    void *head_val = nullptr;   // num_tiles * kMaxK values
};

constexpr int kMaxK = 8;  // right-hand sides handled per pass

struct Plan {
    int kind = 0;
    MergePlan merge[2];     // [0]: tile for k <= 4, [1]: tile for k == 8
    int param = 0;          // kernel parameter set by sspmv_set_kernel (0 = library choice)
    void *extra[12] = {nullptr};  // format-specific device buffers
    int64_t extra_i[12] = {0};
    sspmv_csr *sub = nullptr;     // a library-made CSR view over extra buffers (its own plan freed with this one)
};

// Guards plan creation.  Recursive: building one plan may build another
// (a sliced matrix's overflow CSR gets its stream plan while its own plan is
// being built).
using PlanMutex = std::recursive_mutex;
PlanMutex &plan_mutex();
Plan *get_plan(const sspmv_features *f);  // creates an empty plan if needed
void free_plan(sspmv_features *f, sspmv_stream_t s);

// Builds (once) the merge plan of a CSR-shaped structure: row_offset has m+1
// entries and nnz = row_offset[m].
sspmv_status ensure_merge_plan(Plan *p, int which, int64_t m, int64_t nnz, const int32_t *row_offset,
                               int32_t value_type, sspmv_stream_t s);

}  // namespace sspmv
