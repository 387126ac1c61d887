// spmv_csr.cu -- CSR SpMV / SpMM on sm_103a.
//
// Replaces LeSpMV_csr (src/spmv_csr.cpp:165-185) and its three CPU kernels
// (serial, OpenMP per row, nnz-balanced row partition).
//
// Default kernel (kernel_flag 0): the nonzero-split stream kernel (see
// csr_stream_kernel); matrices with long runs of empty rows fall back to
// merge-path.  kernel_flag 4: the pipelined thread-per-row kernel for
// matrices whose rows all have at most 12 nonzeros (csr_pipe_kernel).
// kernel_flag 3: the row-block kernel for matrices whose rows are all short
// (csr_rowblock_kernel; one launch, no fix-up).  kernel_flag 2: merge-path.
// The (row end, nonzero)
// merge sequence is cut into equal tiles of kTile items, so every CTA does the
// same work whatever the row lengths (power-law rows up to 50k nonzeros and
// empty rows alike).  A CTA stages its nonzeros' products a_ij * x_j into
// shared memory with coalesced streaming loads, then each thread walks
// kItems merge items and writes the rows it finishes.  Row pieces that cross
// thread boundaries are joined by a block-wide segmented scan; rows that cross
// tile boundaries leave (row, partial) carries in the plan and are finished by
// a second kernel, in a fixed order, so results are deterministic.
//
// kernel_flag 1: vector-per-row kernel, `lanes` threads per row (2..32,
// chosen from the mean row length, or set by the autotuner).
#include <atomic>
#include <cuda.h>
#include <mutex>
#include <type_traits>

#include "common.cuh"
#include "plan.cuh"
#include "bulk.cuh"
#include "primitives.cuh"
#include "spmv_common.cuh"
#include "csr_pipe.cuh"
#include "serve.cuh"

namespace sspmv {
namespace {

constexpr int kBlock = 256;

template <int K>
struct MergeShape {
    static constexpr int items = K <= 4 ? 8 : 4;     // merge items per thread
    static constexpr int tile = kBlock * items;       // 2048 or 1024
    static constexpr int which = K <= 4 ? 0 : 1;
};

__global__ void merge_path_search(int64_t num_tiles, int tile_items, int m, int nnz,
                                  const int32_t *__restrict__ row_offset, int2 *__restrict__ coords) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t > num_tiles) return;
    int64_t total = (int64_t)m + nnz;
    int64_t d = t * tile_items;
    if (d > total) d = total;
    int64_t lo = d - nnz > 0 ? d - nnz : 0;
    int64_t hi = d < m ? d : m;
    while (lo < hi) {
        int64_t p = (lo + hi) >> 1;
        if ((int64_t)row_offset[p + 1] <= d - p - 1) lo = p + 1;
        else hi = p;
    }
    coords[t] = make_int2((int)lo, (int)(d - lo));
}

template <typename V, int K>
struct alignas(16) VecK {
    V v[K];
};

// One merge-path tile (split points c0, c1) of one matrix; t indexes the
// per-tile carry slots.  Used by the single-matrix kernel (one tile per CTA)
// and by the batched serving kernel (a CTA loops over tiles of many
// requests); the leading barrier makes back-to-back calls safe.
template <typename V, int K>
__device__ __forceinline__ void merge_tile(
    int m, const int32_t *__restrict__ row_offset, const int32_t *__restrict__ col_index,
    const V *__restrict__ values, const V *__restrict__ x, int64_t ldx, V alpha, V beta,
    V *__restrict__ y, int64_t ldy, const int2 c0, const int2 c1, const int64_t t, int32_t *__restrict__ carry_row,
    int32_t *__restrict__ has_end, V *__restrict__ carry_val, V *__restrict__ head_val,
    unsigned char *__restrict__ smem_raw) {
    constexpr int kItems = MergeShape<K>::items;
    constexpr int kTile = MergeShape<K>::tile;
    constexpr int kWarps = kBlock / 32;
    V *s_prod = reinterpret_cast<V *>(smem_raw);                     // kTile * K
    int *s_rowend = reinterpret_cast<int *>(s_prod + kTile * K);      // kTile + 1
    __shared__ int s_wkey[kWarps];
    __shared__ V s_wval[kWarps][K];
    __shared__ V s_wpref[kWarps][K];
    __shared__ V s_full[kBlock][K];
    __shared__ int s_row0_start;
    __syncthreads();

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int i0 = c0.x, j0 = c0.y;
    const int nrows = c1.x - i0, nnzs = c1.y - j0;

    // ---- stage row ends and products (coalesced, streaming) ----
    // nrows + nnzs <= kTile = kBlock * kItems, so every thread owns at most
    // kItems nonzeros and kItems row ends; all of its loads are issued before
    // any is consumed (kItems independent chains in flight per thread).
    {
        int cidx[kItems];
        V aval[kItems];
#pragma unroll
        for (int u = 0; u < kItems; u++) {
            const int k = tid + u * kBlock;
            cidx[u] = 0;
            aval[u] = V(0);
            if (k < nnzs) {
                cidx[u] = ld_stream(col_index + j0 + k);
                aval[u] = ld_stream(values + j0 + k);
            }
        }
        int rend[kItems];
#pragma unroll
        for (int u = 0; u < kItems; u++) {
            const int k = tid + u * kBlock;
            rend[u] = k < nrows ? ld_stream(row_offset + i0 + 1 + k) : 0;
        }
        if (tid == 0) s_row0_start = i0 < m ? row_offset[i0] : 0;
#pragma unroll
        for (int u = 0; u < kItems; u++) {
            const int k = tid + u * kBlock;
            if (k < nnzs) {
                const V *xp = x + (int64_t)cidx[u] * ldx;
#pragma unroll
                for (int r = 0; r < K; r++) s_prod[k * K + r] = aval[u] * ld_x(xp + r);
            }
            if (k < nrows) s_rowend[k] = rend[u];
        }
    }
    __syncthreads();

    // ---- per-thread merge over kItems items ----
    const int total = nrows + nnzs;
    const int d = min(tid * kItems, total);
    int lo = max(d - nnzs, 0), hi = min(d, nrows);
    while (lo < hi) {
        int p = (lo + hi) >> 1;
        if (s_rowend[p] <= j0 + d - p - 1) lo = p + 1;
        else hi = p;
    }
    int ti = lo, tj = d - lo;
    V sum[K];
#pragma unroll
    for (int r = 0; r < K; r++) sum[r] = V(0);
    int first_row = -1;
    V first_val[K];
#pragma unroll
    for (int r = 0; r < K; r++) first_val[r] = V(0);
#pragma unroll
    for (int s = 0; s < kItems; s++) {
        if (ti < nrows && (tj >= nnzs || s_rowend[ti] <= j0 + tj)) {
            if (first_row < 0) {
                first_row = ti;
#pragma unroll
                for (int r = 0; r < K; r++) first_val[r] = sum[r];
            } else {
                V *yp = y + (int64_t)(i0 + ti) * ldy;
#pragma unroll
                for (int r = 0; r < K; r++) yp[r] = axpby(alpha, sum[r], beta, yp + r);
            }
#pragma unroll
            for (int r = 0; r < K; r++) sum[r] = V(0);
            ti++;
        } else if (tj < nnzs) {
#pragma unroll
            for (int r = 0; r < K; r++) sum[r] += s_prod[tj * K + r];
            tj++;
        }
    }

    // ---- block-wide segmented inclusive scan of carry-outs keyed by row ----
    int key = i0 + ti;
    const int key_up = __shfl_up_sync(0xffffffffu, key, 1);  // every lane shuffles (full mask)
    const int span = unflagged_run(lane == 0 || key_up != key);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        if (o > span) break;  // warp-uniform
        int k2 = __shfl_up_sync(0xffffffffu, key, o);
        V v2[K];
#pragma unroll
        for (int r = 0; r < K; r++) v2[r] = __shfl_up_sync(0xffffffffu, sum[r], o);
        if (lane >= o && k2 == key) {
#pragma unroll
            for (int r = 0; r < K; r++) sum[r] += v2[r];
        }
    }
    if (lane == 31) {
        s_wkey[warp] = key;
#pragma unroll
        for (int r = 0; r < K; r++) s_wval[warp][r] = sum[r];
    }
    __syncthreads();
    if (tid == 0) {
        for (int w = 0; w < kWarps; w++) {
            bool join = w > 0 && s_wkey[w] == s_wkey[w - 1];
#pragma unroll
            for (int r = 0; r < K; r++) s_wpref[w][r] = s_wval[w][r] + (join ? s_wpref[w - 1][r] : V(0));
        }
    }
    __syncthreads();
    if (warp > 0 && key == s_wkey[warp - 1]) {
#pragma unroll
        for (int r = 0; r < K; r++) sum[r] += s_wpref[warp - 1][r];
    }
#pragma unroll
    for (int r = 0; r < K; r++) s_full[tid][r] = sum[r];
    __syncthreads();

    if (first_row >= 0) {
        V tot[K];
#pragma unroll
        for (int r = 0; r < K; r++) tot[r] = first_val[r] + (tid > 0 ? s_full[tid - 1][r] : V(0));
        if (first_row == 0 && s_row0_start < j0) {
            V *hp = head_val + t * kMaxK;
#pragma unroll
            for (int r = 0; r < K; r++) hp[r] = tot[r];
        } else {
            V *yp = y + (int64_t)(i0 + first_row) * ldy;
#pragma unroll
            for (int r = 0; r < K; r++) yp[r] = axpby(alpha, tot[r], beta, yp + r);
        }
    }
    if (tid == kBlock - 1) {
        carry_row[t] = key;
        has_end[t] = nrows > 0;
        V *cp = carry_val + t * kMaxK;
#pragma unroll
        for (int r = 0; r < K; r++) cp[r] = sum[r];
    }
}

template <typename V, int K>
__global__ void __launch_bounds__(kBlock) csr_merge_kernel(
    int m, const int32_t *__restrict__ row_offset, const int32_t *__restrict__ col_index,
    const V *__restrict__ values, const V *__restrict__ x, int64_t ldx, V alpha, V beta,
    V *__restrict__ y, int64_t ldy, const int2 *__restrict__ coords, int32_t *__restrict__ carry_row,
    int32_t *__restrict__ has_end, V *__restrict__ carry_val, V *__restrict__ head_val) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int64_t t = blockIdx.x;
    merge_tile<V, K>(m, row_offset, col_index, values, x, ldx, alpha, beta, y, ldy, coords[t], coords[t + 1], t,
                     carry_row, has_end, carry_val, head_val, smem_raw);
}

// Finishes rows that cross tile boundaries: the tile where such a row starts
// owns it and adds the following tiles' pieces in order.
template <typename V, int K>
__global__ void csr_merge_fixup(int64_t num_tiles, int m, const int32_t *__restrict__ row_offset,
                                const int2 *__restrict__ coords, const int32_t *__restrict__ carry_row,
                                const int32_t *__restrict__ has_end, const V *__restrict__ carry_val,
                                const V *__restrict__ head_val, V alpha, V beta, V *__restrict__ y,
                                int64_t ldy) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t - (threadIdx.x & 31) >= num_tiles) return;  // whole warp past the end
    const int r = t < num_tiles ? carry_row[t] : m;
    bool mine = false;
    if (r < m) {
        const int rs = row_offset[r];
        mine = rs >= coords[t].y && rs < coords[t + 1].y;  // the row starts in tile t
    }
    V tot[K];
    chain_sum<V, K>(mine, t, num_tiles, 0, has_end, carry_val, head_val, tot);
    if (mine) {
        V *yp = y + (int64_t)r * ldy;
#pragma unroll
        for (int q = 0; q < K; q++) yp[q] = axpby(alpha, tot[q], beta, yp + q);
    }
}

constexpr int kVecHoist = 6;

template <typename V, int K, int VS, bool PLAIN = false>
__global__ void __launch_bounds__(kBlock, (VS == 1 && K == 1) ? (sizeof(V) == 4 ? 6 : 5) : 1) csr_vector_kernel(
    int m, const int32_t *__restrict__ row_offset, const int32_t *__restrict__ col_index,
    const V *__restrict__ values, const V *__restrict__ x, int64_t ldx, int xvec, V alpha, V beta,
    V *__restrict__ y, int64_t ldy) {
    constexpr int kRowsPerWarp = 32 / VS;
    const int lane = threadIdx.x & 31;
    const int sub = lane % VS;
    const int64_t warp_id = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t base = warp_id * kRowsPerWarp; base < m; base += nwarps * kRowsPerWarp) {
        const int64_t row = base + lane / VS;
        V s[K];
#pragma unroll
        for (int r = 0; r < K; r++) s[r] = V(0);
        int rs = 0, re = 0;
        if (row < m) {
            rs = ld_stream(row_offset + row);
            re = ld_stream(row_offset + row + 1);
        }
        // One lane per row, short rows (every lane of the warp with at most
        // kVecHoist elements): all of a lane's column and value loads, then
        // all its x gathers, are issued before its first FMA -- one memory
        // round trip each instead of one per element (same summation order
        // as the loop).  Measured: FP32 5-point Laplacian 22 -> 17 us; with
        // 2+ lanes per row the loop below was faster.
        const int cnt = re - rs > sub ? (re - rs - sub + VS - 1) / VS : 0;
        const int wmax = (VS == 1 && K <= 2) ? __reduce_max_sync(0xffffffffu, cnt) : kVecHoist + 1;
        if (wmax <= kVecHoist) {
            int c[kVecHoist];
            V a[kVecHoist];
#pragma unroll
            for (int q = 0; q < kVecHoist; q++) {
                c[q] = 0;  // a lane past its elements gathers x row 0 (exists: some lane has elements) with value 0
                a[q] = V(0);
                if (q < cnt) {
                    c[q] = ld_stream(col_index + rs + sub + q * VS);
                    a[q] = ld_stream(values + rs + sub + q * VS);
                }
            }
            V xr[kVecHoist][K];
#pragma unroll
            for (int q = 0; q < kVecHoist; q++)
                if (q < wmax) ld_xrow<V, K>(x, c[q], ldx, xvec != 0, xr[q]);
#pragma unroll
            for (int q = 0; q < kVecHoist; q++)
                if (q < cnt) {  // never 0 * x[0]: x may hold Inf or NaN
#pragma unroll
                    for (int r = 0; r < K; r++) s[r] += a[q] * xr[q][r];
                }
        } else if (row < m) {
            int j = rs + sub;
            for (; j + 3 * VS < re; j += 4 * VS) {  // four independent gathers in flight
                int c[4];
                V a[4];
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    c[u] = ld_stream(col_index + j + u * VS);
                    a[u] = ld_stream(values + j + u * VS);
                }
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    V xr[K];
                    ld_xrow<V, K>(x, c[u], ldx, xvec != 0, xr);
#pragma unroll
                    for (int r = 0; r < K; r++) s[r] += a[u] * xr[r];
                }
            }
            for (; j < re; j += VS) {
                const int c = ld_stream(col_index + j);
                const V a = ld_stream(values + j);
                V xr[K];
                ld_xrow<V, K>(x, c, ldx, xvec != 0, xr);
#pragma unroll
                for (int r = 0; r < K; r++) s[r] += a * xr[r];
            }
        }
#pragma unroll
        for (int r = 0; r < K; r++) s[r] = warp_sum(s[r], VS);
        if (row < m && sub == 0) {
            V *yp = y + row * ldy;
#pragma unroll
            for (int r = 0; r < K; r++) yp[r] = row_out(PLAIN, alpha, s[r], beta, yp + r);
        }
    }
}

template <typename V, int K>
sspmv_status launch_merge(const sspmv_csr *A, Plan *p, V alpha, const V *x, int64_t ldx, V beta, V *y,
                          int64_t ldy, sspmv_stream_t s) {
    constexpr int which = MergeShape<K>::which;
    SSPMV_TRY(ensure_merge_plan(p, which, A->f.num_rows, A->f.num_nnzs, A->row_offset, A->f.value_type, s));
    MergePlan &mp = p->merge[which];
    const size_t smem = (size_t)MergeShape<K>::tile * K * sizeof(V) + ((size_t)MergeShape<K>::tile + 1) * 4;
    static std::atomic<bool> attr_set{false};  // set after the attribute call returns
    if (!attr_set.load(std::memory_order_acquire)) {
        SSPMV_CUDA_TRY(cudaFuncSetAttribute(csr_merge_kernel<V, K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)smem));
        attr_set.store(true, std::memory_order_release);
    }
    csr_merge_kernel<V, K><<<(unsigned)mp.num_tiles, kBlock, smem, cu(s)>>>(
        (int)A->f.num_rows, A->row_offset, A->col_index, (const V *)A->values, x, ldx, alpha, beta, y, ldy,
        mp.coords, mp.carry_row, mp.has_end, (V *)mp.carry_val, (V *)mp.head_val);
    SSPMV_LAUNCH_CHECK();
    if (mp.num_tiles > 1) {
        csr_merge_fixup<V, K><<<grid_for(mp.num_tiles, 256), 256, 0, cu(s)>>>(
            mp.num_tiles, (int)A->f.num_rows, A->row_offset, mp.coords, mp.carry_row, mp.has_end,
            (const V *)mp.carry_val, (const V *)mp.head_val, alpha, beta, y, ldy);
        SSPMV_LAUNCH_CHECK();
    }
    return SSPMV_OK;
}

template <typename V, int K, int VS>
sspmv_status launch_vector_vs(const sspmv_csr *A, V alpha, const V *x, int64_t ldx, V beta, V *y, int64_t ldy,
                              sspmv_stream_t s) {
    const int64_t m = A->f.num_rows;
    const int64_t warps = (m + (32 / VS) - 1) / (32 / VS);
    const unsigned grid = grid_for(warps * 32, kBlock, (int64_t)num_sms() * 16);
    auto go = [&](auto kernel) {
        kernel<<<grid, kBlock, 0, cu(s)>>>((int)m, A->row_offset, A->col_index, (const V *)A->values, x, ldx,
                                           xrow_vec(x, ldx, sizeof(V), K), alpha, beta, y, ldy);
    };
    if (K == 1 && alpha == V(1) && beta == V(0)) go(csr_vector_kernel<V, K, VS, K == 1>);
    else go(csr_vector_kernel<V, K, VS>);
    SSPMV_LAUNCH_CHECK();
    return SSPMV_OK;
}

template <typename V, int K>
sspmv_status launch_vector(const sspmv_csr *A, Plan *p, V alpha, const V *x, int64_t ldx, V beta, V *y,
                           int64_t ldy, sspmv_stream_t s) {
    int vs = p->param;
    if (vs == 0) {
        double mean = A->f.num_rows > 0 ? (double)A->f.num_nnzs / (double)A->f.num_rows : 1.0;
        vs = 2;
        while (vs < 32 && vs < mean) vs <<= 1;
    }
    switch (vs) {
    case 1: return launch_vector_vs<V, K, 1>(A, alpha, x, ldx, beta, y, ldy, s);
    case 2: return launch_vector_vs<V, K, 2>(A, alpha, x, ldx, beta, y, ldy, s);
    case 4: return launch_vector_vs<V, K, 4>(A, alpha, x, ldx, beta, y, ldy, s);
    case 8: return launch_vector_vs<V, K, 8>(A, alpha, x, ldx, beta, y, ldy, s);
    case 16: return launch_vector_vs<V, K, 16>(A, alpha, x, ldx, beta, y, ldy, s);
    default: return launch_vector_vs<V, K, 32>(A, alpha, x, ldx, beta, y, ldy, s);
    }
}

// ----------------------------------------------------- row-block kernel --
// kernel_flag 3: short rows, one launch, streamed by the copy engine.
//
// The rows are cut into blocks of whole rows: row r opens a block when its
// first nonzero lies in another window of `window` nonzeros than row r - 1's,
// or r is a multiple of kRbRows.  A block therefore holds at most kRbRows
// rows and, with no row longer than kRbMaxRow, at most window + kRbMaxRow - 1
// nonzeros, and no row crosses two blocks: the CTA that takes a block
// finishes its rows itself, with no carries and no fix-up launch (a second
// launch costs about as much as the whole SpMV of an 84 MB matrix).
//
// The grid is persistent (every SM full), CTA g taking blocks g, g + G, ...
// Thread 0 streams each block's row offsets, columns and values into one of
// kRbStages shared-memory stages with three bulk copies (cp.async.bulk, the
// copy engine) completed on the stage's mbarrier, kRbStages blocks ahead of
// the CTA's threads: the matrix moves like a copy, with no per-element load
// instructions and no load latency on the threads' path.  The threads then
// gather x for the block's nonzeros (all gathers of a thread in flight
// together), overwrite each value with its product, and each thread sums its
// rows' products in row order.  The bulk copies cover the 16-byte aligned
// interior of each run; the few elements at its ragged ends are read with
// plain loads.  Deterministic.  Matrices with a row longer than kRbMaxRow use
// the stream kernel instead, and so do arrays not 16-byte aligned.
constexpr int kRbRows = 1024;
constexpr int kRbMaxRow = 64;
constexpr int kRbDefaultWindow = 1024;
constexpr int kRbStages = 2;

// Count of bounded waits that gave up (a copy that never completed) in this
// file's kernels since the library was loaded; read by sspmv_wait_timeouts.
__device__ unsigned long long g_csr_wait_timeouts = 0;

__global__ void rowblock_flags(int m, int lg_window, const int32_t *__restrict__ rp, int32_t *__restrict__ flag) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m) return;
    flag[r] = (r % kRbRows == 0 || (rp[r] >> lg_window) != (rp[r - 1] >> lg_window)) ? 1 : 0;
}

__global__ void rowblock_starts(int m, int nnz, int lg_window, int nb, const int32_t *__restrict__ rp,
                                const int32_t *__restrict__ pos, int2 *__restrict__ blocks) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r == 0) blocks[nb] = make_int2(m, nnz);
    if (r >= m) return;
    const bool opens = r % kRbRows == 0 || (rp[r] >> lg_window) != (rp[r - 1] >> lg_window);
    if (opens) blocks[pos[r]] = make_int2((int)r, rp[r]);
}

// Shared-memory layout of one stage (element capacities; every region starts
// on a 16-byte boundary).  A block's run [e0, e1) of an array is copied as
// the 16-byte aligned superset [e0 rounded down, e1 rounded up) -- its
// neighbours' elements ride along -- and element e sits at index
// e - (e0 rounded down), so a region holds the longest run plus 2 x 16 bytes.
template <typename V, int W>
struct RbStage {
    static constexpr int kNz = W + kRbMaxRow + 8;        // columns and values
    static constexpr int kRp = kRbRows + 1 + 7;          // row offsets
    static constexpr size_t kValBytes = (size_t)kNz * sizeof(V);
    static constexpr size_t kColBytes = (size_t)kNz * 4;
    static constexpr size_t kRpBytes = (size_t)kRp * 4;
    static constexpr size_t kBytes = kValBytes + kColBytes + kRpBytes + 32;  // + header
};

template <typename V, int W>
constexpr size_t rowblock_smem() {
    return kRbStages * RbStage<V, W>::kBytes + kRbStages * sizeof(uint64_t);
}

// [a, end) = [lo rounded down, hi rounded up) to 16 bytes, cut at the array's
// last 16-byte boundary (elements beyond it, at most 15 bytes, are read with
// plain loads: a copy never reads past the array).
template <int E>
__device__ __forceinline__ void copy_span(int64_t lo, int64_t hi, int64_t n, int64_t &a, int64_t &end) {
    constexpr int64_t per = 16 / E;
    a = lo / per * per;
    end = min((hi + per - 1) / per * per, n / per * per);
}

template <typename V, int W, bool PLAIN>
__global__ void __launch_bounds__(kBlock) csr_rowblock_kernel(int64_t nb, int m, int64_t nnz,
                                                              const int2 *__restrict__ blocks,
                                                              const int32_t *__restrict__ rp,
                                                              const int32_t *__restrict__ col,
                                                              const V *__restrict__ val, const V *__restrict__ x,
                                                              int64_t ldx, V alpha, V beta, V *__restrict__ y,
                                                              int64_t ldy) {
    using St = RbStage<V, W>;
    constexpr int kPer = (W + kRbMaxRow + kBlock - 1) / kBlock;
    extern __shared__ __align__(16) unsigned char rb_smem[];
    uint64_t *bars = reinterpret_cast<uint64_t *>(rb_smem + kRbStages * St::kBytes);
    auto sval = [&](int s) { return reinterpret_cast<V *>(rb_smem + s * St::kBytes); };
    auto scol = [&](int s) { return reinterpret_cast<int32_t *>(rb_smem + s * St::kBytes + St::kValBytes); };
    auto srp = [&](int s) {
        return reinterpret_cast<int32_t *>(rb_smem + s * St::kBytes + St::kValBytes + St::kColBytes);
    };
    auto shdr = [&](int s) {
        return reinterpret_cast<int32_t *>(rb_smem + s * St::kBytes + St::kValBytes + St::kColBytes + St::kRpBytes);
    };
    const int t = threadIdx.x;
    const int64_t G = gridDim.x;
    const int64_t g = blockIdx.x;

    // Thread 0: start the copies of the CTA's k-th block (bounds lo, hi) into
    // stage k % kRbStages.
    auto issue = [&](int64_t k, int2 lo, int2 hi) {
        const int64_t b = g + k * G;
        if (b >= nb) return;
        const int s = (int)(k % kRbStages);
        int64_t av, ve, ac, ce, ap, pe;
        copy_span<sizeof(V)>(lo.y, hi.y, nnz, av, ve);
        copy_span<4>(lo.y, hi.y, nnz, ac, ce);
        copy_span<4>(lo.x, (int64_t)hi.x + 1, (int64_t)m + 1, ap, pe);
        int32_t *h = shdr(s);
        h[0] = lo.x;
        h[1] = hi.x - lo.x;
        h[2] = lo.y;
        h[3] = hi.y - lo.y;
        h[4] = (hi.y > ve || hi.y > ce || (int64_t)hi.x + 1 > pe) ? 1 : 0;  // part of a run past the copies
        uint32_t tx = 0;
        tx += ve > av ? (uint32_t)((ve - av) * sizeof(V)) : 0u;
        tx += ce > ac ? (uint32_t)((ce - ac) * 4) : 0u;
        tx += pe > ap ? (uint32_t)((pe - ap) * 4) : 0u;
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&bars[s], tx);
        if (ve > av) bulk_g2s(sval(s), val + av, (uint32_t)((ve - av) * sizeof(V)), &bars[s]);
        if (ce > ac) bulk_g2s(scol(s), col + ac, (uint32_t)((ce - ac) * 4), &bars[s]);
        if (pe > ap) bulk_g2s(srp(s), rp + ap, (uint32_t)((pe - ap) * 4), &bars[s]);
    };

    if (t == 0) {
        for (int s = 0; s < kRbStages; s++) mbar_init(&bars[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (t == 0)
        for (int k = 0; k < kRbStages; k++)
            if (g + k * G < nb) issue(k, blocks[g + k * G], blocks[g + k * G + 1]);

    for (int64_t k = 0;; k++) {
        const int64_t b = g + k * G;
        if (b >= nb) break;
        const int s = (int)(k % kRbStages);
        const uint32_t parity = (uint32_t)((k / kRbStages) & 1);
        // bounds of the block this iteration's stage takes next, loaded now so
        // their latency is spent under this block's work
        const int64_t bn = b + kRbStages * G;
        int2 nlo = make_int2(0, 0), nhi = make_int2(0, 0);
        if (t == 0 && bn < nb) {
            nlo = blocks[bn];
            nhi = blocks[bn + 1];
        }
        // One thread polls; the others sleep at the barrier, then take the
        // completed phase themselves (one poll, for its acquire).
        const bool ok = __syncthreads_and(t == 0 ? mbar_wait(&bars[s], parity) : true);
        if (!ok) {
            // A copy did not complete: record it, wait (bounded) for the
            // CTA's other copies in flight, and leave.
            if (t == 0) {
                atomicAdd(&g_csr_wait_timeouts, 1ull);
                for (int64_t k2 = k + 1; k2 < k + kRbStages && g + k2 * G < nb; k2++)
                    mbar_wait(&bars[k2 % kRbStages], (uint32_t)((k2 / kRbStages) & 1));
            }
            return;
        }
        if (t != 0) mbar_try_wait(&bars[s], parity);
        const int32_t *h = shdr(s);
        const int r0 = h[0], nr = h[1], e0 = h[2], ne = h[3];
        const bool ragged = h[4] != 0;  // the array's last block: read its tail from global memory
        constexpr int kPerV = 16 / (int)sizeof(V);
        const int av = e0 / kPerV * kPerV, ac = e0 / 4 * 4, ap = r0 / 4 * 4;
        V *vs = sval(s);
        const int32_t *cs = scol(s), *ps = srp(s);
        const int64_t vend = nnz / kPerV * kPerV, cend = nnz / 4 * 4, pend = ((int64_t)m + 1) / 4 * 4;
        if (ne > 0) {
            const int last = ne - 1;
            int c[kPer];
            V a[kPer];
#pragma unroll
            for (int j = 0; j < kPer; j++) {
                // past the block's end: the last column again (a valid gather
                // kept in flight with the others) and a zero value; each
                // thread reads only values it overwrites itself
                const int i = t + j * kBlock;
                const int e = e0 + min(i, last);
                if (!ragged) {
                    c[j] = cs[e - ac];
                    a[j] = i > last ? V(0) : vs[e - av];
                } else {
                    c[j] = e < cend ? cs[e - ac] : ld_stream(col + e);
                    a[j] = i > last ? V(0) : e < vend ? vs[e - av] : ld_stream(val + e);
                }
            }
            V xv[kPer];
#pragma unroll
            for (int j = 0; j < kPer; j++) xv[j] = ld_x(x + (int64_t)c[j] * ldx);
#pragma unroll
            for (int j = 0; j < kPer; j++) {
                const int i = t + j * kBlock;
                if (i < ne) vs[e0 + i - av] = a[j] * xv[j];
            }
        }
        __syncthreads();
        // Row sums: L lanes per row, L from the block's mean row length, so
        // that a warp's lanes read neighbouring products (one lane per row of
        // 32 nonzeros would put all 32 lanes of a warp on one bank).
        auto rows = [&](auto lanes) {
            constexpr int L = decltype(lanes)::value;
            const int lane = t & 31, sub = lane % L;
            for (int base = (t >> 5) * (32 / L); base < nr; base += kBlock / L) {
                const int i = base + lane / L;
                V sum = V(0);
                int r = r0 + i;
                if (i < nr) {
                    int rs, re;
                    if (!ragged) {
                        rs = ps[r - ap];
                        re = ps[r + 1 - ap];
                    } else {
                        rs = r < pend ? ps[r - ap] : ld_stream(rp + r);
                        re = r + 1 < pend ? ps[r + 1 - ap] : ld_stream(rp + r + 1);
                    }
                    for (int e = rs + sub; e < re; e += L) sum += vs[e - av];
                }
                if constexpr (L > 1) sum = warp_sum(sum, L);
                if (i < nr && sub == 0) {
                    V *yp = y + (int64_t)r * ldy;
                    *yp = row_out(PLAIN, alpha, sum, beta, yp);
                }
            }
        };
        const int mean = nr > 0 ? ne / nr : 0;
        if (mean < 6) rows(std::integral_constant<int, 1>());
        else if (mean < 12) rows(std::integral_constant<int, 2>());
        else if (mean < 24) rows(std::integral_constant<int, 4>());
        else rows(std::integral_constant<int, 8>());
        __syncthreads();  // stage s free
        if (t == 0) issue(k + kRbStages, nlo, nhi);
    }
}

// Plan slots of the row-block kernel: extra[4] blocks (int2, nb + 1),
// extra_i[4] = nb (-1: a row longer than kRbMaxRow, kernel not usable),
// extra_i[5] = longest row, extra_i[6] = window of the blocks built.
sspmv_status ensure_rowblock_plan(const sspmv_csr *A, Plan *p, int window, sspmv_stream_t s) {
    if (p->extra_i[4] != 0 && (p->extra_i[4] < 0 || p->extra_i[6] == window)) return SSPMV_OK;
    std::lock_guard<PlanMutex> g(plan_mutex());
    if (p->extra_i[4] != 0 && (p->extra_i[4] < 0 || p->extra_i[6] == window)) return SSPMV_OK;
    const int64_t m = A->f.num_rows, nnz = A->f.num_nnzs;
    int32_t longest = 0;
    SSPMV_TRY(max_row_length(A->row_offset, m, &longest, s));
    p->extra_i[5] = longest;
    if (longest > kRbMaxRow) {
        p->extra_i[4] = -1;
        return SSPMV_OK;
    }
    int lg = 0;
    while ((1 << lg) < window) lg++;
    int32_t *pos = nullptr;
    SSPMV_TRY(dalloc(&pos, (size_t)m, s));
    rowblock_flags<<<grid_for(m, 256), 256, 0, cu(s)>>>((int)m, lg, A->row_offset, pos);
    SSPMV_LAUNCH_CHECK();
    int32_t nb = 0;
    sspmv_status st = exclusive_scan_i32(pos, pos, m, &nb, s);
    if (st != SSPMV_OK) {
        dfree(pos, s);
        return st;
    }
    int2 *blocks = nullptr;
    st = dalloc(&blocks, (size_t)nb + 1, s);
    if (st != SSPMV_OK) {
        dfree(pos, s);
        return st;
    }
    rowblock_starts<<<grid_for(m, 256), 256, 0, cu(s)>>>((int)m, (int)nnz, lg, nb, A->row_offset, pos, blocks);
    SSPMV_LAUNCH_CHECK();
    dfree(pos, s);
    if (p->extra[4]) dfree(p->extra[4], s);
    p->extra[4] = blocks;
    p->extra_i[6] = window;
    p->extra_i[4] = nb;
    return SSPMV_OK;
}

template <typename V, int W, bool PLAIN>
sspmv_status go_rowblock_k(const sspmv_csr *A, const int2 *blocks, int64_t nb, V alpha, const V *x, int64_t ldx,
                           V beta, V *y, int64_t ldy, sspmv_stream_t s) {
    constexpr size_t smem = rowblock_smem<V, W>();
    // resident CTAs per SM, set once per instantiation after its shared
    // memory attribute (a thread that reads it non-zero may launch)
    static std::atomic<int> per_sm{0};
    if (per_sm.load(std::memory_order_acquire) == 0) {
        SSPMV_CUDA_TRY(cudaFuncSetAttribute(csr_rowblock_kernel<V, W, PLAIN>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int n = 0;
        SSPMV_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, csr_rowblock_kernel<V, W, PLAIN>, kBlock,
                                                                     smem));
        per_sm.store(n > 0 ? n : 1, std::memory_order_release);
    }
    const int64_t grid = std::min<int64_t>(nb, (int64_t)num_sms() * per_sm.load(std::memory_order_acquire));
    csr_rowblock_kernel<V, W, PLAIN><<<(unsigned)grid, kBlock, smem, cu(s)>>>(
        nb, (int)A->f.num_rows, A->f.num_nnzs, blocks, A->row_offset, A->col_index, (const V *)A->values, x, ldx,
        alpha, beta, y, ldy);
    SSPMV_LAUNCH_CHECK();
    return SSPMV_OK;
}

template <typename V, int W>
sspmv_status go_rowblock(const sspmv_csr *A, const int2 *blocks, int64_t nb, V alpha, const V *x, int64_t ldx,
                         V beta, V *y, int64_t ldy, sspmv_stream_t s) {
    if (alpha == V(1) && beta == V(0))
        return go_rowblock_k<V, W, true>(A, blocks, nb, alpha, x, ldx, beta, y, ldy, s);
    return go_rowblock_k<V, W, false>(A, blocks, nb, alpha, x, ldx, beta, y, ldy, s);
}

// Sets *launched = false (nothing launched) when the matrix has a row longer
// than kRbMaxRow or arrays that are not 16-byte aligned; the caller then runs
// another kernel.
template <typename V>
sspmv_status launch_rowblock(const sspmv_csr *A, Plan *p, V alpha, const V *x, int64_t ldx, V beta, V *y,
                             int64_t ldy, sspmv_stream_t s, bool *launched) {
    *launched = false;
    const uintptr_t bases = reinterpret_cast<uintptr_t>(A->row_offset) | reinterpret_cast<uintptr_t>(A->col_index) |
                            reinterpret_cast<uintptr_t>(A->values);
    if ((bases & 15) != 0) return SSPMV_OK;
    int window = p->param > 0 ? p->param : kRbDefaultWindow;
    if (window != 512 && window != 1024 && window != 2048 && window != 4096) window = kRbDefaultWindow;
    SSPMV_TRY(ensure_rowblock_plan(A, p, window, s));
    if (p->extra_i[4] < 0) return SSPMV_OK;
    const int2 *blocks = (const int2 *)p->extra[4];
    const int64_t nb = p->extra_i[4];
    switch (window) {
    case 512: SSPMV_TRY((go_rowblock<V, 512>(A, blocks, nb, alpha, x, ldx, beta, y, ldy, s))); break;
    case 2048: SSPMV_TRY((go_rowblock<V, 2048>(A, blocks, nb, alpha, x, ldx, beta, y, ldy, s))); break;
    case 4096: SSPMV_TRY((go_rowblock<V, 4096>(A, blocks, nb, alpha, x, ldx, beta, y, ldy, s))); break;
    default: SSPMV_TRY((go_rowblock<V, 1024>(A, blocks, nb, alpha, x, ldx, beta, y, ldy, s))); break;
    }
    *launched = true;
    return SSPMV_OK;
}

// ------------------------------------------------------- stream kernel --
// kernel_flag 0: nonzero-split "stream" kernel.  A warp takes 256 consecutive
// nonzeros, lane l the 8 at 8l (vector loads of columns and values, all 8
// gathers issued before use for k <= 2).  A lane finds the row of its first
// nonzero by binary search inside the warp's row range (row_start of the
// chunk, from the plan) and walks row_offset from there; a nonzero ends its
// row when row_offset[r + 1] == e + 1.  Rows that start and end inside a lane
// are written by it; the open sums before a lane's first row end and after
// its last are joined by one segmented shuffle scan per warp, rows crossing
// warps by a fix-up in chunk order (deterministic, no atomics).  The lane that
// ends a row also writes the empty rows right after it (and the lane holding
// nonzero 0 the empty rows before it); matrices with a run of more than
// kStreamMaxGap empty rows use the merge-path kernel instead.
constexpr int kStreamPerLane = 8;
constexpr int kStreamChunk = 32 * kStreamPerLane;
constexpr int kStreamMaxGap = 256;

__global__ void stream_row_starts(int64_t nt, int m, int64_t nnz, const int32_t *__restrict__ rp,
                                  int32_t *__restrict__ row_start) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t > nt) return;
    const int64_t e = t * kStreamChunk;
    if (e >= nnz) {
        row_start[t] = m;
        return;
    }
    int lo = 0, hi = m - 1;  // last row r with rp[r] <= e: the row holding nonzero e
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (rp[mid] <= e) lo = mid;
        else hi = mid - 1;
    }
    row_start[t] = lo;
}

// Longest run of empty rows (runs longer than kStreamMaxGap stop counting).
__global__ void stream_max_gap(int m, const int32_t *__restrict__ rp, int *__restrict__ out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        if (rp[i + 1] != rp[i] || (i > 0 && rp[i] == rp[i - 1])) continue;  // not the start of an empty run
        int len = 0;
        for (int64_t j = i; j < m && rp[j + 1] == rp[j] && len <= kStreamMaxGap; j++) len++;
        atomicMax(out, len);
    }
}

template <typename V>
__device__ __forceinline__ void stream_load8(const int32_t *__restrict__ ci, const V *__restrict__ cv, int64_t e0,
                                             int nv, bool vec, int (&c)[8], V (&a)[8]) {
    if (vec && nv == 8) {
        const int4 c0 = __ldcs(reinterpret_cast<const int4 *>(ci + e0));
        const int4 c1 = __ldcs(reinterpret_cast<const int4 *>(ci + e0 + 4));
        c[0] = c0.x; c[1] = c0.y; c[2] = c0.z; c[3] = c0.w; c[4] = c1.x; c[5] = c1.y; c[6] = c1.z; c[7] = c1.w;
        if constexpr (sizeof(V) == 8) {
#pragma unroll
            for (int h = 0; h < 4; h++) {
                const double2 v = __ldcs(reinterpret_cast<const double2 *>(cv + e0) + h);
                a[2 * h] = v.x;
                a[2 * h + 1] = v.y;
            }
        } else {
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const float4 v = __ldcs(reinterpret_cast<const float4 *>(cv + e0) + h);
                a[4 * h] = v.x; a[4 * h + 1] = v.y; a[4 * h + 2] = v.z; a[4 * h + 3] = v.w;
            }
        }
        return;
    }
#pragma unroll
    for (int u = 0; u < 8; u++) {
        c[u] = u < nv ? ld_stream(ci + e0 + u) : 0;
        a[u] = u < nv ? ld_stream(cv + e0 + u) : V(0);
    }
}

// The stream kernel for FP64 with k = 8 right-hand sides: groups of G = k
// lanes share a run of 8G consecutive nonzeros, lane q of a group owning column q,
// so each gathered row X[col, 0:k] (k consecutive values) is read by G
// adjacent lanes in one coalesced access instead of k scattered loads by one
// lane.  A group walks its nonzeros in order (loads of 8 in flight) with the
// row logic of the per-lane form; the groups' open sums are joined by a
// segmented shuffle scan with stride G.
template <typename V, int K, int G>
__device__ __forceinline__ void stream_chunk_cols(
    int m, int64_t nnz, const int32_t *__restrict__ rp, const int32_t *__restrict__ ci, const V *__restrict__ cv,
    const V *__restrict__ x, int64_t ldx, V alpha, V beta, V *__restrict__ y, int64_t ldy,
    const int32_t *__restrict__ row_start, const int64_t w, const int64_t slot, int32_t *__restrict__ carry_row,
    int32_t *__restrict__ has_end, V *__restrict__ carry_val, V *__restrict__ head_val) {
    static_assert(K % G == 0 && 32 % G == 0, "group shape");
    constexpr int KL = K / G;                 // columns per lane
    constexpr int NG = 32 / G;                // groups per warp
    constexpr int EPG = kStreamChunk / NG;    // nonzeros per group (8G)
    constexpr unsigned kFull = 0xffffffffu;
    const int lane = threadIdx.x & 31, gi = lane / G, q0 = (lane % G) * KL;
    const int64_t j0 = w * kStreamChunk;
    if (j0 >= nnz) return;  // warp-uniform
    const int64_t j1 = min(j0 + (int64_t)kStreamChunk, nnz);
    const int64_t e0 = j0 + (int64_t)gi * EPG;
    const int nv = (int)max((int64_t)0, min((int64_t)EPG, j1 - e0));
    const int ra = __ldg(row_start + w);
    const bool head_open = __ldg(rp + ra) < j0;
    int r = ra;
    if (nv > 0) {
        int lo = ra, hi = min(__ldg(row_start + w + 1), m - 1);
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(rp + mid) <= e0) lo = mid;
            else hi = mid - 1;
        }
        r = lo;
    }
    if (e0 == 0 && nv > 0) {  // empty rows before the first nonzero
        for (int r2 = 0; r2 < r; r2++) {
            V *yp = y + (int64_t)r2 * ldy + q0;
#pragma unroll
            for (int q = 0; q < KL; q++) yp[q] = axpby(alpha, V(0), beta, yp + q);
        }
    }
    int rend = nv > 0 ? __ldg(rp + r + 1) : 0;
    V seg[KL], head[KL];
#pragma unroll
    for (int q = 0; q < KL; q++) seg[q] = head[q] = V(0);
    bool any_end = false, last_open = false;
    int head_row = -1, last_row = -1;
    constexpr int SB = 8;  // nonzeros whose loads are in flight together
    for (int s0 = 0; s0 < nv; s0 += SB) {  // group-uniform
        int c[SB];
        V a[SB], xv[SB][KL];
#pragma unroll
        for (int u = 0; u < SB; u++) {
            const bool ok = s0 + u < nv;
            c[u] = ok ? ld_stream(ci + e0 + s0 + u) : 0;
            a[u] = ok ? ld_stream(cv + e0 + s0 + u) : V(0);
        }
#pragma unroll
        for (int u = 0; u < SB; u++)
#pragma unroll
            for (int q = 0; q < KL; q++)
                xv[u][q] = s0 + u < nv ? ld_x(x + (int64_t)c[u] * ldx + q0 + q) : V(0);
#pragma unroll
        for (int u = 0; u < SB; u++) {
            if (s0 + u < nv) {
                const int64_t e = e0 + s0 + u;
                while (rend <= e) rend = __ldg(rp + (++r) + 1);
#pragma unroll
                for (int q = 0; q < KL; q++) seg[q] += a[u] * xv[u][q];
                last_row = r;
                last_open = rend != e + 1;
                if (!last_open) {
                    if (!any_end) {
                        any_end = true;
                        head_row = r;
#pragma unroll
                        for (int q = 0; q < KL; q++) head[q] = seg[q];
                    } else {
                        V *yp = y + (int64_t)r * ldy + q0;
#pragma unroll
                        for (int q = 0; q < KL; q++) yp[q] = axpby(alpha, seg[q], beta, yp + q);
                    }
#pragma unroll
                    for (int q = 0; q < KL; q++) seg[q] = V(0);
                    for (int r2 = r + 1; r2 < m && __ldg(rp + r2 + 1) == e + 1; r2++) {
                        V *yp = y + (int64_t)r2 * ldy + q0;
#pragma unroll
                        for (int q = 0; q < KL; q++) yp[q] = axpby(alpha, V(0), beta, yp + q);
                    }
                }
            }
        }
    }
    V S[KL];
#pragma unroll
    for (int q = 0; q < KL; q++) S[q] = seg[q];
    bool f = any_end;
#pragma unroll
    for (int o = 1; o < NG; o <<= 1) {
        V up[KL];
#pragma unroll
        for (int q = 0; q < KL; q++) up[q] = __shfl_up_sync(kFull, S[q], o * G);
        const bool fu = __shfl_up_sync(kFull, f, o * G);
        if (gi >= o) {
            if (!f) {
#pragma unroll
                for (int q = 0; q < KL; q++) S[q] += up[q];
            }
            f = f || fu;
        }
    }
    V cin[KL];
#pragma unroll
    for (int q = 0; q < KL; q++) {
        cin[q] = __shfl_up_sync(kFull, S[q], G);
        if (gi == 0) cin[q] = V(0);
    }
    if (any_end) {
        V tot[KL];
#pragma unroll
        for (int q = 0; q < KL; q++) tot[q] = head[q] + cin[q];
        if (head_row == ra && head_open) {
            V *hp = head_val + slot * kMaxK + q0;
#pragma unroll
            for (int q = 0; q < KL; q++) hp[q] = tot[q];
        } else {
            V *yp = y + (int64_t)head_row * ldy + q0;
#pragma unroll
            for (int q = 0; q < KL; q++) yp[q] = axpby(alpha, tot[q], beta, yp + q);
        }
    }
    const bool chunk_end = __any_sync(kFull, any_end);
    if (nv > 0 && e0 + nv == j1) {  // the group holding the chunk's last nonzero
        if (q0 == 0) {
            has_end[slot] = chunk_end ? 1 : 0;
            carry_row[slot] = last_open ? last_row : -1;
        }
        if (last_open) {
            V *cp = carry_val + slot * kMaxK + q0;
#pragma unroll
            for (int q = 0; q < KL; q++) cp[q] = S[q];
        }
    }
}

// Chunk w (nonzeros 256w ..) of one matrix, run by one warp; `slot` indexes
// the carry arrays.  Shared by the single-matrix kernel and the batched
// serving kernel.
template <typename V, int K, bool PLAIN = false>
__device__ __forceinline__ void stream_chunk_lanes(
    int m, int64_t nnz, const int32_t *__restrict__ rp, const int32_t *__restrict__ ci, const V *__restrict__ cv,
    const V *__restrict__ x, int64_t ldx, V alpha, V beta, V *__restrict__ y, int64_t ldy,
    const int32_t *__restrict__ row_start, const int64_t w, const int64_t slot, int32_t *__restrict__ carry_row,
    int32_t *__restrict__ has_end, V *__restrict__ carry_val, V *__restrict__ head_val, int vec, int xvec) {
    constexpr unsigned kFull = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    constexpr bool plain = PLAIN;  // alpha == 1 and beta == 0: y = sum
    const int64_t j0 = w * kStreamChunk;
    if (j0 >= nnz) return;  // warp-uniform
    const int64_t j1 = min(j0 + (int64_t)kStreamChunk, nnz);
    const int64_t e0 = j0 + (int64_t)lane * kStreamPerLane;
    const int nv = (int)max((int64_t)0, min((int64_t)kStreamPerLane, j1 - e0));
    int c[8];
    V a[8];
    stream_load8<V>(ci, cv, e0, nv, vec != 0, c, a);
    const int ra = __ldg(row_start + w);
    const bool head_open = __ldg(rp + ra) < j0;  // the chunk's first row began in an earlier chunk
    int r = ra;
    if (nv > 0) {
        int lo = ra, hi = min(__ldg(row_start + w + 1), m - 1);
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(rp + mid) <= e0) lo = mid;
            else hi = mid - 1;
        }
        r = lo;
    }
    V xv[K <= 2 ? 8 : 1][K];
    if constexpr (K <= 2) {
#pragma unroll
        for (int u = 0; u < 8; u++) {
            if (u < nv) {
                ld_xrow<V, K>(x, c[u], ldx, xvec != 0, xv[u]);
            } else {
#pragma unroll
                for (int q = 0; q < K; q++) xv[u][q] = V(0);
            }
        }
    }
    if (e0 == 0 && nv > 0) {  // empty rows before the first nonzero
        for (int r2 = 0; r2 < r; r2++) {
            V *yp = y + (int64_t)r2 * ldy;
#pragma unroll
            for (int q = 0; q < K; q++) yp[q] = row_out(plain, alpha, V(0), beta, yp + q);
        }
    }
    int rend = nv > 0 ? __ldg(rp + r + 1) : 0;
    V seg[K], head[K];
#pragma unroll
    for (int q = 0; q < K; q++) seg[q] = head[q] = V(0);
    bool any_end = false, last_open = false;
    int head_row = -1, last_row = -1;
#pragma unroll
    for (int u = 0; u < 8; u++) {
        if (u < nv) {
            const int64_t e = e0 + u;
            while (rend <= e) rend = __ldg(rp + (++r) + 1);  // skip empty rows
            if constexpr (K <= 2) {
#pragma unroll
                for (int q = 0; q < K; q++) seg[q] += a[u] * xv[u][q];
            } else {
                V xr[K];
                ld_xrow<V, K>(x, c[u], ldx, xvec != 0, xr);
#pragma unroll
                for (int q = 0; q < K; q++) seg[q] += a[u] * xr[q];
            }
            last_row = r;
            last_open = rend != e + 1;
            if (!last_open) {  // row r ends at e
                if (!any_end) {
                    any_end = true;
                    head_row = r;
#pragma unroll
                    for (int q = 0; q < K; q++) head[q] = seg[q];
                } else {
                    V *yp = y + (int64_t)r * ldy;
#pragma unroll
                    for (int q = 0; q < K; q++) yp[q] = row_out(plain, alpha, seg[q], beta, yp + q);
                }
#pragma unroll
                for (int q = 0; q < K; q++) seg[q] = V(0);
                for (int r2 = r + 1; r2 < m && __ldg(rp + r2 + 1) == e + 1; r2++) {  // empty rows after r
                    V *yp = y + (int64_t)r2 * ldy;
#pragma unroll
                    for (int q = 0; q < K; q++) yp[q] = row_out(plain, alpha, V(0), beta, yp + q);
                }
            }
        }
    }
    V S[K];
#pragma unroll
    for (int q = 0; q < K; q++) S[q] = seg[q];
    bool f = any_end;
    const int span = unflagged_run(f);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        if (o > span) break;  // warp-uniform
        V up[K];
#pragma unroll
        for (int q = 0; q < K; q++) up[q] = __shfl_up_sync(kFull, S[q], o);
        const bool fu = __shfl_up_sync(kFull, f, o);
        if (lane >= o) {
            if (!f) {
#pragma unroll
                for (int q = 0; q < K; q++) S[q] += up[q];
            }
            f = f || fu;
        }
    }
    V cin[K];
#pragma unroll
    for (int q = 0; q < K; q++) {
        cin[q] = __shfl_up_sync(kFull, S[q], 1);
        if (lane == 0) cin[q] = V(0);
    }
    if (any_end) {
        V tot[K];
#pragma unroll
        for (int q = 0; q < K; q++) tot[q] = head[q] + cin[q];
        if (head_row == ra && head_open) {
            V *hp = head_val + slot * kMaxK;
#pragma unroll
            for (int q = 0; q < K; q++) hp[q] = tot[q];
        } else {
            V *yp = y + (int64_t)head_row * ldy;
#pragma unroll
            for (int q = 0; q < K; q++) yp[q] = row_out(plain, alpha, tot[q], beta, yp + q);
        }
    }
    const bool chunk_end = __any_sync(kFull, any_end);
    if (nv > 0 && e0 + nv == j1) {  // the lane holding the chunk's last nonzero
        has_end[slot] = chunk_end ? 1 : 0;
        carry_row[slot] = last_open ? last_row : -1;
        if (last_open) {
            V *cp = carry_val + slot * kMaxK;
#pragma unroll
            for (int q = 0; q < K; q++) cp[q] = S[q];
        }
    }
}

// The chunk of a matrix without empty rows: the rows starting inside the
// chunk are read once (row_offset[ra ..], one row per lane per step) and
// marked as bits in shared memory (one 8-bit word per lane, position p of the
// chunk at word p / 8, bit p % 8); each lane then knows which of its 8
// nonzeros end a row (the next position starts one) and, by a prefix count of
// the bits, the row of its first nonzero -- no search and no chain of
// dependent loads on row_offset.  The arithmetic (per-lane sums in nonzero
// order, the segmented scan, the carry slots) is that of stream_chunk_lanes,
// so both give the same bits.  sbits: the warp's 33 words of shared memory.
template <typename V, int K, bool PLAIN = false>
__device__ __forceinline__ void stream_chunk_fast(
    int m, int64_t nnz, const int32_t *__restrict__ rp, const int32_t *__restrict__ ci, const V *__restrict__ cv,
    const V *__restrict__ x, int64_t ldx, V alpha, V beta, V *__restrict__ y, int64_t ldy, const int ra,
    const int last, const int64_t w, const int64_t slot, int32_t *__restrict__ carry_row,
    int32_t *__restrict__ has_end, V *__restrict__ carry_val, V *__restrict__ head_val, int vec, int xvec,
    uint32_t *__restrict__ sbits) {
    constexpr unsigned kFull = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    constexpr bool plain = PLAIN;  // alpha == 1 and beta == 0: y = sum
    const int64_t j0 = w * kStreamChunk;
    const int64_t j1 = min(j0 + (int64_t)kStreamChunk, nnz);
    const int64_t e0 = j0 + (int64_t)lane * kStreamPerLane;
    const int nv = (int)max((int64_t)0, min((int64_t)kStreamPerLane, j1 - e0));
    int c[8];
    V a[8];
    stream_load8<V>(ci, cv, e0, nv, vec != 0, c, a);
    sbits[lane] = 0u;
    if (lane == 0) sbits[32] = 0u;
    __syncwarp();
    // rows ra .. last (last = one past the row holding the chunk's end): mark
    // each start p in (0, 256] (p = 256: a row starting right after the chunk)
    bool head_open = false;
    for (int r0 = ra; r0 <= last; r0 += 32) {  // warp-uniform
        const int rr = r0 + lane;
        if (rr <= last) {
            const int64_t p = (int64_t)__ldg(rp + rr) - j0;
            if (p > 0 && p <= kStreamChunk) atomicOr(sbits + (p >> 3), 1u << (p & 7));
            if (rr == ra) head_open = p < 0;  // the chunk's first row began in an earlier chunk
        }
    }
    head_open = __shfl_sync(kFull, head_open, 0);
    __syncwarp();
    const uint32_t starts = sbits[lane], starts_next = sbits[lane + 1];
    // bit u of `ends`: nonzero u ends its row (a row starts at e0 + u + 1)
    const uint32_t ends = (starts >> 1) | ((starts_next & 1u) << 7);
    // the lane's first row: ra + the starts in (j0, e0]
    int before = __popc(starts);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(kFull, before, o);
        if (lane >= o) before += t;
    }
    before -= __popc(starts);  // starts in lanes before this one
    const int pos = before + (int)(starts & 1u);
    V xv[K <= 2 ? 8 : 1][K];
    if constexpr (K <= 2) {
#pragma unroll
        for (int u = 0; u < 8; u++) {
            if (u < nv) {
                ld_xrow<V, K>(x, c[u], ldx, xvec != 0, xv[u]);
            } else {
#pragma unroll
                for (int q = 0; q < K; q++) xv[u][q] = V(0);
            }
        }
    }
    int r = ra + pos;
    V seg[K], head[K];
#pragma unroll
    for (int q = 0; q < K; q++) seg[q] = head[q] = V(0);
    bool any_end = false, last_open = false;
    int head_row = -1, last_row = -1;
#pragma unroll
    for (int u = 0; u < 8; u++) {
        if (u < nv) {
            if constexpr (K <= 2) {
#pragma unroll
                for (int q = 0; q < K; q++) seg[q] += a[u] * xv[u][q];
            } else {
                V xr[K];
                ld_xrow<V, K>(x, c[u], ldx, xvec != 0, xr);
#pragma unroll
                for (int q = 0; q < K; q++) seg[q] += a[u] * xr[q];
            }
            last_row = r;
            last_open = !((ends >> u) & 1u);
            if (!last_open) {  // row r ends here
                if (!any_end) {
                    any_end = true;
                    head_row = r;
#pragma unroll
                    for (int q = 0; q < K; q++) head[q] = seg[q];
                } else {
                    V *yp = y + (int64_t)r * ldy;
#pragma unroll
                    for (int q = 0; q < K; q++) yp[q] = row_out(plain, alpha, seg[q], beta, yp + q);
                }
#pragma unroll
                for (int q = 0; q < K; q++) seg[q] = V(0);
                r++;
            }
        }
    }
    V S[K];
#pragma unroll
    for (int q = 0; q < K; q++) S[q] = seg[q];
    bool f = any_end;
    const int span = unflagged_run(f);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        if (o > span) break;  // warp-uniform
        V up[K];
#pragma unroll
        for (int q = 0; q < K; q++) up[q] = __shfl_up_sync(kFull, S[q], o);
        const bool fu = __shfl_up_sync(kFull, f, o);
        if (lane >= o) {
            if (!f) {
#pragma unroll
                for (int q = 0; q < K; q++) S[q] += up[q];
            }
            f = f || fu;
        }
    }
    V cin[K];
#pragma unroll
    for (int q = 0; q < K; q++) {
        cin[q] = __shfl_up_sync(kFull, S[q], 1);
        if (lane == 0) cin[q] = V(0);
    }
    if (any_end) {
        V tot[K];
#pragma unroll
        for (int q = 0; q < K; q++) tot[q] = head[q] + cin[q];
        if (head_row == ra && head_open) {
            V *hp = head_val + slot * kMaxK;
#pragma unroll
            for (int q = 0; q < K; q++) hp[q] = tot[q];
        } else {
            V *yp = y + (int64_t)head_row * ldy;
#pragma unroll
            for (int q = 0; q < K; q++) yp[q] = row_out(plain, alpha, tot[q], beta, yp + q);
        }
    }
    const bool chunk_end = __any_sync(kFull, any_end);
    if (nv > 0 && e0 + nv == j1) {  // the lane holding the chunk's last nonzero
        has_end[slot] = chunk_end ? 1 : 0;
        carry_row[slot] = last_open ? last_row : -1;
        if (last_open) {
            V *cp = carry_val + slot * kMaxK;
#pragma unroll
            for (int q = 0; q < K; q++) cp[q] = S[q];
        }
    }
}

// One lane per nonzero run (stream_chunk_lanes), except FP64 with k = 8:
// column groups (stream_chunk_cols), which read each 64-byte row of X with
// one coalesced access (measured 1.3-1.4x faster there; slower for FP32 and
// mixed for k = 4).
template <typename V, int K, bool PLAIN = false>
__device__ __forceinline__ void stream_chunk(
    int m, int64_t nnz, const int32_t *__restrict__ rp, const int32_t *__restrict__ ci, const V *__restrict__ cv,
    const V *__restrict__ x, int64_t ldx, V alpha, V beta, V *__restrict__ y, int64_t ldy,
    const int32_t *__restrict__ row_start, const int64_t w, const int64_t slot, int32_t *__restrict__ carry_row,
    int32_t *__restrict__ has_end, V *__restrict__ carry_val, V *__restrict__ head_val, int vec, int xvec,
    int no_empty, uint32_t *__restrict__ sbits) {
    if constexpr (K == 8 && sizeof(V) == 8) {
        stream_chunk_cols<V, K, K>(m, nnz, rp, ci, cv, x, ldx, alpha, beta, y, ldy, row_start, w, slot, carry_row,
                                   has_end, carry_val, head_val);
    } else {
        if (no_empty && w * kStreamChunk < nnz) {  // warp-uniform
            const int ra = __ldg(row_start + w);
            const int last = min(__ldg(row_start + w + 1), m - 1) + 1;
            stream_chunk_fast<V, K, PLAIN>(m, nnz, rp, ci, cv, x, ldx, alpha, beta, y, ldy, ra, last, w, slot,
                                           carry_row, has_end, carry_val, head_val, vec, xvec, sbits);
            return;
        }
        stream_chunk_lanes<V, K, PLAIN>(m, nnz, rp, ci, cv, x, ldx, alpha, beta, y, ldy, row_start, w, slot,
                                        carry_row, has_end, carry_val, head_val, vec, xvec);
    }
}

#define SSPMV_STREAM_KERNEL_BODY                                                                          \
    __shared__ uint32_t s_bits[kBlock / 32][33];                                                          \
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;                              \
    stream_chunk<V, K, PLAIN>(m, nnz, rp, ci, cv, x, ldx, alpha, beta, y, ldy, row_start, w, w, carry_row,    \
                              has_end, carry_val, head_val, vec, xvec, no_empty, s_bits[threadIdx.x >> 5]);

// PLAIN: alpha == 1 and beta == 0 (y = sum), instantiated for k = 1: the
// rows' writes then carry no FP64 multiply.
template <typename V, int K, bool PLAIN = false>
__global__ void __launch_bounds__(kBlock) csr_stream_kernel(
    int m, int64_t nnz, const int32_t *__restrict__ rp, const int32_t *__restrict__ ci, const V *__restrict__ cv,
    const V *__restrict__ x, int64_t ldx, V alpha, V beta, V *__restrict__ y, int64_t ldy,
    const int32_t *__restrict__ row_start, int32_t *__restrict__ carry_row, int32_t *__restrict__ has_end,
    V *__restrict__ carry_val, V *__restrict__ head_val, int vec, int xvec, int no_empty) {
    SSPMV_STREAM_KERNEL_BODY
}

// The same kernel held to six resident CTAs per SM (at most 42 registers):
// measured 5-8% faster for FP32 at k = 1; FP64 slows down when squeezed.
template <typename V, int K, bool PLAIN = false>
__global__ void __launch_bounds__(kBlock, 6) csr_stream_kernel_occ6(
    int m, int64_t nnz, const int32_t *__restrict__ rp, const int32_t *__restrict__ ci, const V *__restrict__ cv,
    const V *__restrict__ x, int64_t ldx, V alpha, V beta, V *__restrict__ y, int64_t ldy,
    const int32_t *__restrict__ row_start, int32_t *__restrict__ carry_row, int32_t *__restrict__ has_end,
    V *__restrict__ carry_val, V *__restrict__ head_val, int vec, int xvec, int no_empty) {
    SSPMV_STREAM_KERNEL_BODY
}
#undef SSPMV_STREAM_KERNEL_BODY

// Rows crossing chunks: a thread per chunk; the chunk where the row starts
// adds the later chunks' pieces (chain_sum).
template <typename V, int K>
__global__ void csr_stream_fixup(int64_t nt, const int32_t *__restrict__ rp, const int32_t *__restrict__ carry_row,
                                 const int32_t *__restrict__ has_end, const V *__restrict__ carry_val,
                                 const V *__restrict__ head_val, V alpha, V beta, V *__restrict__ y, int64_t ldy) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t - (threadIdx.x & 31) >= nt) return;  // whole warp past the end
    const int r = t < nt ? carry_row[t] : -1;
    const bool mine = r >= 0 && (int64_t)rp[r] >= t * kStreamChunk;  // open here and began here
    V tot[K];
    chain_sum<V, K>(mine, t, nt, 0, has_end, carry_val, head_val, tot);
    if (mine) {
        V *yp = y + (int64_t)r * ldy;
#pragma unroll
        for (int q = 0; q < K; q++) yp[q] = axpby(alpha, tot[q], beta, yp + q);
    }
}

// Plan slots of the stream kernel (CSR matrices use no other extra slots):
// extra[0] row_start[nt + 1], extra[1] carry_row/has_end [2 nt], extra[2]
// carry values, extra[3] head values; extra_i[0] = nt, extra_i[1] = longest
// empty-row run (capped just above kStreamMaxGap).
sspmv_status ensure_stream_plan(const sspmv_csr *A, Plan *p, sspmv_stream_t s) {
    if (p->extra[0]) return SSPMV_OK;
    std::lock_guard<PlanMutex> g(plan_mutex());
    if (p->extra[0]) return SSPMV_OK;
    const int64_t m = A->f.num_rows, nnz = A->f.num_nnzs;
    const int64_t nt = std::max<int64_t>((nnz + kStreamChunk - 1) / kStreamChunk, 1);
    const size_t sv = vsize(A->f.value_type);
    int32_t *starts = nullptr, *ints = nullptr;
    unsigned char *cvals = nullptr, *hvals = nullptr;
    int *gap = nullptr;
    SSPMV_TRY(dalloc(&starts, (size_t)nt + 1, s));
    SSPMV_TRY(dalloc(&ints, (size_t)nt * 2, s));
    SSPMV_TRY(dalloc(&cvals, (size_t)nt * kMaxK * sv, s));
    SSPMV_TRY(dalloc(&hvals, (size_t)nt * kMaxK * sv, s));
    SSPMV_TRY(dalloc(&gap, 1, s));
    SSPMV_CUDA_TRY(cudaMemsetAsync(gap, 0, sizeof(int), cu(s)));
    stream_row_starts<<<grid_for(nt + 1, 256), 256, 0, cu(s)>>>(nt, (int)m, nnz, A->row_offset, starts);
    SSPMV_LAUNCH_CHECK();
    stream_max_gap<<<grid_for(m, 256, (int64_t)num_sms() * 16), 256, 0, cu(s)>>>((int)m, A->row_offset, gap);
    SSPMV_LAUNCH_CHECK();
    int hgap = 0;
    SSPMV_CUDA_TRY(cudaMemcpyAsync(&hgap, gap, sizeof(int), cudaMemcpyDeviceToHost, cu(s)));
    SSPMV_CUDA_TRY(cudaStreamSynchronize(cu(s)));
    dfree(gap, s);
    p->extra_i[0] = nt;
    p->extra_i[1] = hgap;
    p->extra[1] = ints;
    p->extra[2] = cvals;
    p->extra[3] = hvals;
    p->extra[0] = starts;  // published last
    return SSPMV_OK;
}

template <typename V, int K>
sspmv_status launch_stream(const sspmv_csr *A, Plan *p, V alpha, const V *x, int64_t ldx, V beta, V *y,
                           int64_t ldy, sspmv_stream_t s) {
    if (A->f.num_nnzs == 0) return launch_merge<V, K>(A, p, alpha, x, ldx, beta, y, ldy, s);
    SSPMV_TRY(ensure_stream_plan(A, p, s));
    if (p->extra_i[1] > kStreamMaxGap) return launch_merge<V, K>(A, p, alpha, x, ldx, beta, y, ldy, s);
    const int64_t nt = p->extra_i[0];
    int32_t *ints = (int32_t *)p->extra[1];
    const int vec = ((reinterpret_cast<uintptr_t>(A->col_index) | reinterpret_cast<uintptr_t>(A->values)) & 15) == 0;
    const unsigned grid = grid_for(nt * 32, kBlock);
    const int no_empty = p->extra_i[1] == 0 ? 1 : 0;
    const int xvec = xrow_vec(x, ldx, sizeof(V), K);
    auto go = [&](auto kernel) {
        kernel<<<grid, kBlock, 0, cu(s)>>>((int)A->f.num_rows, A->f.num_nnzs, A->row_offset, A->col_index,
                                           (const V *)A->values, x, ldx, alpha, beta, y, ldy,
                                           (const int32_t *)p->extra[0], ints, ints + nt, (V *)p->extra[2],
                                           (V *)p->extra[3], vec, xvec, no_empty);
    };
    const bool plain = alpha == V(1) && beta == V(0);
    if constexpr (sizeof(V) == 4 && K == 1) {
        if (plain) go(csr_stream_kernel_occ6<V, K, true>);
        else go(csr_stream_kernel_occ6<V, K>);
    } else if constexpr (K == 1) {
        if (plain) go(csr_stream_kernel<V, K, true>);
        else go(csr_stream_kernel<V, K>);
    } else {
        go(csr_stream_kernel<V, K>);
    }
    SSPMV_LAUNCH_CHECK();
    if (nt > 1) {
        csr_stream_fixup<V, K><<<grid_for(nt, 256), 256, 0, cu(s)>>>(nt, A->row_offset, ints, ints + nt,
                                                                     (const V *)p->extra[2], (const V *)p->extra[3],
                                                                     alpha, beta, y, ldy);
        SSPMV_LAUNCH_CHECK();
    }
    return SSPMV_OK;
}

// ---------------------------------------------------- batched (serving) --
// Index of the item owning global chunk gc: the last item whose chunk_begin
// is <= gc (items of a group have increasing chunk_begin).
__device__ __forceinline__ int batch_item_of(const BatchItem *__restrict__ items, int n, int64_t gc) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&items[mid].chunk_begin) <= gc) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Persistent stream kernel over the chunks of every request of group g:
// warp i of the grid takes global chunks i, i + warps, ...  A request is cut
// into the chunks a lone sspmv_spmm_csr call uses (the matrix's own
// row_start), and its carries go to per-batch slots, so its result does not
// depend on the rest of the batch and equals the single-request call's.
template <typename V, int K>
__global__ void __launch_bounds__(kBlock) csr_batch_kernel(int g, const BatchHeader *__restrict__ hdr,
                                                           const BatchItem *__restrict__ all_items,
                                                           int32_t *__restrict__ carry_row,
                                                           int32_t *__restrict__ has_end, V *__restrict__ carry_val,
                                                           V *__restrict__ head_val) {
    const int n = hdr->n_items[g];
    const int64_t total = hdr->total_chunks[g];
    const int64_t base = hdr->carry_base[g];
    const BatchItem *items = all_items + hdr->item_begin[g];
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t gc = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; gc < total; gc += warps) {
        const BatchItem *q = items + batch_item_of(items, n, gc);
        stream_chunk<V, K>(q->m, q->nnz, q->row_offset, q->col_index, (const V *)q->values, (const V *)q->x, q->ldx,
                           (V)q->alpha, (V)q->beta, (V *)q->y, q->ldy, q->row_start, gc - q->chunk_begin, base + gc,
                           carry_row, has_end, carry_val, head_val, q->vec, q->xvec, 0, nullptr);
    }
}

// The batched counterpart of csr_stream_fixup: one thread per global chunk.
template <typename V, int K>
__global__ void csr_batch_fixup(int g, const BatchHeader *__restrict__ hdr, const BatchItem *__restrict__ all_items,
                                const int32_t *__restrict__ carry_row, const int32_t *__restrict__ has_end,
                                const V *__restrict__ carry_val, const V *__restrict__ head_val) {
    const int n = hdr->n_items[g];
    const int64_t total = hdr->total_chunks[g];
    const int64_t base = hdr->carry_base[g];
    const BatchItem *items = all_items + hdr->item_begin[g];
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    // warp-uniform trip count: lane l takes global chunk w0 + l of each round
    for (int64_t w0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x - lane; w0 < total; w0 += stride) {
        const int64_t gc = w0 + lane;
        const BatchItem *q = gc < total ? items + batch_item_of(items, n, gc) : items;
        const int64_t t = gc - q->chunk_begin, nt = q->num_chunks;
        const int64_t slot = base + gc;
        const int r = gc < total && nt > 1 ? carry_row[slot] : -1;
        const bool mine = r >= 0 && (int64_t)q->row_offset[r] >= t * kStreamChunk;
        V tot[K];
        const int64_t shift = slot - t;  // chunk u of this lane's item lives in slot u + shift
        chain_sum<V, K>(mine, t, nt, shift, has_end, carry_val, head_val, tot);
        if (mine) {
            V *yp = (V *)q->y + (int64_t)r * q->ldy;
            const V alpha = (V)q->alpha, beta = (V)q->beta;
#pragma unroll
            for (int c = 0; c < K; c++) yp[c] = axpby(alpha, tot[c], beta, yp + c);
        }
    }
}

// Resident CTAs per SM of csr_batch_kernel<V, K>.
template <typename V, int K>
int batch_blocks_per_sm() {
    static int blocks = 0;
    if (blocks == 0) {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, csr_batch_kernel<V, K>, kBlock, 0) != cudaSuccess ||
            b < 1)
            b = 1;
        blocks = b;
    }
    return blocks;
}

template <typename V, int K>
sspmv_status launch_batch_vk(int g, const BatchHeader *hdr, const BatchItem *items, void *carry, int64_t slots,
                             sspmv_stream_t s) {
    unsigned char *c = (unsigned char *)carry;
    int32_t *carry_row = (int32_t *)c;
    int32_t *has_end = (int32_t *)(c + (size_t)slots * 4);
    V *carry_val = (V *)(c + (size_t)slots * 8);
    V *head_val = (V *)(c + (size_t)slots * (8 + kMaxK * 8));
    const unsigned grid = (unsigned)(num_sms() * batch_blocks_per_sm<V, K>());
    csr_batch_kernel<V, K><<<grid, kBlock, 0, cu(s)>>>(g, hdr, items, carry_row, has_end, carry_val, head_val);
    SSPMV_LAUNCH_CHECK();
    csr_batch_fixup<V, K><<<(unsigned)num_sms() * 4, 256, 0, cu(s)>>>(g, hdr, items, carry_row, has_end, carry_val,
                                                                        head_val);
    SSPMV_LAUNCH_CHECK();
    return SSPMV_OK;
}

// kernel_flag 0 (default): stream kernel (merge-path for matrices it does
// not take; the request server's batched CSR work sums in the same order, so
// a request's result does not depend on whether it was batched); 1: vector;
// 2: merge-path; 3: row-block; 4: pipelined thread per row (3 and 4 fall
// back to the default on matrices they do not take).
template <typename V, int K>
sspmv_status csr_pass(const sspmv_csr *A, Plan *p, V alpha, const V *x, int64_t ldx, V beta, V *y,
                      int64_t ldy, sspmv_stream_t s) {
    if (A->f.kernel_flag == 1) return launch_vector<V, K>(A, p, alpha, x, ldx, beta, y, ldy, s);
    if (A->f.kernel_flag == 2) return launch_merge<V, K>(A, p, alpha, x, ldx, beta, y, ldy, s);
    if constexpr (K == 1) {
        if (A->f.kernel_flag == 3) {
            bool launched = false;
            SSPMV_TRY(launch_rowblock<V>(A, p, alpha, x, ldx, beta, y, ldy, s, &launched));
            if (launched) return SSPMV_OK;
        }
        if (A->f.kernel_flag == 4) {
            bool launched = false;
            SSPMV_TRY(launch_csr_pipe<V>(A, p, alpha, x, ldx, beta, y, ldy, s, &launched));
            if (launched) return SSPMV_OK;
        }
    }
    return launch_stream<V, K>(A, p, alpha, x, ldx, beta, y, ldy, s);
}

}  // namespace

sspmv_status check_spmm_args(const sspmv_features *f, int32_t k, const void *X, int64_t ldx, const void *Y,
                             int64_t ldy) {
    if (k < 1) return fail(SSPMV_INVALID_ARG, "k must be >= 1 (got %d)", k);
    if (ldx < k || ldy < k) return fail(SSPMV_INVALID_ARG, "ldx/ldy must be >= k");
    if ((f->num_cols > 0 && !X) || (f->num_rows > 0 && !Y)) return fail(SSPMV_INVALID_ARG, "null x or y");
    if (!valid_vt(f->value_type)) return fail(SSPMV_INVALID_ARG, "bad value_type");
    return SSPMV_OK;
}

sspmv_status spmm_csr_impl(double alpha, const sspmv_csr *A, int32_t k, const void *X, int64_t ldx, double beta,
                           void *Y, int64_t ldy, sspmv_stream_t s) {
    if (!A) return fail(SSPMV_INVALID_ARG, "null matrix");
    SSPMV_TRY(check_spmm_args(&A->f, k, X, ldx, Y, ldy));
    if (A->f.num_rows == 0) return SSPMV_OK;
    Plan *p = get_plan(&A->f);
    if (!p) return fail(SSPMV_OUT_OF_MEMORY, "plan allocation failed");
    return dispatch_value(A->f.value_type, [&](auto tag) -> sspmv_status {
        using V = decltype(tag);
        return for_rhs_chunks<V>(k, (const V *)X, (V *)Y, [&](int32_t step, const V *xs, V *ys) {
            const V a = (V)alpha, b = (V)beta;
            switch (step) {
            case 8: return csr_pass<V, 8>(A, p, a, xs, ldx, b, ys, ldy, s);
            case 4: return csr_pass<V, 4>(A, p, a, xs, ldx, b, ys, ldy, s);
            case 2: return csr_pass<V, 2>(A, p, a, xs, ldx, b, ys, ldy, s);
            default: return csr_pass<V, 1>(A, p, a, xs, ldx, b, ys, ldy, s);
            }
        });
    });
}

sspmv_status ensure_merge_plan(Plan *p, int which, int64_t m, int64_t nnz, const int32_t *row_offset,
                               int32_t value_type, sspmv_stream_t s) {
    MergePlan &mp = p->merge[which];
    if (mp.coords) return SSPMV_OK;
    std::lock_guard<PlanMutex> g(plan_mutex());
    if (mp.coords) return SSPMV_OK;
    const int tile = which == 0 ? MergeShape<1>::tile : MergeShape<8>::tile;
    const int64_t tiles = (m + nnz + tile - 1) / tile;
    const int64_t nt = tiles > 0 ? tiles : 1;
    MergePlan q;
    q.tile_items = tile;
    q.num_tiles = nt;
    const size_t vs = vsize(value_type);
    SSPMV_TRY(dalloc(&q.coords, (size_t)nt + 1, s));
    SSPMV_TRY(dalloc(&q.carry_row, (size_t)nt, s));
    SSPMV_TRY(dalloc(&q.has_end, (size_t)nt, s));
    SSPMV_TRY(dalloc((unsigned char **)&q.carry_val, (size_t)nt * kMaxK * vs, s));
    SSPMV_TRY(dalloc((unsigned char **)&q.head_val, (size_t)nt * kMaxK * vs, s));
    merge_path_search<<<grid_for(nt + 1, 256), 256, 0, cu(s)>>>(nt, tile, (int)m, (int)nnz, row_offset, q.coords);
    SSPMV_LAUNCH_CHECK();
    mp = q;
    return SSPMV_OK;
}

sspmv_status csr_stream_plan(const sspmv_csr *A, const int32_t **row_start, int64_t *num_chunks, int32_t *max_gap,
                             sspmv_stream_t s) {
    Plan *p = get_plan(&A->f);
    if (!p) return fail(SSPMV_OUT_OF_MEMORY, "plan allocation failed");
    SSPMV_TRY(ensure_stream_plan(A, p, s));
    *row_start = (const int32_t *)p->extra[0];
    *num_chunks = p->extra_i[0];
    *max_gap = (int32_t)p->extra_i[1];
    return SSPMV_OK;
}

bool csr_stream_takes(int64_t num_nnzs, int32_t max_gap) { return num_nnzs > 0 && max_gap <= kStreamMaxGap; }

unsigned csr_batch_grid(int g) {
    int b = 1;
    switch (g) {
    case 0: b = batch_blocks_per_sm<float, 1>(); break;
    case 1: b = batch_blocks_per_sm<float, 2>(); break;
    case 2: b = batch_blocks_per_sm<float, 4>(); break;
    case 3: b = batch_blocks_per_sm<float, 8>(); break;
    case 4: b = batch_blocks_per_sm<double, 1>(); break;
    case 5: b = batch_blocks_per_sm<double, 2>(); break;
    case 6: b = batch_blocks_per_sm<double, 4>(); break;
    default: b = batch_blocks_per_sm<double, 8>(); break;
    }
    return (unsigned)(num_sms() * b);
}

sspmv_status launch_csr_batch_group(int g, const BatchHeader *d_hdr, const BatchItem *d_items, void *carry,
                                    int64_t carry_slots, sspmv_stream_t s) {
    switch (g) {
    case 0: return launch_batch_vk<float, 1>(g, d_hdr, d_items, carry, carry_slots, s);
    case 1: return launch_batch_vk<float, 2>(g, d_hdr, d_items, carry, carry_slots, s);
    case 2: return launch_batch_vk<float, 4>(g, d_hdr, d_items, carry, carry_slots, s);
    case 3: return launch_batch_vk<float, 8>(g, d_hdr, d_items, carry, carry_slots, s);
    case 4: return launch_batch_vk<double, 1>(g, d_hdr, d_items, carry, carry_slots, s);
    case 5: return launch_batch_vk<double, 2>(g, d_hdr, d_items, carry, carry_slots, s);
    case 6: return launch_batch_vk<double, 4>(g, d_hdr, d_items, carry, carry_slots, s);
    case 7: return launch_batch_vk<double, 8>(g, d_hdr, d_items, carry, carry_slots, s);
    }
    return fail(SSPMV_INVALID_ARG, "batch group %d out of range", g);
}

}  // namespace sspmv

using namespace sspmv;

extern "C" sspmv_status sspmv_LeSpMV_csr(double alpha, const sspmv_csr *A, const void *x, double beta, void *y,
                                         sspmv_stream_t stream) {
    return spmm_csr_impl(alpha, A, 1, x, 1, beta, y, 1, stream);
}

extern "C" sspmv_status sspmv_spmm_csr(double alpha, const sspmv_csr *A, int32_t k, const void *X, int64_t ldx,
                                       double beta, void *Y, int64_t ldy, sspmv_stream_t stream) {
    return spmm_csr_impl(alpha, A, k, X, ldx, beta, Y, ldy, stream);
}

extern "C" double sspmv_algorithmic_bytes_csr(const sspmv_csr *A, int32_t k, int32_t beta_nonzero) {
    const double sv = (double)vsize(A->f.value_type);
    return (double)A->f.num_nnzs * (sv + 4.0) + (double)(A->f.num_rows + 1) * 4.0 +
           (double)k * (double)A->f.num_cols * sv + (double)k * (double)A->f.num_rows * sv * (beta_nonzero ? 2.0 : 1.0);
}

// ===================================================== allocation-free CSR ===
//
// sspmv_LeSpMV_csr_noalloc: the merge-path CSR SpMV (one right-hand side)
// with its scratch -- tile split points and per-tile carries -- in a fixed
// device array that every GPU loading this library holds until the process
// exits, so the call itself allocates nothing.
//
// Who needs it: code that cannot call cudaMalloc at SpMV time.  An iterative
// solver or serving loop whose device heap is carved up by its own pool
// allocator up front (a cudaMalloc there either fails or steals memory the
// pool has promised elsewhere); a latency-bound loop where the implicit device
// synchronisation of cudaMalloc/cudaFree is not acceptable; a component
// running under a strict device-memory budget enforced outside this library.
// The regular entry point builds a per-matrix plan on first use and keeps it
// in device memory it allocates; this one does not.
//
// Limits and rules:
//  - scratch is kNoAllocScratchBytes (16 MiB); a matrix needs
//    ceil((num_rows + num_nnzs) / 2048) tiles of kNoAllocTileBytes each, so
//    num_rows + num_nnzs may be at most kNoAllocMaxTiles * 2048 (about 238
//    million); larger matrices get SSPMV_INVALID_ARG.
//  - the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current; make that first call
//    before any stream capture.  The address is kept per device and per
//    context: after a cudaDeviceReset the next call looks it up again.
//  - every call writes all the scratch it later reads (split points, carries),
//    so nothing has to be cleared between calls; but all calls share the one
//    array: calls that overlap on the GPU (different streams, or a graph
//    replayed concurrently) race on it and must be serialised by the caller.
namespace {

constexpr size_t kNoAllocScratchBytes = 16u << 20;
constexpr int kNoAllocTile = MergeShape<1>::tile;  // 2048 merge items
// per tile: split point (int2) + carry_row + has_end + carry and head values
// (kMaxK slots of up to 8 bytes each, the layout csr_merge_kernel uses)
constexpr size_t kNoAllocTileBytes = sizeof(int2) + 4 + 4 + 2 * kMaxK * 8;
constexpr int64_t kNoAllocMaxTiles = (int64_t)((kNoAllocScratchBytes - 4 * 256 - sizeof(int2)) / kNoAllocTileBytes);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mutex;
void *g_noalloc_ptr[kNoAllocMaxDevices] = {nullptr};
unsigned long long g_noalloc_ctx[kNoAllocMaxDevices] = {0};

// Unique id of the calling thread's current CUDA context (0 if the driver
// cannot tell), through the driver entry points the runtime hands out, so
// no link against the driver library is needed.  A device reset
// (cudaDeviceReset) ends the primary context and the next call gets a new
// one with a new id: the array's address is then looked up again.
unsigned long long current_context_id() {
    using GetCurrent = CUresult (*)(CUcontext *);
    using GetId = CUresult (*)(CUcontext, unsigned long long *);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<GetCurrent>(f);
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetId>(f);
    });
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (get_current && get_id && get_current(&ctx) == CUDA_SUCCESS && ctx && get_id(ctx, &id) == CUDA_SUCCESS)
        return id;
    return 0;
}

// The scratch array's device address on the current device, looked up with
// cudaGetSymbolAddress the first time this device (context) is seen.
sspmv_status noalloc_scratch(void **out) {
    int dev = 0;
    SSPMV_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(SSPMV_NOT_SUPPORTED, "device ordinal %d too large", dev);
    SSPMV_CUDA_TRY(cudaSetDevice(dev));  // makes the device's primary context current (allocates nothing)
    const unsigned long long ctx = current_context_id();
    std::lock_guard<std::mutex> g(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev] || g_noalloc_ctx[dev] != ctx || ctx == 0) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(SSPMV_CUDA_ERROR, "cudaGetSymbolAddress(scratch) on device %d: %s", dev, cudaGetErrorString(e));
        g_noalloc_ptr[dev] = p;
        g_noalloc_ctx[dev] = ctx;
    }
    *out = g_noalloc_ptr[dev];
    return SSPMV_OK;
}

inline size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

}  // namespace

extern "C" sspmv_status sspmv_LeSpMV_csr_noalloc(double alpha, const sspmv_csr *A, const void *x, double beta,
                                                 void *y, sspmv_stream_t s) {
    if (!A) return fail(SSPMV_INVALID_ARG, "null matrix");
    SSPMV_TRY(check_spmm_args(&A->f, 1, x, 1, y, 1));
    const int64_t m = A->f.num_rows, nnz = A->f.num_nnzs;
    if (m == 0) return SSPMV_OK;
    const int64_t tiles = std::max<int64_t>((m + nnz + kNoAllocTile - 1) / kNoAllocTile, 1);
    if (tiles > kNoAllocMaxTiles)
        return fail(SSPMV_INVALID_ARG,
                    "sspmv_LeSpMV_csr_noalloc: num_rows + num_nnzs = %lld exceeds the fixed scratch limit of %lld "
                    "(%lld tiles of %d); use sspmv_LeSpMV_csr",
                    (long long)(m + nnz), (long long)(kNoAllocMaxTiles * kNoAllocTile), (long long)kNoAllocMaxTiles,
                    kNoAllocTile);
    void *base = nullptr;
    SSPMV_TRY(noalloc_scratch(&base));
    unsigned char *b = (unsigned char *)base;
    size_t off = 0;
    int2 *coords = (int2 *)(b + off);
    off = align256(off + (size_t)(tiles + 1) * sizeof(int2));
    int32_t *carry_row = (int32_t *)(b + off);
    off = align256(off + (size_t)tiles * 4);
    int32_t *has_end = (int32_t *)(b + off);
    off = align256(off + (size_t)tiles * 4);
    unsigned char *carry_val = b + off;
    off = align256(off + (size_t)tiles * kMaxK * 8);
    unsigned char *head_val = b + off;
    merge_path_search<<<grid_for(tiles + 1, 256), 256, 0, cu(s)>>>(tiles, kNoAllocTile, (int)m, (int)nnz,
                                                                    A->row_offset, coords);
    SSPMV_LAUNCH_CHECK();
    return dispatch_value(A->f.value_type, [&](auto tag) -> sspmv_status {
        using V = decltype(tag);
        const size_t smem = (size_t)kNoAllocTile * sizeof(V) + ((size_t)kNoAllocTile + 1) * 4;
        csr_merge_kernel<V, 1><<<(unsigned)tiles, kBlock, smem, cu(s)>>>(
            (int)m, A->row_offset, A->col_index, (const V *)A->values, (const V *)x, 1, (V)alpha, (V)beta, (V *)y, 1,
            coords, carry_row, has_end, (V *)carry_val, (V *)head_val);
        SSPMV_LAUNCH_CHECK();
        if (tiles > 1) {
            csr_merge_fixup<V, 1><<<grid_for(tiles, 256), 256, 0, cu(s)>>>(
                tiles, (int)m, A->row_offset, coords, carry_row, has_end, (const V *)carry_val, (const V *)head_val,
                (V)alpha, (V)beta, (V *)y, 1);
            SSPMV_LAUNCH_CHECK();
        }
        return SSPMV_OK;
    });
}

namespace sspmv {
sspmv_status dia_wait_timeouts(unsigned long long *out);
}

extern "C" sspmv_status sspmv_wait_timeouts(int64_t *count) {
    if (!count) return fail(SSPMV_INVALID_ARG, "null output");
    unsigned long long v = 0, w = 0;
    SSPMV_CUDA_TRY(cudaMemcpyFromSymbol(&v, g_csr_wait_timeouts, sizeof(v)));
    SSPMV_TRY(sspmv::dia_wait_timeouts(&w));
    *count = (int64_t)(v + w);
    return SSPMV_OK;
}
