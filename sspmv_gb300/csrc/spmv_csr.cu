// spmv_csr.cu -- CSR SpMV / SpMM on sm_103a.
//
// Replaces LeSpMV_csr (src/spmv_csr.cpp:165-185) and its three CPU kernels
// (serial, OpenMP per row, nnz-balanced row partition).
//
// Default kernel (kernel_flag 0 or 2): merge-path.  The (row end, nonzero)
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
#include "common.cuh"
#include "plan.cuh"
#include "spmv_common.cuh"
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
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
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
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= num_tiles) return;
    const int r = carry_row[t];
    if (r >= m) return;
    const int rs = row_offset[r];
    if (rs < coords[t].y || rs >= coords[t + 1].y) return;
    V tot[K];
#pragma unroll
    for (int q = 0; q < K; q++) tot[q] = carry_val[t * kMaxK + q];
    for (int64_t u = t + 1; u < num_tiles; u++) {
        if (has_end[u]) {
#pragma unroll
            for (int q = 0; q < K; q++) tot[q] += head_val[u * kMaxK + q];
            break;
        }
#pragma unroll
        for (int q = 0; q < K; q++) tot[q] += carry_val[u * kMaxK + q];
    }
    V *yp = y + (int64_t)r * ldy;
#pragma unroll
    for (int q = 0; q < K; q++) yp[q] = axpby(alpha, tot[q], beta, yp + q);
}

// ---------------------------------------------------- batched (serving) --
// Index of the item owning global tile gt: the last item whose tile_begin is
// <= gt (items of a group have increasing tile_begin).
__device__ __forceinline__ int batch_item_of(const BatchItem *__restrict__ items, int n, int64_t gt) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&items[mid].tile_begin) <= gt) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Persistent merge-path kernel over the tiles of every request of group g:
// CTA b takes global tiles b, b + gridDim.x, ...  The tile body is the one
// the single-matrix kernel runs, with the request's own split points, and
// the carries go to per-batch slots, so results match a lone sspmv_LeSpMV_csr
// / sspmv_spmm_csr call bit for bit.
template <typename V, int K>
__global__ void __launch_bounds__(kBlock) csr_batch_kernel(int g, const BatchHeader *__restrict__ hdr,
                                                           const BatchItem *__restrict__ all_items,
                                                           int32_t *__restrict__ carry_row,
                                                           int32_t *__restrict__ has_end, V *__restrict__ carry_val,
                                                           V *__restrict__ head_val) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = hdr->n_items[g];
    const int64_t total = hdr->total_tiles[g];
    const int64_t base = hdr->carry_base[g];
    const BatchItem *items = all_items + hdr->item_begin[g];
    for (int64_t gt = blockIdx.x; gt < total; gt += gridDim.x) {
        const BatchItem *q = items + batch_item_of(items, n, gt);
        const int64_t t = gt - q->tile_begin;
        const int2 *coords = q->coords;
        merge_tile<V, K>(q->m, q->row_offset, q->col_index, (const V *)q->values, (const V *)q->x, q->ldx,
                         (V)q->alpha, (V)q->beta, (V *)q->y, q->ldy, coords[t], coords[t + 1], base + gt,
                         carry_row, has_end, carry_val, head_val, smem_raw);
    }
}

// The batched counterpart of csr_merge_fixup: one thread per global tile.
template <typename V, int K>
__global__ void csr_batch_fixup(int g, const BatchHeader *__restrict__ hdr, const BatchItem *__restrict__ all_items,
                                const int32_t *__restrict__ carry_row, const int32_t *__restrict__ has_end,
                                const V *__restrict__ carry_val, const V *__restrict__ head_val) {
    const int n = hdr->n_items[g];
    const int64_t total = hdr->total_tiles[g];
    const int64_t base = hdr->carry_base[g];
    const BatchItem *items = all_items + hdr->item_begin[g];
    for (int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; gt < total;
         gt += (int64_t)gridDim.x * blockDim.x) {
        const BatchItem *q = items + batch_item_of(items, n, gt);
        const int64_t t = gt - q->tile_begin, nt = q->num_tiles;
        if (nt <= 1) continue;
        const int64_t slot = base + gt;
        const int r = carry_row[slot];
        if (r >= q->m) continue;
        const int rs = q->row_offset[r];
        if (rs < q->coords[t].y || rs >= q->coords[t + 1].y) continue;
        V tot[K];
#pragma unroll
        for (int c = 0; c < K; c++) tot[c] = carry_val[slot * kMaxK + c];
        for (int64_t u = t + 1; u < nt; u++) {
            const int64_t su = slot + (u - t);
            if (has_end[su]) {
#pragma unroll
                for (int c = 0; c < K; c++) tot[c] += head_val[su * kMaxK + c];
                break;
            }
#pragma unroll
            for (int c = 0; c < K; c++) tot[c] += carry_val[su * kMaxK + c];
        }
        V *yp = (V *)q->y + (int64_t)r * q->ldy;
        const V alpha = (V)q->alpha, beta = (V)q->beta;
#pragma unroll
        for (int c = 0; c < K; c++) yp[c] = axpby(alpha, tot[c], beta, yp + c);
    }
}

template <typename V, int K>
size_t merge_smem_bytes() {
    return (size_t)MergeShape<K>::tile * K * sizeof(V) + ((size_t)MergeShape<K>::tile + 1) * 4;
}

// Resident CTAs per SM of csr_batch_kernel<V, K> (sets its shared-memory
// attribute on first use).
template <typename V, int K>
int batch_blocks_per_sm() {
    static int blocks = 0;
    if (blocks == 0) {
        const size_t smem = merge_smem_bytes<V, K>();
        cudaFuncSetAttribute(csr_batch_kernel<V, K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, csr_batch_kernel<V, K>, kBlock, smem) != cudaSuccess ||
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
    csr_batch_kernel<V, K><<<grid, kBlock, merge_smem_bytes<V, K>(), cu(s)>>>(g, hdr, items, carry_row, has_end,
                                                                              carry_val, head_val);
    SSPMV_LAUNCH_CHECK();
    csr_batch_fixup<V, K><<<(unsigned)num_sms() * 2, 256, 0, cu(s)>>>(g, hdr, items, carry_row, has_end, carry_val,
                                                                        head_val);
    SSPMV_LAUNCH_CHECK();
    return SSPMV_OK;
}

template <typename V, int K, int VS>
__global__ void __launch_bounds__(kBlock) csr_vector_kernel(
    int m, const int32_t *__restrict__ row_offset, const int32_t *__restrict__ col_index,
    const V *__restrict__ values, const V *__restrict__ x, int64_t ldx, V alpha, V beta,
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
        if (row < m) {
            const int rs = ld_stream(row_offset + row), re = ld_stream(row_offset + row + 1);
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
                for (int u = 0; u < 4; u++)
#pragma unroll
                    for (int r = 0; r < K; r++) s[r] += a[u] * ld_x(x + (int64_t)c[u] * ldx + r);
            }
            for (; j < re; j += VS) {
                const int c = ld_stream(col_index + j);
                const V a = ld_stream(values + j);
#pragma unroll
                for (int r = 0; r < K; r++) s[r] += a * ld_x(x + (int64_t)c * ldx + r);
            }
        }
#pragma unroll
        for (int r = 0; r < K; r++) s[r] = warp_sum(s[r], VS);
        if (row < m && sub == 0) {
            V *yp = y + row * ldy;
#pragma unroll
            for (int r = 0; r < K; r++) yp[r] = axpby(alpha, s[r], beta, yp + r);
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
    static bool attr_set = false;
    if (!attr_set) {
        SSPMV_CUDA_TRY(cudaFuncSetAttribute(csr_merge_kernel<V, K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)smem));
        attr_set = true;
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
    csr_vector_kernel<V, K, VS><<<grid, kBlock, 0, cu(s)>>>((int)m, A->row_offset, A->col_index,
                                                            (const V *)A->values, x, ldx, alpha, beta, y, ldy);
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
    case 2: return launch_vector_vs<V, K, 2>(A, alpha, x, ldx, beta, y, ldy, s);
    case 4: return launch_vector_vs<V, K, 4>(A, alpha, x, ldx, beta, y, ldy, s);
    case 8: return launch_vector_vs<V, K, 8>(A, alpha, x, ldx, beta, y, ldy, s);
    case 16: return launch_vector_vs<V, K, 16>(A, alpha, x, ldx, beta, y, ldy, s);
    default: return launch_vector_vs<V, K, 32>(A, alpha, x, ldx, beta, y, ldy, s);
    }
}

template <typename V, int K>
sspmv_status csr_pass(const sspmv_csr *A, Plan *p, V alpha, const V *x, int64_t ldx, V beta, V *y,
                      int64_t ldy, sspmv_stream_t s) {
    if (A->f.kernel_flag == 1) return launch_vector<V, K>(A, p, alpha, x, ldx, beta, y, ldy, s);
    return launch_merge<V, K>(A, p, alpha, x, ldx, beta, y, ldy, s);
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
    std::lock_guard<std::mutex> g(plan_mutex());
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

int csr_merge_tile_items(int32_t k) { return k > 4 ? MergeShape<8>::tile : MergeShape<1>::tile; }

sspmv_status csr_merge_coords(const sspmv_csr *A, int32_t k, const int2 **coords, int64_t *num_tiles,
                              sspmv_stream_t s) {
    Plan *p = get_plan(&A->f);
    if (!p) return fail(SSPMV_OUT_OF_MEMORY, "plan allocation failed");
    const int which = k > 4 ? 1 : 0;
    SSPMV_TRY(ensure_merge_plan(p, which, A->f.num_rows, A->f.num_nnzs, A->row_offset, A->f.value_type, s));
    *coords = p->merge[which].coords;
    *num_tiles = p->merge[which].num_tiles;
    return SSPMV_OK;
}

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
//    before any stream capture.
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

sspmv_status noalloc_scratch(void **out) {
    int dev = 0;
    SSPMV_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(SSPMV_NOT_SUPPORTED, "device ordinal %d too large", dev);
    std::lock_guard<std::mutex> g(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(SSPMV_CUDA_ERROR, "cudaGetSymbolAddress(scratch) on device %d: %s", dev, cudaGetErrorString(e));
        g_noalloc_ptr[dev] = p;
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
