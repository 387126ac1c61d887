// dia.cu -- DIA format on sm_103a: GPU converter, SpMV / SpMM, export.
//
// Converter (csr_to_dia, include/sparse_conversion.h:612-766): diagonals are
// numbered in the order a row-major scan first meets them.  On the GPU every
// diagonal records the smallest CSR position holding it (atomicMin), the
// occupied diagonals are sorted by that position, and the rank is the
// diagonal's number -- the same order as the sequential scan.  Values are then
// written row by row in CSR order, so a duplicated (row, col) keeps its last
// value as in the reference.  More than max_diags diagonals: SSPMV_INFEASIBLE
// (the reference exits).  stride = num_rows rounded up to `alignment`.
//
// SpMV (LeSpMV_dia, src/spmv_dia.cpp:177-197): one thread per row walks the
// diagonals: data[d*stride + i] and x[i + offset_d] are both contiguous
// across a warp, and x is reused from L1/L2 across diagonals.  No atomics
// (the reference scatters into y with atomics, one OpenMP task per diagonal).
// Column bound is num_cols (the reference uses num_rows, wrong when not square).
#include <algorithm>
#include <mutex>
#include <vector>

#include "bulk.cuh"
#include "common.cuh"
#include "plan.cuh"
#include "primitives.cuh"
#include "spmv_common.cuh"

namespace sspmv {
sspmv_status check_dims(int32_t vt, int64_t m, int64_t n, int64_t nnz);
void init_features(sspmv_features *f, int32_t vt, int64_t m, int64_t n, int64_t nnz, int32_t owns);
}  // namespace sspmv

using namespace sspmv;

namespace {

constexpr int kBlock = 256;

__global__ void fill_i32(int64_t n, int32_t v, int32_t *__restrict__ p) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

// first[d] = smallest CSR position on diagonal d (the reference's
// first-encounter order).  Where the 32 rows of a warp start on a few common
// diagonals (banded matrices), the warp walks them in step (k-th nonzero of
// each row together), groups the lanes on the same diagonal and lets only the
// lowest one -- the smallest row, so the smallest position -- issue the
// atomicMin: one atomic per diagonal per warp instead of one per nonzero to
// the same few addresses.  Other warps (scattered diagonals, where lockstep
// would only add work) walk their rows one thread per row.
__global__ void dia_first_pos(int64_t m, const int32_t *__restrict__ rp, const int32_t *__restrict__ ci,
                              int32_t *__restrict__ first) {
    constexpr unsigned kFull = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + threadIdx.x - lane; base < m;
         base += (int64_t)gridDim.x * blockDim.x) {  // warp-uniform
        const int64_t i = base + lane;
        int32_t j0 = 0, len = 0;
        if (i < m) {
            j0 = rp[i];
            len = rp[i + 1] - j0;
        }
        const bool act0 = len > 0;
        const unsigned on0 = __ballot_sync(kFull, act0);
        bool leader0 = false;
        if (act0) {
            const unsigned grp = __match_any_sync(on0, (unsigned long long)(m - i + ci[j0]));
            leader0 = lane == __ffs(grp) - 1;
        }
        if (__popc(__ballot_sync(kFull, leader0)) > 4) {  // scattered: a thread per row
            for (int32_t jj = j0; jj < j0 + len; jj++) atomicMin(&first[m - i + ci[jj]], jj);
            continue;
        }
        const int32_t most = __reduce_max_sync(kFull, (unsigned)len);
        for (int32_t k = 0; k < most; k++) {
            const bool act = k < len;
            const unsigned on = __ballot_sync(kFull, act);
            if (act) {
                const int32_t jj = j0 + k;
                const unsigned long long key = (unsigned long long)(m - i + ci[jj]);
                const unsigned grp = __match_any_sync(on, key);
                if (lane == __ffs(grp) - 1) atomicMin(&first[key], jj);
            }
        }
    }
}

__global__ void dia_collect(int64_t len, const int32_t *__restrict__ first, int32_t cap,
                            unsigned long long *__restrict__ count, uint64_t *__restrict__ keys,
                            uint32_t *__restrict__ vals) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < len; t += (int64_t)gridDim.x * blockDim.x) {
        const int32_t f = first[t];
        if (f != 0x7fffffff) {
            unsigned long long k = atomicAdd(count, 1ull);
            if (k < (unsigned long long)cap) {
                keys[k] = (uint64_t)f;
                vals[k] = (uint32_t)t;
            }
        }
    }
}

__global__ void dia_rank(int32_t nd, int64_t m, const uint32_t *__restrict__ vals, int32_t *__restrict__ dmap,
                         int64_t *__restrict__ offsets) {
    int32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < nd) {
        dmap[vals[r]] = r;
        offsets[r] = (int64_t)vals[r] - m;
    }
}

template <typename V>
__global__ void dia_fill(int64_t m, int64_t stride, const int32_t *__restrict__ rp, const int32_t *__restrict__ ci,
                         const V *__restrict__ cv, const int32_t *__restrict__ dmap, V *__restrict__ data) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        for (int32_t jj = rp[i]; jj < rp[i + 1]; jj++) data[(int64_t)dmap[m - i + ci[jj]] * stride + i] = cv[jj];
}

template <typename V, int K, bool PLAIN = false>
__global__ void __launch_bounds__(kBlock) dia_spmv_kernel(int m, int n, int nd, int64_t stride,
                                                        const int64_t *__restrict__ offsets,
                                                        const V *__restrict__ data, const V *__restrict__ x,
                                                        int64_t ldx, int xvec, V alpha, V beta, V *__restrict__ y,
                                                        int64_t ldy) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        V s[K];
#pragma unroll
        for (int q = 0; q < K; q++) s[q] = V(0);
        int d = 0;
        for (; d + 4 <= nd; d += 4) {
            int64_t j[4];
            V a[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                // data[d][i] exists for every row i < m (stride >= m): the load
                // does not wait for the offset that decides whether it is used
                j[u] = i + __ldg(offsets + d + u);
                a[u] = ld_stream(data + (int64_t)(d + u) * stride + i);
            }
#pragma unroll
            for (int u = 0; u < 4; u++)
                if (j[u] >= 0 && j[u] < n) {
                    V xr[K];
                    ld_xrow<V, K>(x, j[u], ldx, xvec != 0, xr);
#pragma unroll
                    for (int q = 0; q < K; q++) s[q] += a[u] * xr[q];
                }
        }
        for (; d < nd; d++) {
            const int64_t j = i + __ldg(offsets + d);
            if (j >= 0 && j < n) {
                const V a = ld_stream(data + (int64_t)d * stride + i);
                V xr[K];
                ld_xrow<V, K>(x, j, ldx, xvec != 0, xr);
#pragma unroll
                for (int q = 0; q < K; q++) s[q] += a * xr[q];
            }
        }
        V *yp = y + i * ldy;
#pragma unroll
        for (int q = 0; q < K; q++) yp[q] = row_out(PLAIN, alpha, s[q], beta, yp + q);
    }
}

// ------------------------------------------------------------ x staging --
// kernel_flag 1 (k = 1, at most kDiaStageMax diagonals): rows in tiles of
// kBlock, CTA g taking tiles g, g + G, ... of a persistent grid.  For a tile,
// thread 0 streams into one of two shared-memory stages, with bulk copies
// (cp.async.bulk) completed on the stage's mbarrier: each diagonal's values of
// the tile's rows, and each diagonal's x window x[r0 + offset_d, ... + tile)
// (rounded out to 16 bytes, cut at the ends of x).  A tile ahead of the
// threads; the threads then read values and x from shared memory only (an
// element outside the staged ranges -- the array's ragged end -- comes from
// global memory), one FMA per stored element in diagonal order, as the
// thread-per-row kernel.  Waits are bounded (kMaxPolls); a wait that gives up
// is counted (sspmv_wait_timeouts) and the CTA leaves after its other copies.
constexpr int kDiaStageMax = 16;
constexpr int kDiaStages = 2;

__device__ unsigned long long g_dia_wait_timeouts = 0;

template <typename V>
struct DiaStage {
    static constexpr int kPerV = 16 / (int)sizeof(V);
    static constexpr int kWin = kBlock + 2 * kPerV;          // x window capacity (elements)
    static constexpr size_t kDataBytes = (size_t)kBlock * sizeof(V);
    static constexpr size_t kWinBytes = (size_t)kWin * sizeof(V);
    static size_t bytes(int nd) { return (size_t)nd * (kDataBytes + kWinBytes) + 16 + 2 * kDiaStageMax * 4 + 16; }
};

template <typename V, bool PLAIN>
__global__ void __launch_bounds__(kBlock) dia_staged_kernel(int m, int n, int nd, int64_t stride,
                                                          const int64_t *__restrict__ offsets,
                                                          const V *__restrict__ data, const V *__restrict__ x,
                                                          V alpha, V beta, V *__restrict__ y, size_t stage_bytes) {
    using St = DiaStage<V>;
    constexpr int kPerV = St::kPerV;
    extern __shared__ __align__(16) unsigned char dia_smem[];
    __shared__ int64_t soff[kDiaStageMax];
    uint64_t *bars = reinterpret_cast<uint64_t *>(dia_smem + kDiaStages * stage_bytes);
    auto sdata = [&](int st, int d) {
        return reinterpret_cast<V *>(dia_smem + st * stage_bytes + (size_t)d * St::kDataBytes);
    };
    auto swin = [&](int st, int d) {
        return reinterpret_cast<V *>(dia_smem + st * stage_bytes + (size_t)nd * St::kDataBytes +
                                     (size_t)d * St::kWinBytes);
    };
    // header: [0] r0, [1] rows, [2] rows staged; then a[nd], b[nd] window bounds
    auto shdr = [&](int st) {
        return reinterpret_cast<int32_t *>(dia_smem + st * stage_bytes + (size_t)nd * (St::kDataBytes + St::kWinBytes));
    };
    const int t = threadIdx.x;
    const int64_t G = gridDim.x, g = blockIdx.x;
    const int64_t tiles = ((int64_t)m + kBlock - 1) / kBlock;
    if (t < nd) soff[t] = offsets[t];
    if (t == 0) {
        for (int st = 0; st < kDiaStages; st++) mbar_init(&bars[st], 1);
        fence_mbar_init();
    }
    __syncthreads();

    auto issue = [&](int64_t k) {  // thread 0: tile g + k G into stage k % kDiaStages
        const int64_t tile = g + k * G;
        if (tile >= tiles) return;
        const int st = (int)(k % kDiaStages);
        const int64_t r0 = tile * kBlock;
        const int rows = (int)min((int64_t)kBlock, (int64_t)m - r0);
        const int staged = rows / kPerV * kPerV;  // values copied: whole 16-byte words of the tile
        int32_t *h = shdr(st);
        h[0] = (int)r0;
        h[1] = rows;
        h[2] = staged;
        uint32_t tx = (uint32_t)((size_t)nd * staged * sizeof(V));
        const int64_t nfloor = (int64_t)n / kPerV * kPerV;
        for (int d = 0; d < nd; d++) {
            const int64_t lo = max(r0 + soff[d], (int64_t)0), hi = min(r0 + soff[d] + rows, (int64_t)n);
            int64_t a = 0, b = 0;
            if (hi > lo) {
                a = lo / kPerV * kPerV;
                b = min((hi + kPerV - 1) / kPerV * kPerV, nfloor);
                if (b < a) b = a;
            }
            h[3 + d] = (int)a;
            h[3 + kDiaStageMax + d] = (int)b;
            tx += (uint32_t)((b - a) * (int64_t)sizeof(V));
        }
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&bars[st], tx);
        for (int d = 0; d < nd; d++) {
            if (staged > 0)
                bulk_g2s(sdata(st, d), data + (int64_t)d * stride + r0, (uint32_t)(staged * sizeof(V)), &bars[st]);
            const int a = h[3 + d], b = h[3 + kDiaStageMax + d];
            if (b > a) bulk_g2s(swin(st, d), x + a, (uint32_t)((int64_t)(b - a) * sizeof(V)), &bars[st]);
        }
    };

    if (t == 0)
        for (int k = 0; k < kDiaStages; k++) issue(k);
    for (int64_t k = 0;; k++) {
        const int64_t tile = g + k * G;
        if (tile >= tiles) break;
        const int st = (int)(k % kDiaStages);
        const uint32_t parity = (uint32_t)((k / kDiaStages) & 1);
        const bool ok = __syncthreads_and(t == 0 ? mbar_wait(&bars[st], parity) : true);
        if (!ok) {
            if (t == 0) {
                atomicAdd(&g_dia_wait_timeouts, 1ull);
                for (int64_t k2 = k + 1; k2 < k + kDiaStages && g + k2 * G < tiles; k2++)
                    mbar_wait(&bars[k2 % kDiaStages], (uint32_t)((k2 / kDiaStages) & 1));
            }
            return;
        }
        if (t != 0) mbar_try_wait(&bars[st], parity);  // acquire the completed phase
        const int32_t *h = shdr(st);
        const int r0 = h[0], rows = h[1], staged = h[2];
        if (t < rows) {
            const int64_t i = (int64_t)r0 + t;
            V sum = V(0);
            for (int d = 0; d < nd; d++) {
                const int64_t j = i + soff[d];
                if (j >= 0 && j < n) {
                    const V av = t < staged ? sdata(st, d)[t] : ld_stream(data + (int64_t)d * stride + i);
                    const int a = h[3 + d], b = h[3 + kDiaStageMax + d];
                    const V xv = (j >= a && j < b) ? swin(st, d)[j - a] : ld_x(x + j);
                    sum += av * xv;
                }
            }
            y[i] = row_out(PLAIN, alpha, sum, beta, y + i);
        }
        __syncthreads();  // stage st free
        if (t == 0) issue(k + kDiaStages);
    }
}

// One instantiation per kernel: the shared-memory attribute and the
// occupancy are the kernel's own.
template <typename V, bool PLAIN>
sspmv_status launch_dia_staged(const sspmv_dia *A, V alpha, const V *x, V beta, V *y, size_t stage, size_t smem,
                               sspmv_stream_t s) {
    auto kernel = dia_staged_kernel<V, PLAIN>;
    const int nd = A->complete_ndiags;
    static std::mutex mu;
    static size_t allowed = 0;                  // dynamic shared memory the kernel may use so far
    static int per_sm[kDiaStageMax + 1] = {0};  // resident CTAs per SM, by diagonal count
    {
        std::lock_guard<std::mutex> g(mu);
        if (smem > allowed) {
            SSPMV_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            allowed = smem;
        }
        if (per_sm[nd] == 0) {
            int c = 0;
            SSPMV_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, kernel, kBlock, smem));
            per_sm[nd] = c > 0 ? c : 1;
        }
    }
    const int64_t tiles = (A->f.num_rows + kBlock - 1) / kBlock;
    const int64_t grid = std::min<int64_t>(tiles, (int64_t)num_sms() * per_sm[nd]);
    kernel<<<(unsigned)grid, kBlock, smem, cu(s)>>>((int)A->f.num_rows, (int)A->f.num_cols, nd, A->stride,
                                                    A->diag_offsets, (const V *)A->diag_data, x, alpha, beta, y,
                                                    stage);
    SSPMV_LAUNCH_CHECK();
    return SSPMV_OK;
}

// The staged kernel, or false when it does not apply (k > 1, too many
// diagonals, arrays not 16-byte aligned, x rows not contiguous).
template <typename V>
bool try_dia_staged(const sspmv_dia *A, V alpha, const V *x, int64_t ldx, V beta, V *y, int64_t ldy,
                    sspmv_stream_t s, sspmv_status *st) {
    const int nd = A->complete_ndiags;
    if (A->f.kernel_flag != 1 || nd < 1 || nd > kDiaStageMax || ldx != 1 || ldy != 1) return false;
    if (((reinterpret_cast<uintptr_t>(A->diag_data) | reinterpret_cast<uintptr_t>(x)) & 15) != 0) return false;
    if (((int64_t)A->stride * (int64_t)sizeof(V)) % 16 != 0) return false;
    const size_t stage = DiaStage<V>::bytes(nd);
    const size_t smem = kDiaStages * stage + kDiaStages * sizeof(uint64_t);
    if (alpha == V(1) && beta == V(0)) *st = launch_dia_staged<V, true>(A, alpha, x, beta, y, stage, smem, s);
    else *st = launch_dia_staged<V, false>(A, alpha, x, beta, y, stage, smem, s);
    return true;
}

template <typename V, int K>
sspmv_status launch_dia(const sspmv_dia *A, V alpha, const V *x, int64_t ldx, V beta, V *y, int64_t ldy,
                        sspmv_stream_t s) {
    if constexpr (K == 1) {
        sspmv_status st = SSPMV_OK;
        if (try_dia_staged<V>(A, alpha, x, ldx, beta, y, ldy, s, &st)) return st;
    }
    const unsigned grid = grid_for(A->f.num_rows, kBlock, (int64_t)num_sms() * 16);
    auto go = [&](auto kernel) {
        kernel<<<grid, kBlock, 0, cu(s)>>>((int)A->f.num_rows, (int)A->f.num_cols, A->complete_ndiags, A->stride,
                                           A->diag_offsets, (const V *)A->diag_data, x, ldx,
                                           xrow_vec(x, ldx, sizeof(V), K), alpha, beta, y, ldy);
    };
    if (K == 1 && alpha == V(1) && beta == V(0)) go(dia_spmv_kernel<V, K, K == 1>);  // y = sum
    else go(dia_spmv_kernel<V, K>);
    SSPMV_LAUNCH_CHECK();
    return SSPMV_OK;
}

}  // namespace

extern "C" sspmv_status sspmv_csr_to_dia(const sspmv_csr *csr, int32_t max_diags, int32_t align, sspmv_dia *out,
                                         sspmv_stream_t s) {
    if (!csr || !out) return fail(SSPMV_INVALID_ARG, "null argument");
    SSPMV_TRY(check_dims(csr->f.value_type, csr->f.num_rows, csr->f.num_cols, csr->f.num_nnzs));
    if (max_diags == 0) max_diags = 10240;
    if (align == 0) align = default_alignment(csr->f.value_type);
    if (max_diags < 0 || align < 1) return fail(SSPMV_INVALID_ARG, "max_diags >= 0 and alignment >= 1 required");
    const int64_t m = csr->f.num_rows, n = csr->f.num_cols, len = m + n;
    const int32_t vt = csr->f.value_type;
    int32_t *first = nullptr, *dmap = nullptr;
    uint64_t *keys = nullptr;
    uint32_t *vals = nullptr;
    unsigned long long *d_count = nullptr;
    sspmv_dia A;
    init_features(&A.f, vt, m, n, csr->f.num_nnzs, 1);
    A.diag_offsets = nullptr;
    A.diag_data = nullptr;
    auto cleanup = [&]() {
        dfree(first, s);
        dfree(dmap, s);
        dfree(keys, s);
        dfree(vals, s);
        dfree(d_count, s);
    };
    const unsigned g = grid_for(std::max<int64_t>(m, 1), 256, (int64_t)num_sms() * 16);
    const unsigned gl = grid_for(std::max<int64_t>(len, 1), 256, (int64_t)num_sms() * 16);
    sspmv_status st = dalloc(&first, (size_t)len, s);
    if (st == SSPMV_OK) st = dalloc(&keys, (size_t)max_diags + 1, s);
    if (st == SSPMV_OK) st = dalloc(&vals, (size_t)max_diags + 1, s);
    if (st == SSPMV_OK) st = dalloc(&d_count, 1, s);
    unsigned long long count = 0;
    if (st == SSPMV_OK && len > 0) {
        fill_i32<<<gl, 256, 0, cu(s)>>>(len, 0x7fffffff, first);
        note_launch();
        cudaMemsetAsync(d_count, 0, 8, cu(s));
        if (m > 0) {
            dia_first_pos<<<g, 256, 0, cu(s)>>>(m, csr->row_offset, csr->col_index, first);
            note_launch();
        }
        dia_collect<<<gl, 256, 0, cu(s)>>>(len, first, max_diags + 1, d_count, keys, vals);
        note_launch();
        cudaError_t e = cudaMemcpyAsync(&count, d_count, 8, cudaMemcpyDeviceToHost, cu(s));
        if (e == cudaSuccess) e = cudaStreamSynchronize(cu(s));
        if (e != cudaSuccess) st = fail(SSPMV_CUDA_ERROR, "csr_to_dia: %s", cudaGetErrorString(e));
    }
    if (st == SSPMV_OK && count > (unsigned long long)max_diags)
        st = fail(SSPMV_INFEASIBLE, "number of diagonals (%llu) exceeds limit (%d)", count, max_diags);
    const int32_t nd = (int32_t)count;
    const int64_t stride = (int64_t)align * ((m + align - 1) / align);
    if (st == SSPMV_OK) st = radix_sort_pairs(keys, vals, nd, bits_for((uint64_t)std::max<int64_t>(csr->f.num_nnzs, 1)), s);
    if (st == SSPMV_OK) st = dalloc(&dmap, (size_t)len, s);
    if (st == SSPMV_OK) st = dalloc(&A.diag_offsets, (size_t)nd, s);
    if (st == SSPMV_OK) st = dalloc((unsigned char **)&A.diag_data, (size_t)nd * stride * vsize(vt), s);
    if (st == SSPMV_OK) {
        cudaMemsetAsync(A.diag_data, 0, (size_t)nd * stride * vsize(vt), cu(s));
        if (nd > 0) {
            dia_rank<<<grid_for(nd, 256), 256, 0, cu(s)>>>(nd, m, vals, dmap, A.diag_offsets);
            note_launch();
        }
        if (m > 0) {
            st = dispatch_value(vt, [&](auto tag) -> sspmv_status {
                using V = decltype(tag);
                dia_fill<V><<<g, 256, 0, cu(s)>>>(m, stride, csr->row_offset, csr->col_index, (const V *)csr->values,
                                                  dmap, (V *)A.diag_data);
                SSPMV_LAUNCH_CHECK();
                return SSPMV_OK;
            });
        }
        cudaError_t e = cudaStreamSynchronize(cu(s));
        if (st == SSPMV_OK && e != cudaSuccess) st = fail(SSPMV_CUDA_ERROR, "csr_to_dia: %s", cudaGetErrorString(e));
    }
    cleanup();
    if (st != SSPMV_OK) {
        dfree(A.diag_offsets, s);
        dfree(A.diag_data, s);
        return st;
    }
    A.stride = (int32_t)stride;
    A.complete_ndiags = nd;
    *out = A;
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_spmm_dia(double alpha, const sspmv_dia *A, int32_t k, const void *X, int64_t ldx,
                                       double beta, void *Y, int64_t ldy, sspmv_stream_t s) {
    if (!A) return fail(SSPMV_INVALID_ARG, "null matrix");
    SSPMV_TRY(check_spmm_args(&A->f, k, X, ldx, Y, ldy));
    if (A->f.num_rows == 0) return SSPMV_OK;
    return dispatch_value(A->f.value_type, [&](auto tag) -> sspmv_status {
        using V = decltype(tag);
        return for_rhs_chunks<V>(k, (const V *)X, (V *)Y, [&](int32_t step, const V *xs, V *ys) {
            const V a = (V)alpha, b = (V)beta;
            switch (step) {
            case 8: return launch_dia<V, 8>(A, a, xs, ldx, b, ys, ldy, s);
            case 4: return launch_dia<V, 4>(A, a, xs, ldx, b, ys, ldy, s);
            case 2: return launch_dia<V, 2>(A, a, xs, ldx, b, ys, ldy, s);
            default: return launch_dia<V, 1>(A, a, xs, ldx, b, ys, ldy, s);
            }
        });
    });
}

extern "C" sspmv_status sspmv_LeSpMV_dia(double alpha, const sspmv_dia *A, const void *x, double beta, void *y,
                                         sspmv_stream_t s) {
    return sspmv_spmm_dia(alpha, A, 1, x, 1, beta, y, 1, s);
}

namespace sspmv {
// Bounded waits of the staged DIA kernel that gave up (sspmv_wait_timeouts).
sspmv_status dia_wait_timeouts(unsigned long long *out) {
    SSPMV_CUDA_TRY(cudaMemcpyFromSymbol(out, g_dia_wait_timeouts, sizeof(*out)));
    return SSPMV_OK;
}
}  // namespace sspmv

extern "C" sspmv_status sspmv_dia_export(const sspmv_dia *A, int64_t *diag_offsets, void *diag_data,
                                         sspmv_stream_t s) {
    if (!A) return fail(SSPMV_INVALID_ARG, "null matrix");
    const size_t nd = (size_t)A->complete_ndiags;
    if (diag_offsets && nd)
        SSPMV_CUDA_TRY(cudaMemcpyAsync(diag_offsets, A->diag_offsets, nd * 8, cudaMemcpyDeviceToHost, cu(s)));
    if (diag_data && nd)
        SSPMV_CUDA_TRY(cudaMemcpyAsync(diag_data, A->diag_data, nd * (size_t)A->stride * vsize(A->f.value_type),
                                       cudaMemcpyDeviceToHost, cu(s)));
    SSPMV_CUDA_TRY(cudaStreamSynchronize(cu(s)));
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_delete_dia(sspmv_dia *A) {
    if (!A) return SSPMV_OK;
    delete_barrier();
    free_plan(&A->f, nullptr);
    if (A->f.owns) {
        dfree(A->diag_offsets, nullptr);
        dfree(A->diag_data, nullptr);
    }
    A->diag_offsets = nullptr;
    A->diag_data = nullptr;
    return SSPMV_OK;
}

extern "C" double sspmv_algorithmic_bytes_dia(const sspmv_dia *A, int32_t k, int32_t beta_nonzero) {
    const double sv = (double)vsize(A->f.value_type);
    return (double)A->f.num_nnzs * sv + (double)A->complete_ndiags * 8.0 + (double)k * (double)A->f.num_cols * sv +
           (double)k * (double)A->f.num_rows * sv * (beta_nonzero ? 2.0 : 1.0);
}
