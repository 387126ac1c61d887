// coo.cu -- COO format on sm_103a: CSR<->COO converters, SpMV / SpMM, export.
//
// csr_to_coo (include/sparse_conversion.h:145-168): row-sorted triplets.
// coo_to_csr (:30-91): stable counting sort by row (duplicates kept, order
// within a row = triplet order) -- a stable radix sort of (row, position).
//
// SpMV (LeSpMV_coo, src/spmv_coo.cpp:161-182).  The reference scales y by
// beta, then scatters alpha*a*x with OpenMP atomics (and skips the scaling
// when beta == 0, leaving stale y).  Here, for row-sorted COO, each warp takes
// 256 consecutive nonzeros and reduces runs of equal rows with a segmented
// shuffle scan (kernel_flag 0, default); kernel_flag 1 uses CTA tiles of 2048
// nonzeros staged in shared memory with a block-wide segmented scan.  Rows
// that cross chunk boundaries are finished by a second kernel in a fixed
// order, and rows with no nonzeros (listed once, when the plan is built) get
// y = beta*y.  No atomics: results are deterministic.  Unsorted COO
// (row_sorted == 0) uses a scale pass plus an atomic scatter, like the
// reference.
#include <algorithm>
#include <atomic>

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

template <int K>
struct CooShape {
    static constexpr int items = K <= 4 ? 8 : 4;
    static constexpr int tile = kBlock * items;
};

__global__ void expand_rows(int64_t m, const int32_t *__restrict__ rp, int32_t *__restrict__ ri) {
    // one warp per row
    const int lane = threadIdx.x & 31;
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < m;
         i += ((int64_t)gridDim.x * blockDim.x) >> 5)
        for (int32_t j = rp[i] + lane; j < rp[i + 1]; j += 32) ri[j] = (int32_t)i;
}

__global__ void coo_keys(int64_t nnz, const int32_t *__restrict__ ri, uint64_t *__restrict__ keys,
                         uint32_t *__restrict__ vals) {
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nnz; j += (int64_t)gridDim.x * blockDim.x) {
        keys[j] = (uint64_t)(uint32_t)ri[j];
        vals[j] = (uint32_t)j;
    }
}

template <typename V>
__global__ void coo_gather(int64_t nnz, const uint32_t *__restrict__ perm, const int32_t *__restrict__ ci,
                           const V *__restrict__ cv, int32_t *__restrict__ col, V *__restrict__ val) {
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nnz; j += (int64_t)gridDim.x * blockDim.x) {
        col[j] = ci[perm[j]];
        val[j] = cv[perm[j]];
    }
}

// row_offset[i] = first sorted position whose row >= i
__global__ void rows_to_offsets(int64_t m, int64_t nnz, const uint64_t *__restrict__ rows, int32_t *__restrict__ rp) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= m; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t lo = 0, hi = nnz;
        while (lo < hi) {
            int64_t mid = (lo + hi) >> 1;
            if (rows[mid] < (uint64_t)i) lo = mid + 1;
            else hi = mid;
        }
        rp[i] = (int32_t)lo;
    }
}

__global__ void mark_present(int64_t nnz, const int32_t *__restrict__ ri, int32_t *__restrict__ present) {
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nnz; j += (int64_t)gridDim.x * blockDim.x)
        present[ri[j]] = 1;
}

__global__ void absent_flags(int64_t m, int32_t *__restrict__ flag) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        flag[i] = flag[i] ? 0 : 1;
}

__global__ void absent_scatter(int64_t m, const int32_t *__restrict__ flag, const int32_t *__restrict__ pos,
                               int32_t *__restrict__ list) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        if (flag[i]) list[pos[i]] = (int32_t)i;
}

template <typename V, int K>
__global__ void scale_rows(int64_t cnt, const int32_t *__restrict__ list, V beta, V *__restrict__ y, int64_t ldy) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < cnt; t += (int64_t)gridDim.x * blockDim.x) {
        V *yp = y + (int64_t)(list ? list[t] : t) * ldy;
#pragma unroll
        for (int q = 0; q < K; q++) yp[q] = beta == V(0) ? V(0) : beta * yp[q];
    }
}

template <typename V, int K>
__global__ void coo_atomic(int64_t nnz, const int32_t *__restrict__ ri, const int32_t *__restrict__ ci,
                           const V *__restrict__ cv, V alpha, const V *__restrict__ x, int64_t ldx, V *__restrict__ y,
                           int64_t ldy) {
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nnz; j += (int64_t)gridDim.x * blockDim.x) {
        const V a = alpha * cv[j];
#pragma unroll
        for (int q = 0; q < K; q++) atomicAdd(y + (int64_t)ri[j] * ldy + q, a * x[(int64_t)ci[j] * ldx + q]);
    }
}

// Tile t covers nonzeros [t*tile, min((t+1)*tile, nnz)).
template <typename V, int K>
__global__ void __launch_bounds__(kBlock) coo_tile_kernel(
    int64_t nnz, const int32_t *__restrict__ ri, const int32_t *__restrict__ ci, const V *__restrict__ cv,
    const V *__restrict__ x, int64_t ldx, V alpha, V beta, V *__restrict__ y, int64_t ldy,
    int32_t *__restrict__ carry_row, int32_t *__restrict__ has_end, V *__restrict__ carry_val,
    V *__restrict__ head_val) {
    constexpr int kItems = CooShape<K>::items;
    constexpr int kTile = CooShape<K>::tile;
    constexpr int kWarps = kBlock / 32;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    V *s_prod = reinterpret_cast<V *>(smem_raw);
    int *s_row = reinterpret_cast<int *>(s_prod + kTile * K);
    __shared__ int s_wkey[kWarps];
    __shared__ V s_wval[kWarps][K];
    __shared__ V s_wpref[kWarps][K];
    __shared__ V s_full[kBlock][K];
    __shared__ int s_key[kBlock];
    __shared__ int s_prev_row, s_next_row;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t t = blockIdx.x;
    const int64_t j0 = t * kTile;
    const int cnt = (int)min((int64_t)kTile, nnz - j0);
    {
        int rr[kItems], cc[kItems];
        V aa[kItems];
#pragma unroll
        for (int u = 0; u < kItems; u++) {
            const int k = tid + u * kBlock;
            rr[u] = 0;
            cc[u] = 0;
            aa[u] = V(0);
            if (k < cnt) {
                rr[u] = ld_stream(ri + j0 + k);
                cc[u] = ld_stream(ci + j0 + k);
                aa[u] = ld_stream(cv + j0 + k);
            }
        }
        if (tid == 0) {
            s_prev_row = j0 > 0 ? ri[j0 - 1] : -1;
            s_next_row = j0 + cnt < nnz ? ri[j0 + cnt] : -1;
        }
#pragma unroll
        for (int u = 0; u < kItems; u++) {
            const int k = tid + u * kBlock;
            if (k < cnt) {
                s_row[k] = rr[u];
                const V *xp = x + (int64_t)cc[u] * ldx;
#pragma unroll
                for (int q = 0; q < K; q++) s_prod[k * K + q] = aa[u] * ld_x(xp + q);
            }
        }
    }
    __syncthreads();

    // Thread owns items [b, e) (blocked).  A run of equal rows "ends" at its
    // last nonzero in the whole matrix.  The first run a thread closes may
    // have started in earlier threads (or tiles); later ones are complete.
    const int b = min(tid * kItems, cnt), e = min(b + kItems, cnt);
    V sum[K];
#pragma unroll
    for (int q = 0; q < K; q++) sum[q] = V(0);
    int first_row = -1;
    V first_val[K];
#pragma unroll
    for (int q = 0; q < K; q++) first_val[q] = V(0);
    for (int k = b; k < e; k++) {
#pragma unroll
        for (int q = 0; q < K; q++) sum[q] += s_prod[k * K + q];
        const bool ends = (k + 1 < cnt) ? (s_row[k + 1] != s_row[k]) : (s_next_row != s_row[k]);
        if (ends) {
            if (first_row < 0) {
                first_row = s_row[k];
#pragma unroll
                for (int q = 0; q < K; q++) first_val[q] = sum[q];
            } else {
                V *yp = y + (int64_t)s_row[k] * ldy;
#pragma unroll
                for (int q = 0; q < K; q++) yp[q] = axpby(alpha, sum[q], beta, yp + q);
            }
#pragma unroll
            for (int q = 0; q < K; q++) sum[q] = V(0);
        }
    }
    // trailing open run of the thread, keyed by its row (unique key if idle)
    int key = b < e ? s_row[e - 1] : -2 - tid;

    // block-wide segmented inclusive scan of (key, sum)
    const int key_up = __shfl_up_sync(0xffffffffu, key, 1);  // every lane shuffles (full mask)
    const int span = unflagged_run(lane == 0 || key_up != key);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        if (o > span) break;  // warp-uniform
        int k2 = __shfl_up_sync(0xffffffffu, key, o);
        V v2[K];
#pragma unroll
        for (int q = 0; q < K; q++) v2[q] = __shfl_up_sync(0xffffffffu, sum[q], o);
        if (lane >= o && k2 == key) {
#pragma unroll
            for (int q = 0; q < K; q++) sum[q] += v2[q];
        }
    }
    if (lane == 31) {
        s_wkey[warp] = key;
#pragma unroll
        for (int q = 0; q < K; q++) s_wval[warp][q] = sum[q];
    }
    __syncthreads();
    if (tid == 0) {
        for (int w = 0; w < kWarps; w++) {
            bool join = w > 0 && s_wkey[w] == s_wkey[w - 1];
#pragma unroll
            for (int q = 0; q < K; q++) s_wpref[w][q] = s_wval[w][q] + (join ? s_wpref[w - 1][q] : V(0));
        }
    }
    __syncthreads();
    if (warp > 0 && key == s_wkey[warp - 1]) {
#pragma unroll
        for (int q = 0; q < K; q++) sum[q] += s_wpref[warp - 1][q];
    }
#pragma unroll
    for (int q = 0; q < K; q++) s_full[tid][q] = sum[q];
    s_key[tid] = key;
    __syncthreads();

    if (first_row >= 0) {
        const bool carry = tid > 0 && s_key[tid - 1] == first_row;
        V tot[K];
#pragma unroll
        for (int q = 0; q < K; q++) tot[q] = first_val[q] + (carry ? s_full[tid - 1][q] : V(0));
        if (first_row == s_row[0] && s_prev_row == first_row) {
            V *hp = head_val + t * kMaxK;  // the run began in an earlier tile
#pragma unroll
            for (int q = 0; q < K; q++) hp[q] = tot[q];
        } else {
            V *yp = y + (int64_t)first_row * ldy;
#pragma unroll
            for (int q = 0; q < K; q++) yp[q] = axpby(alpha, tot[q], beta, yp + q);
        }
    }
    if (tid == 0) {
        const int row_last = s_row[cnt - 1];
        const bool continues = s_next_row == row_last;
        has_end[t] = !(s_row[0] == row_last && continues);
        if (continues) {
            carry_row[t] = row_last;
            const int owner = (cnt - 1) / kItems;
            V *cp = carry_val + t * kMaxK;
#pragma unroll
            for (int q = 0; q < K; q++) cp[q] = s_full[owner][q];
        } else {
            carry_row[t] = -1;
        }
    }
}

// Warp kernel (default): a warp takes kWarpChunk = 256 consecutive nonzeros,
// lane l the 8 consecutive ones at 8l (vector loads of rows, columns and
// values; all 8 gathers of x issued before use for k <= 2).  Each lane sums
// its nonzeros in order, writing every row that starts and ends inside its 8;
// the open sum before its first row end (head) and after its last (tail) are
// joined across lanes by one segmented shuffle scan keyed by "lane has a row
// end".  The row that ends first in a lane gets head + the carried tail sum;
// a row that began before the warp's chunk is left in head_val for the
// fix-up, and the chunk's open last row in carry_val.  No shared memory, no
// barriers, one shuffle scan per 256 nonzeros.
constexpr int kCooPerLane = 8;
constexpr int kWarpChunk = 32 * kCooPerLane;

template <typename V>
struct Vec2 {
    using T = double2;
};
template <>
struct Vec2<float> {
    using T = float4;
};

// Loads this lane's 8 consecutive nonzeros (n_valid of them exist).
template <typename V>
__device__ __forceinline__ void coo_load8(const int32_t *__restrict__ ri, const int32_t *__restrict__ ci,
                                          const V *__restrict__ cv, int64_t e0, int nv, bool vec, int (&r)[8],
                                          int (&c)[8], V (&a)[8]) {
    if (vec && nv == 8) {
        const int4 r0 = __ldcs(reinterpret_cast<const int4 *>(ri + e0));
        const int4 r1 = __ldcs(reinterpret_cast<const int4 *>(ri + e0 + 4));
        const int4 c0 = __ldcs(reinterpret_cast<const int4 *>(ci + e0));
        const int4 c1 = __ldcs(reinterpret_cast<const int4 *>(ci + e0 + 4));
        r[0] = r0.x; r[1] = r0.y; r[2] = r0.z; r[3] = r0.w; r[4] = r1.x; r[5] = r1.y; r[6] = r1.z; r[7] = r1.w;
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
        r[u] = u < nv ? ld_stream(ri + e0 + u) : -1;
        c[u] = u < nv ? ld_stream(ci + e0 + u) : 0;
        a[u] = u < nv ? ld_stream(cv + e0 + u) : V(0);
    }
}

// k = 1: four (FP64) or five (FP32) resident CTAs per SM, the best of 3-6
// measured on uniform, power-law and banded rows.
template <typename V, int K, bool PLAIN = false>
__global__ void __launch_bounds__(kBlock, K == 1 ? (sizeof(V) == 4 ? 5 : 4) : 1) coo_warp_kernel(
    int64_t nnz, const int32_t *__restrict__ ri, const int32_t *__restrict__ ci, const V *__restrict__ cv,
    const V *__restrict__ x, int64_t ldx, V alpha, V beta, V *__restrict__ y, int64_t ldy,
    int32_t *__restrict__ carry_row, int32_t *__restrict__ has_end, V *__restrict__ carry_val,
    V *__restrict__ head_val, int vec, int xvec) {
    constexpr unsigned kFull = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    constexpr bool plain = PLAIN;  // alpha == 1 and beta == 0: y = sum
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t j0 = w * kWarpChunk;
    if (j0 >= nnz) return;  // warp-uniform
    const int64_t j1 = min(j0 + (int64_t)kWarpChunk, nnz);
    const int64_t e0 = j0 + (int64_t)lane * kCooPerLane;
    const int nv = (int)max((int64_t)0, min((int64_t)kCooPerLane, j1 - e0));
    int r[8], c[8];
    V a[8];
    coo_load8<V>(ri, ci, cv, e0, nv, vec != 0, r, c, a);
    const int first_row = __shfl_sync(kFull, r[0], 0);
    const bool head_open = j0 > 0 && __ldg(ri + j0 - 1) == first_row;  // chunk starts inside a row
    // row of the nonzero after this lane's last one
    int next = __shfl_down_sync(kFull, r[0], 1);
    if (nv > 0 && e0 + nv == j1) next = j1 < nnz ? __ldg(ri + j1) : -1;
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
    V seg[K], head[K];
#pragma unroll
    for (int q = 0; q < K; q++) seg[q] = head[q] = V(0);
    bool any_end = false;
    int head_row = -1, last_row = -1;
#pragma unroll
    for (int u = 0; u < 8; u++) {
        if (u < nv) {
            last_row = r[u];
            if constexpr (K <= 2) {
#pragma unroll
                for (int q = 0; q < K; q++) seg[q] += a[u] * xv[u][q];
            } else {
                V xr[K];
                ld_xrow<V, K>(x, c[u], ldx, xvec != 0, xr);
#pragma unroll
                for (int q = 0; q < K; q++) seg[q] += a[u] * xr[q];
            }
            const int rn = u + 1 < nv ? r[u + 1] : next;
            if (rn != r[u]) {  // r[u] ends here
                if (!any_end) {
                    any_end = true;
                    head_row = r[u];
#pragma unroll
                    for (int q = 0; q < K; q++) head[q] = seg[q];
                } else {
                    V *yp = y + (int64_t)r[u] * ldy;
#pragma unroll
                    for (int q = 0; q < K; q++) yp[q] = row_out(plain, alpha, seg[q], beta, yp + q);
                }
#pragma unroll
                for (int q = 0; q < K; q++) seg[q] = V(0);
            }
        }
    }
    // segmented inclusive scan of the open tails; a lane with a row end starts a segment
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
    V cin[K];  // tail sums carried into this lane's first row
#pragma unroll
    for (int q = 0; q < K; q++) {
        cin[q] = __shfl_up_sync(kFull, S[q], 1);
        if (lane == 0) cin[q] = V(0);
    }
    if (any_end) {
        V tot[K];
#pragma unroll
        for (int q = 0; q < K; q++) tot[q] = head[q] + cin[q];
        if (head_row == first_row && head_open) {
            V *hp = head_val + w * kMaxK;
#pragma unroll
            for (int q = 0; q < K; q++) hp[q] = tot[q];
        } else {
            V *yp = y + (int64_t)head_row * ldy;
#pragma unroll
            for (int q = 0; q < K; q++) yp[q] = row_out(plain, alpha, tot[q], beta, yp + q);
        }
    }
    const bool chunk_end = __any_sync(kFull, any_end);
    // the lane holding the chunk's last nonzero reports the open last row
    if (nv > 0 && e0 + nv == j1) {
        const bool open = next == last_row;
        has_end[w] = chunk_end ? 1 : 0;
        carry_row[w] = open ? last_row : -1;
        if (open) {
            V *cp = carry_val + w * kMaxK;
#pragma unroll
            for (int q = 0; q < K; q++) cp[q] = S[q];
        }
    }
}

template <typename V, int K>
__global__ void coo_fixup(int64_t ntiles, const int32_t *__restrict__ ri, int tile,
                          const int32_t *__restrict__ carry_row, const int32_t *__restrict__ has_end,
                          const V *__restrict__ carry_val, const V *__restrict__ head_val, V alpha, V beta,
                          V *__restrict__ y, int64_t ldy) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t - (threadIdx.x & 31) >= ntiles) return;  // whole warp past the end
    const int r = t < ntiles ? carry_row[t] : -1;
    // owner: the tile where row r starts (it does not continue from tile t-1,
    // or tile t holds other rows before it)
    bool mine = false;
    if (r >= 0) {
        const int64_t j0 = t * (int64_t)tile;
        mine = !(ri[j0] == r && j0 > 0 && ri[j0 - 1] == r);
    }
    V tot[K];
    chain_sum<V, K>(mine, t, ntiles, 0, has_end, carry_val, head_val, tot);
    if (mine) {
        V *yp = y + (int64_t)r * ldy;
#pragma unroll
        for (int q = 0; q < K; q++) yp[q] = axpby(alpha, tot[q], beta, yp + q);
    }
}

struct CooPlan {
    int64_t ntiles[2] = {0, 0};
    int32_t *carry_row[2] = {nullptr, nullptr};
    int32_t *has_end[2] = {nullptr, nullptr};
    void *carry_val[2] = {nullptr, nullptr};
    void *head_val[2] = {nullptr, nullptr};
};

// extra[0..]: carry buffers per tile size, extra[10] = absent-row list (extra[6..8]: warp chunks)
sspmv_status ensure_coo_plan(const sspmv_coo *A, Plan *p, int which, int tile, sspmv_stream_t s) {
    if (p->extra[which * 3]) return SSPMV_OK;
    std::lock_guard<PlanMutex> g(plan_mutex());
    if (p->extra[which * 3]) return SSPMV_OK;
    const int64_t nnz = A->f.num_nnzs, m = A->f.num_rows;
    const int64_t nt = std::max<int64_t>((nnz + tile - 1) / tile, 1);
    const size_t sv = vsize(A->f.value_type);
    int32_t *ints = nullptr;
    unsigned char *cv = nullptr, *hv = nullptr;
    SSPMV_TRY(dalloc(&ints, (size_t)nt * 2, s));
    SSPMV_TRY(dalloc(&cv, (size_t)nt * kMaxK * sv, s));
    SSPMV_TRY(dalloc(&hv, (size_t)nt * kMaxK * sv, s));
    if (!p->extra[10]) {  // rows without nonzeros
        int32_t *flag = nullptr, *pos = nullptr, *list = nullptr;
        int32_t cnt = 0;
        SSPMV_TRY(dalloc(&flag, (size_t)m, s));
        SSPMV_TRY(dalloc(&pos, (size_t)m, s));
        cudaMemsetAsync(flag, 0, (size_t)std::max<int64_t>(m, 1) * 4, cu(s));
        if (nnz > 0) {
            mark_present<<<grid_for(nnz, 256, (int64_t)num_sms() * 16), 256, 0, cu(s)>>>(nnz, A->row_index, flag);
            note_launch();
        }
        if (m > 0) {
            absent_flags<<<grid_for(m, 256, (int64_t)num_sms() * 16), 256, 0, cu(s)>>>(m, flag);
            note_launch();
            SSPMV_TRY(exclusive_scan_i32(flag, pos, m, &cnt, s));
        }
        SSPMV_TRY(dalloc(&list, (size_t)cnt, s));
        if (cnt > 0) {
            absent_scatter<<<grid_for(m, 256, (int64_t)num_sms() * 16), 256, 0, cu(s)>>>(m, flag, pos, list);
            note_launch();
        }
        dfree(flag, s);
        dfree(pos, s);
        p->extra[10] = list;
        p->extra_i[10] = cnt;
    }
    p->extra_i[which * 3] = nt;
    p->extra[which * 3 + 1] = cv;
    p->extra[which * 3 + 2] = hv;
    p->extra[which * 3] = ints;  // published last
    return SSPMV_OK;
}

template <typename V, int K>
sspmv_status coo_pass(const sspmv_coo *A, Plan *p, V alpha, const V *x, int64_t ldx, V beta, V *y, int64_t ldy,
                      sspmv_stream_t s) {
    const int64_t nnz = A->f.num_nnzs, m = A->f.num_rows;
    if (!A->row_sorted) {
        scale_rows<V, K><<<grid_for(m, 256, (int64_t)num_sms() * 16), 256, 0, cu(s)>>>(m, nullptr, beta, y, ldy);
        SSPMV_LAUNCH_CHECK();
        if (nnz > 0) {
            coo_atomic<V, K><<<grid_for(nnz, 256, (int64_t)num_sms() * 16), 256, 0, cu(s)>>>(
                nnz, A->row_index, A->col_index, (const V *)A->values, alpha, x, ldx, y, ldy);
            SSPMV_LAUNCH_CHECK();
        }
        return SSPMV_OK;
    }
    const bool warp_kernel = A->f.kernel_flag != 1;
    const int tile = warp_kernel ? kWarpChunk : CooShape<K>::tile;
    const int which = warp_kernel ? 2 : (K <= 4 ? 0 : 1);
    SSPMV_TRY(ensure_coo_plan(A, p, which, tile, s));
    const int64_t nt = p->extra_i[which * 3];
    int32_t *ints = (int32_t *)p->extra[which * 3];
    const int64_t nabs = p->extra_i[10];
    if (nabs > 0) {
        scale_rows<V, K><<<grid_for(nabs, 256, (int64_t)num_sms() * 16), 256, 0, cu(s)>>>(
            nabs, (const int32_t *)p->extra[10], beta, y, ldy);
        SSPMV_LAUNCH_CHECK();
    }
    if (nnz == 0) return SSPMV_OK;
    if (warp_kernel) {
        const int vec = ((reinterpret_cast<uintptr_t>(A->row_index) | reinterpret_cast<uintptr_t>(A->col_index) |
                          reinterpret_cast<uintptr_t>(A->values)) & 15) == 0;
        auto go = [&](auto kernel) {
            kernel<<<grid_for(nt * 32, kBlock), kBlock, 0, cu(s)>>>(
                nnz, A->row_index, A->col_index, (const V *)A->values, x, ldx, alpha, beta, y, ldy, ints, ints + nt,
                (V *)p->extra[which * 3 + 1], (V *)p->extra[which * 3 + 2], vec, xrow_vec(x, ldx, sizeof(V), K));
        };
        if (K == 1 && alpha == V(1) && beta == V(0)) go(coo_warp_kernel<V, K, K == 1>);
        else go(coo_warp_kernel<V, K>);
        SSPMV_LAUNCH_CHECK();
        if (nt > 1) {
            coo_fixup<V, K><<<grid_for(nt, 256), 256, 0, cu(s)>>>(nt, A->row_index, tile, ints, ints + nt,
                                                                  (const V *)p->extra[which * 3 + 1],
                                                                  (const V *)p->extra[which * 3 + 2], alpha, beta, y,
                                                                  ldy);
            SSPMV_LAUNCH_CHECK();
        }
        return SSPMV_OK;
    }
    const size_t smem = (size_t)tile * K * sizeof(V) + (size_t)tile * 4;
    static std::atomic<bool> attr{false};  // set after the attribute call returns
    if (!attr.load(std::memory_order_acquire)) {
        SSPMV_CUDA_TRY(cudaFuncSetAttribute(coo_tile_kernel<V, K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr.store(true, std::memory_order_release);
    }
    coo_tile_kernel<V, K><<<(unsigned)nt, kBlock, smem, cu(s)>>>(nnz, A->row_index, A->col_index, (const V *)A->values,
                                                                 x, ldx, alpha, beta, y, ldy, ints, ints + nt,
                                                                 (V *)p->extra[which * 3 + 1],
                                                                 (V *)p->extra[which * 3 + 2]);
    SSPMV_LAUNCH_CHECK();
    if (nt > 1) {
        coo_fixup<V, K><<<grid_for(nt, 256), 256, 0, cu(s)>>>(nt, A->row_index, tile, ints, ints + nt,
                                                              (const V *)p->extra[which * 3 + 1],
                                                              (const V *)p->extra[which * 3 + 2], alpha, beta, y, ldy);
        SSPMV_LAUNCH_CHECK();
    }
    return SSPMV_OK;
}

}  // namespace

extern "C" sspmv_status sspmv_csr_to_coo(const sspmv_csr *csr, sspmv_coo *out, sspmv_stream_t s) {
    if (!csr || !out) return fail(SSPMV_INVALID_ARG, "null argument");
    SSPMV_TRY(check_dims(csr->f.value_type, csr->f.num_rows, csr->f.num_cols, csr->f.num_nnzs));
    const int64_t m = csr->f.num_rows, nnz = csr->f.num_nnzs;
    const size_t sv = vsize(csr->f.value_type);
    sspmv_coo A;
    init_features(&A.f, csr->f.value_type, m, csr->f.num_cols, nnz, 1);
    A.row_index = A.col_index = nullptr;
    A.values = nullptr;
    A.row_sorted = 1;
    sspmv_status st = dalloc(&A.row_index, (size_t)nnz, s);
    if (st == SSPMV_OK) st = dalloc(&A.col_index, (size_t)nnz, s);
    if (st == SSPMV_OK) st = dalloc((unsigned char **)&A.values, (size_t)nnz * sv, s);
    if (st == SSPMV_OK && nnz > 0) {
        expand_rows<<<grid_for(m * 32, 256, (int64_t)num_sms() * 32), 256, 0, cu(s)>>>(m, csr->row_offset, A.row_index);
        note_launch();
        cudaError_t e = cudaMemcpyAsync(A.col_index, csr->col_index, (size_t)nnz * 4, cudaMemcpyDeviceToDevice, cu(s));
        if (e == cudaSuccess) e = cudaMemcpyAsync(A.values, csr->values, (size_t)nnz * sv, cudaMemcpyDeviceToDevice, cu(s));
        if (e == cudaSuccess) e = cudaStreamSynchronize(cu(s));
        if (e != cudaSuccess) st = fail(SSPMV_CUDA_ERROR, "csr_to_coo: %s", cudaGetErrorString(e));
    }
    if (st != SSPMV_OK) {
        dfree(A.row_index, s);
        dfree(A.col_index, s);
        dfree(A.values, s);
        return st;
    }
    *out = A;
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_coo_create(sspmv_coo *out, int32_t vt, int64_t m, int64_t n, int64_t nnz,
                                         const int32_t *row_index, const int32_t *col_index, const void *values,
                                         int32_t from_host, sspmv_stream_t s) {
    if (!out) return fail(SSPMV_INVALID_ARG, "null output");
    SSPMV_TRY(check_dims(vt, m, n, nnz));
    if (nnz > 0 && (!row_index || !col_index || !values)) return fail(SSPMV_INVALID_ARG, "null array");
    int32_t sorted = 1;
    if (from_host) {
        long long bad = 0, unsorted = 0;
#pragma omp parallel for reduction(+ : bad, unsorted)
        for (int64_t j = 0; j < nnz; j++) {
            bad += row_index[j] < 0 || row_index[j] >= m || col_index[j] < 0 || col_index[j] >= n;
            unsorted += j > 0 && row_index[j] < row_index[j - 1];
        }
        if (bad) return fail(SSPMV_INVALID_ARG, "row or column index out of range");
        sorted = unsorted == 0;
    }
    const size_t sv = vsize(vt);
    sspmv_coo A;
    init_features(&A.f, vt, m, n, nnz, 1);
    A.row_index = A.col_index = nullptr;
    A.values = nullptr;
    A.row_sorted = from_host ? sorted : 0;
    sspmv_status st = dalloc(&A.row_index, (size_t)nnz, s);
    if (st == SSPMV_OK) st = dalloc(&A.col_index, (size_t)nnz, s);
    if (st == SSPMV_OK) st = dalloc((unsigned char **)&A.values, (size_t)nnz * sv, s);
    if (st == SSPMV_OK && nnz > 0) {
        cudaMemcpyKind kd = from_host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
        cudaError_t e = cudaMemcpyAsync(A.row_index, row_index, (size_t)nnz * 4, kd, cu(s));
        if (e == cudaSuccess) e = cudaMemcpyAsync(A.col_index, col_index, (size_t)nnz * 4, kd, cu(s));
        if (e == cudaSuccess) e = cudaMemcpyAsync(A.values, values, (size_t)nnz * sv, kd, cu(s));
        if (e == cudaSuccess) e = cudaStreamSynchronize(cu(s));
        if (e != cudaSuccess) st = fail(SSPMV_CUDA_ERROR, "coo_create: %s", cudaGetErrorString(e));
    }
    if (st != SSPMV_OK) {
        dfree(A.row_index, s);
        dfree(A.col_index, s);
        dfree(A.values, s);
        return st;
    }
    *out = A;
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_coo_to_csr(const sspmv_coo *coo, sspmv_csr *out, sspmv_stream_t s) {
    if (!coo || !out) return fail(SSPMV_INVALID_ARG, "null argument");
    const int64_t m = coo->f.num_rows, nnz = coo->f.num_nnzs;
    const int32_t vt = coo->f.value_type;
    const size_t sv = vsize(vt);
    uint64_t *keys = nullptr;
    uint32_t *perm = nullptr;
    sspmv_csr A;
    init_features(&A.f, vt, m, coo->f.num_cols, nnz, 1);
    A.row_offset = A.col_index = nullptr;
    A.values = nullptr;
    sspmv_status st = dalloc(&keys, (size_t)nnz, s);
    if (st == SSPMV_OK) st = dalloc(&perm, (size_t)nnz, s);
    if (st == SSPMV_OK) st = dalloc(&A.row_offset, (size_t)m + 1, s);
    if (st == SSPMV_OK) st = dalloc(&A.col_index, (size_t)nnz, s);
    if (st == SSPMV_OK) st = dalloc((unsigned char **)&A.values, (size_t)nnz * sv, s);
    const unsigned g = grid_for(std::max<int64_t>(nnz, 1), 256, (int64_t)num_sms() * 16);
    if (st == SSPMV_OK && nnz > 0) {
        coo_keys<<<g, 256, 0, cu(s)>>>(nnz, coo->row_index, keys, perm);
        note_launch();
        st = radix_sort_pairs(keys, perm, nnz, bits_for((uint64_t)std::max<int64_t>(m - 1, 1)), s);
        if (st == SSPMV_OK)
            st = dispatch_value(vt, [&](auto tag) -> sspmv_status {
                using V = decltype(tag);
                coo_gather<V><<<g, 256, 0, cu(s)>>>(nnz, perm, coo->col_index, (const V *)coo->values, A.col_index,
                                                    (V *)A.values);
                SSPMV_LAUNCH_CHECK();
                return SSPMV_OK;
            });
    }
    if (st == SSPMV_OK) {
        rows_to_offsets<<<grid_for(m + 1, 256, (int64_t)num_sms() * 16), 256, 0, cu(s)>>>(m, nnz, keys, A.row_offset);
        note_launch();
        cudaError_t e = cudaStreamSynchronize(cu(s));
        if (e != cudaSuccess) st = fail(SSPMV_CUDA_ERROR, "coo_to_csr: %s", cudaGetErrorString(e));
    }
    dfree(keys, s);
    dfree(perm, s);
    if (st != SSPMV_OK) {
        dfree(A.row_offset, s);
        dfree(A.col_index, s);
        dfree(A.values, s);
        return st;
    }
    *out = A;
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_spmm_coo(double alpha, const sspmv_coo *A, int32_t k, const void *X, int64_t ldx,
                                       double beta, void *Y, int64_t ldy, sspmv_stream_t s) {
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
            case 8: return coo_pass<V, 8>(A, p, a, xs, ldx, b, ys, ldy, s);
            case 4: return coo_pass<V, 4>(A, p, a, xs, ldx, b, ys, ldy, s);
            case 2: return coo_pass<V, 2>(A, p, a, xs, ldx, b, ys, ldy, s);
            default: return coo_pass<V, 1>(A, p, a, xs, ldx, b, ys, ldy, s);
            }
        });
    });
}

extern "C" sspmv_status sspmv_LeSpMV_coo(double alpha, const sspmv_coo *A, const void *x, double beta, void *y,
                                         sspmv_stream_t s) {
    return sspmv_spmm_coo(alpha, A, 1, x, 1, beta, y, 1, s);
}

extern "C" sspmv_status sspmv_coo_export(const sspmv_coo *A, int32_t *row_index, int32_t *col_index, void *values,
                                         sspmv_stream_t s) {
    if (!A) return fail(SSPMV_INVALID_ARG, "null matrix");
    const size_t nnz = (size_t)A->f.num_nnzs;
    if (row_index && nnz) SSPMV_CUDA_TRY(cudaMemcpyAsync(row_index, A->row_index, nnz * 4, cudaMemcpyDeviceToHost, cu(s)));
    if (col_index && nnz) SSPMV_CUDA_TRY(cudaMemcpyAsync(col_index, A->col_index, nnz * 4, cudaMemcpyDeviceToHost, cu(s)));
    if (values && nnz)
        SSPMV_CUDA_TRY(cudaMemcpyAsync(values, A->values, nnz * vsize(A->f.value_type), cudaMemcpyDeviceToHost, cu(s)));
    SSPMV_CUDA_TRY(cudaStreamSynchronize(cu(s)));
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_delete_coo(sspmv_coo *A) {
    if (!A) return SSPMV_OK;
    delete_barrier();
    free_plan(&A->f, nullptr);
    if (A->f.owns) {
        dfree(A->row_index, nullptr);
        dfree(A->col_index, nullptr);
        dfree(A->values, nullptr);
    }
    A->row_index = A->col_index = nullptr;
    A->values = nullptr;
    return SSPMV_OK;
}

extern "C" double sspmv_algorithmic_bytes_coo(const sspmv_coo *A, int32_t k, int32_t beta_nonzero) {
    const double sv = (double)vsize(A->f.value_type);
    return (double)A->f.num_nnzs * (sv + 8.0) + (double)k * (double)A->f.num_cols * sv +
           (double)k * (double)A->f.num_rows * sv * (beta_nonzero ? 2.0 : 1.0);
}
