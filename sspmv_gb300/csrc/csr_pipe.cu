// csr_pipe.cu -- the pipelined CSR kernel (LeSpMV_csr kernel_flag 4, one
// right-hand side) on sm_103a.
//
// Short rows, a persistent grid striding over rows r, r + T, r + 2T, ... (T =
// the rows one grid step takes), VS lanes per row (1, 2, 4 or 8).  A
// short-row SpMV is a chain of three dependent loads per row -- row offsets,
// then columns, then x -- and with one row per thread at a time the chain's
// latency, not DRAM bandwidth, sets the time of an 84 MB matrix.  Here each
// lane keeps three rows in flight: the iteration that finishes row r first
// issues row r's x gathers (its columns were loaded one iteration earlier),
// the columns of row r + T (offsets loaded one iteration earlier) and the
// offsets of row r + 2T, and only then waits for row r's gathers and runs its
// FMA chain (lane `sub` takes elements sub, sub + VS, ... in order; VS > 1
// joins the lanes' sums with a fixed shuffle tree).  EARLY: a row's values
// are loaded with its columns, one iteration ahead, off the FMA's critical
// path (fewer threads per SM); otherwise with its gathers, so no value waits
// in registers across an iteration (more threads per SM).  Measured (ncu, L2
// flushed): the FP64 1024^2 Laplacian 15.4 us against 19.3 us for the
// one-lane vector kernel, banded rows of 9 FP64 45 against 57 us; the two
// value-load points within a few percent of each other.
//
// H (the lane's share of the longest row, rounded up to a template size) sets
// the hoisted loads per row; lanes past their row's end multiply 0 by 0
// (never x: it may hold Inf or NaN), and a warp's FMA steps stop at its
// longest share.  BLK (256 or 1024 threads per CTA) changes only how many
// CTAs the grid has: with a quarter as many, a launch reaches its first
// loads sooner (FP64 Laplacian 19.65 against 20.13 us per launch, FP32
// 14.18 against 15.24 us, dithered CUDA-event times).
#include <atomic>
#include <mutex>

#include "common.cuh"
#include "csr_pipe.cuh"
#include "primitives.cuh"

namespace sspmv {
namespace {

constexpr int kPipeMaxRow = 12;     // one lane per row
constexpr int kPipeMaxPerLane = 8;  // more lanes per row

// Resident CTAs of 256 threads per SM the register budget is set for.
template <typename V, int H, bool EARLY>
constexpr int pipe_min_blocks() {
    if constexpr (sizeof(V) == 8) return EARLY ? (H > 8 ? 2 : H > 6 ? 3 : 4) : (H > 8 ? 3 : H > 6 ? 4 : H > 5 ? 5 : 6);
    return EARLY ? (H > 8 ? 4 : 5) : (H > 8 ? 5 : H > 5 ? 6 : 8);
}

// The same budget for CTAs of BLK threads (256 or 1024).
template <typename V, int H, bool EARLY, int BLK>
constexpr int pipe_min_ctas() {
    return pipe_min_blocks<V, H, EARLY>() * 256 / BLK > 0 ? pipe_min_blocks<V, H, EARLY>() * 256 / BLK : 1;
}

template <typename V, int H, int VS, bool EARLY, bool PLAIN, int BLK>
__global__ void __launch_bounds__(BLK, (pipe_min_ctas<V, H, EARLY, BLK>())) csr_pipe_kernel(
    int64_t m, const int32_t *__restrict__ rp, const int32_t *__restrict__ col, const V *__restrict__ val,
    const V *__restrict__ x, int64_t ldx, V alpha, V beta, V *__restrict__ y, int64_t ldy) {
    constexpr unsigned kAll = 0xffffffffu;
    const int64_t T = (int64_t)gridDim.x * (BLK / VS);
    const int lane = threadIdx.x & 31, sub = lane % VS, lead = lane / VS;
    int64_t r = ((int64_t)blockIdx.x * BLK + threadIdx.x) / VS;
    // this lane's elements of a row of n nonzeros: sub, sub + VS, ...
    auto share = [&](int n) { return n > sub ? (n - sub + VS - 1) / VS : 0; };
    // prologue: row r's offsets (waited for) and columns (values: EARLY),
    // row r + T's offsets
    int rs0 = 0, n0 = 0;
    if (r < m) {
        rs0 = ld_stream(rp + r);
        n0 = share(ld_stream(rp + r + 1) - rs0);
    }
    int c0[H];
    V a0[H];
#pragma unroll
    for (int q = 0; q < H; q++) {
        c0[q] = 0;
        a0[q] = V(0);
        if (q < n0) {
            c0[q] = ld_stream(col + rs0 + sub + q * VS);
            if constexpr (EARLY) a0[q] = ld_stream(val + rs0 + sub + q * VS);
        }
    }
    int rs1 = 0, re1 = 0;
    if (r + T < m) {
        rs1 = ld_stream(rp + r + T);
        re1 = ld_stream(rp + r + T + 1);
    }
#pragma unroll 1
    for (; r - lead < m; r += T) {  // warp-uniform: the warp's first row
        V xv[H];
#pragma unroll
        for (int q = 0; q < H; q++) {
            xv[q] = V(0);
            if (q < n0) {
                xv[q] = ld_x(x + (int64_t)c0[q] * ldx);
                if constexpr (!EARLY) a0[q] = ld_stream(val + rs0 + sub + q * VS);
            }
        }
        const int n1 = share(re1 - rs1);
        int c1[H];
        V a1[H];
#pragma unroll
        for (int q = 0; q < H; q++) {
            c1[q] = 0;
            a1[q] = V(0);
            if (q < n1) {
                c1[q] = ld_stream(col + rs1 + sub + q * VS);
                if constexpr (EARLY) a1[q] = ld_stream(val + rs1 + sub + q * VS);
            }
        }
        int rs2 = 0, re2 = 0;
        if (r + 2 * T < m) {
            rs2 = ld_stream(rp + r + 2 * T);
            re2 = ld_stream(rp + r + 2 * T + 1);
        }
        const int wmax = __reduce_max_sync(kAll, n0);
        V sum = V(0);
#pragma unroll
        for (int q = 0; q < H; q++)
            if (q < wmax) sum = fma(a0[q], xv[q], sum);
        if constexpr (VS > 1) sum = warp_sum(sum, VS);
        if (r < m && sub == 0) {
            V *yp = y + r * ldy;
            *yp = row_out(PLAIN, alpha, sum, beta, yp);
        }
#pragma unroll
        for (int q = 0; q < H; q++) {
            c0[q] = c1[q];
            a0[q] = EARLY ? a1[q] : V(0);
        }
        rs0 = rs1;
        n0 = n1;
        rs1 = rs2;
        re1 = re2;
    }
}

template <typename V, int H, int VS, bool EARLY, bool PLAIN, int BLK>
sspmv_status go_pipe_k(const sspmv_csr *A, V alpha, const V *x, int64_t ldx, V beta, V *y, int64_t ldy,
                       sspmv_stream_t s) {
    // resident CTAs per SM, found once per instantiation
    static std::atomic<int> per_sm{0};
    if (per_sm.load(std::memory_order_acquire) == 0) {
        int n = 0;
        SSPMV_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &n, csr_pipe_kernel<V, H, VS, EARLY, PLAIN, BLK>, BLK, 0));
        per_sm.store(n > 0 ? n : 1, std::memory_order_release);
    }
    const int64_t m = A->f.num_rows;
    const unsigned grid = grid_for(m * VS, BLK, (int64_t)num_sms() * per_sm.load(std::memory_order_acquire));
    csr_pipe_kernel<V, H, VS, EARLY, PLAIN, BLK><<<grid, BLK, 0, cu(s)>>>(
        m, A->row_offset, A->col_index, (const V *)A->values, x, ldx, alpha, beta, y, ldy);
    SSPMV_LAUNCH_CHECK();
    return SSPMV_OK;
}

template <typename V, int H, int VS, bool EARLY, int BLK>
sspmv_status go_pipe_p(const sspmv_csr *A, V alpha, const V *x, int64_t ldx, V beta, V *y, int64_t ldy,
                       sspmv_stream_t s) {
    if (alpha == V(1) && beta == V(0)) return go_pipe_k<V, H, VS, EARLY, true, BLK>(A, alpha, x, ldx, beta, y, ldy, s);
    return go_pipe_k<V, H, VS, EARLY, false, BLK>(A, alpha, x, ldx, beta, y, ldy, s);
}

// big: CTAs of 1024 threads instead of 256 (a quarter as many CTAs), where
// the register budget allows four 256-thread CTAs per SM; otherwise 256.
template <typename V, int H, int VS>
sspmv_status go_pipe(const sspmv_csr *A, bool early, bool big, V alpha, const V *x, int64_t ldx, V beta, V *y,
                     int64_t ldy, sspmv_stream_t s) {
    if (early) {
        if constexpr (pipe_min_blocks<V, H, true>() >= 4)
            if (big) return go_pipe_p<V, H, VS, true, 1024>(A, alpha, x, ldx, beta, y, ldy, s);
        return go_pipe_p<V, H, VS, true, 256>(A, alpha, x, ldx, beta, y, ldy, s);
    }
    if constexpr (pipe_min_blocks<V, H, false>() >= 4)
        if (big) return go_pipe_p<V, H, VS, false, 1024>(A, alpha, x, ldx, beta, y, ldy, s);
    return go_pipe_p<V, H, VS, false, 256>(A, alpha, x, ldx, beta, y, ldy, s);
}

// VS > 1: H = the lane's share of the longest row, rounded up to 4 or 8.
template <typename V, int VS>
sspmv_status go_pipe_lanes(const sspmv_csr *A, int64_t per_lane, bool early, bool big, V alpha, const V *x,
                           int64_t ldx, V beta, V *y, int64_t ldy, sspmv_stream_t s) {
    if (per_lane <= 4) return go_pipe<V, 4, VS>(A, early, big, alpha, x, ldx, beta, y, ldy, s);
    return go_pipe<V, 8, VS>(A, early, big, alpha, x, ldx, beta, y, ldy, s);
}

}  // namespace

template <typename V>
sspmv_status launch_csr_pipe(const sspmv_csr *A, Plan *p, V alpha, const V *x, int64_t ldx, V beta, V *y,
                             int64_t ldy, sspmv_stream_t s, bool *launched) {
    *launched = false;
    if (p->extra_i[7] == 0) {
        std::lock_guard<PlanMutex> g(plan_mutex());
        if (p->extra_i[7] == 0) {
            int32_t longest = 0;
            SSPMV_TRY(max_row_length(A->row_offset, A->f.num_rows, &longest, s));
            p->extra_i[7] = (int64_t)longest + 1;
        }
    }
    const int64_t longest = p->extra_i[7] - 1;
    const bool early = (p->param & 1) != 0;
    const int vs = 1 << ((p->param >> 1) & 3);
    const bool big = (p->param & 8) != 0;
    if (vs == 1) {
        if (longest > kPipeMaxRow) return SSPMV_OK;
        switch (longest) {
        case 0:
        case 1:
        case 2: SSPMV_TRY((go_pipe<V, 2, 1>(A, early, big, alpha, x, ldx, beta, y, ldy, s))); break;
        case 3: SSPMV_TRY((go_pipe<V, 3, 1>(A, early, big, alpha, x, ldx, beta, y, ldy, s))); break;
        case 4: SSPMV_TRY((go_pipe<V, 4, 1>(A, early, big, alpha, x, ldx, beta, y, ldy, s))); break;
        case 5: SSPMV_TRY((go_pipe<V, 5, 1>(A, early, big, alpha, x, ldx, beta, y, ldy, s))); break;
        case 6: SSPMV_TRY((go_pipe<V, 6, 1>(A, early, big, alpha, x, ldx, beta, y, ldy, s))); break;
        case 7:
        case 8: SSPMV_TRY((go_pipe<V, 8, 1>(A, early, big, alpha, x, ldx, beta, y, ldy, s))); break;
        case 9:
        case 10: SSPMV_TRY((go_pipe<V, 10, 1>(A, early, big, alpha, x, ldx, beta, y, ldy, s))); break;
        default: SSPMV_TRY((go_pipe<V, 12, 1>(A, early, big, alpha, x, ldx, beta, y, ldy, s))); break;
        }
    } else {
        const int64_t per_lane = (longest + vs - 1) / vs;
        if (per_lane > kPipeMaxPerLane) return SSPMV_OK;
        switch (vs) {
        case 2: SSPMV_TRY((go_pipe_lanes<V, 2>(A, per_lane, early, big, alpha, x, ldx, beta, y, ldy, s))); break;
        case 4: SSPMV_TRY((go_pipe_lanes<V, 4>(A, per_lane, early, big, alpha, x, ldx, beta, y, ldy, s))); break;
        default: SSPMV_TRY((go_pipe_lanes<V, 8>(A, per_lane, early, big, alpha, x, ldx, beta, y, ldy, s))); break;
        }
    }
    *launched = true;
    return SSPMV_OK;
}

template sspmv_status launch_csr_pipe<float>(const sspmv_csr *, Plan *, float, const float *, int64_t, float,
                                             float *, int64_t, sspmv_stream_t, bool *);
template sspmv_status launch_csr_pipe<double>(const sspmv_csr *, Plan *, double, const double *, int64_t, double,
                                              double *, int64_t, sspmv_stream_t, bool *);

}  // namespace sspmv
