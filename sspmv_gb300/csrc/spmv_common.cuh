// spmv_common.cuh -- helpers shared by the SpMV / SpMM entry points.
#pragma once

#include "common.cuh"
#include "plan.cuh"

namespace sspmv {

// Validates the arguments of an SpMM call on a matrix with features f.
sspmv_status check_spmm_args(const sspmv_features *f, int32_t k, const void *X, int64_t ldx, const void *Y,
                             int64_t ldy);

// Runs pass(step, X + done, Y + done) over k right-hand sides in passes of
// 8, 4, 2 and 1 columns (the kernels are instantiated for those widths).
template <typename V, typename Pass>
sspmv_status for_rhs_chunks(int32_t k, const V *X, V *Y, Pass &&pass) {
    int32_t done = 0;
    while (done < k) {
        int32_t left = k - done, step = left >= 8 ? 8 : left >= 4 ? 4 : left >= 2 ? 2 : 1;
        SSPMV_TRY(pass(step, X + done, Y + done));
        done += step;
    }
    return SSPMV_OK;
}

// Rows that cross tile (or chunk) boundaries: the tile t where such a row
// begins holds its open sum in carry_val[t]; each later tile u holds either a
// piece of it in carry_val[u] (has_end[u] == 0: the row runs through u) or its
// last piece in head_val[u] (has_end[u] != 0).  chain_sum totals the row for
// every lane of a warp whose `mine` is set (lane = tile t): each lane first
// walks up to kChainWalk following tiles itself (most rows end in the next
// tile); the warp then finishes the longer chains one at a time, 32 tiles per
// step, each step's pieces summed by a fixed shuffle tree.  The order of the
// additions depends only on the chain, so the result is deterministic, and a
// row crossing hundreds of tiles costs a few steps instead of a sequential
// walk.  Called by all 32 lanes; tile u of a lane's matrix has carry slot
// u + shift (lanes may belong to different matrices of a batch: a chain is
// finished with its own lane's n and shift).
constexpr int kChainWalk = 4;

template <typename V, int K>
__device__ __forceinline__ void chain_sum(bool mine, int64_t t, int64_t n, int64_t shift,
                                          const int32_t *__restrict__ has_end, const V *__restrict__ carry_val,
                                          const V *__restrict__ head_val, V (&tot)[K]) {
    constexpr unsigned kFull = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    auto at = [shift](int64_t u) { return u + shift; };
    bool open = mine;
    int64_t u = t + 1;
#pragma unroll
    for (int q = 0; q < K; q++) tot[q] = mine ? carry_val[at(t) * kMaxK + q] : V(0);
#pragma unroll
    for (int step = 0; step < kChainWalk; step++) {
        if (open) {
            if (u >= n) {
                open = false;
            } else if (has_end[at(u)]) {
#pragma unroll
                for (int q = 0; q < K; q++) tot[q] += head_val[at(u) * kMaxK + q];
                open = false;
            } else {
#pragma unroll
                for (int q = 0; q < K; q++) tot[q] += carry_val[at(u) * kMaxK + q];
                u++;
            }
        }
    }
    unsigned pending = __ballot_sync(kFull, open);
    while (pending) {  // warp-uniform: lane l's chain, with lane l's tile count and slot shift
        const int l = __ffs(pending) - 1;
        pending &= pending - 1;
        const int64_t ln = __shfl_sync(kFull, n, l), lshift = __shfl_sync(kFull, shift, l);
        for (int64_t b = __shfl_sync(kFull, u, l); b < ln; b += 32) {
            const int64_t w = b + lane;
            const bool in = w < ln;
            const int64_t sw = in ? w + lshift : 0;
            const unsigned ends = __ballot_sync(kFull, in && has_end[sw] != 0);
            const int first = ends ? __ffs(ends) - 1 : 32;
#pragma unroll
            for (int q = 0; q < K; q++) {
                V part = V(0);
                if (in && lane < first) part = carry_val[sw * kMaxK + q];
                else if (in && lane == first) part = head_val[sw * kMaxK + q];
                part = warp_sum(part);
                if (lane == l) tot[q] += part;
            }
            if (ends) break;
        }
    }
}

}  // namespace sspmv
