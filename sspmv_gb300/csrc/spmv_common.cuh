// spmv_common.cuh -- helpers shared by the SpMV / SpMM entry points.
#pragma once

#include "common.cuh"

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

}  // namespace sspmv
