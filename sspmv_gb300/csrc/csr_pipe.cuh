// csr_pipe.cuh -- the pipelined CSR kernel (LeSpMV_csr kernel_flag 4), built
// in its own translation unit (csr_pipe.cu).
#pragma once

#include "plan.cuh"

namespace sspmv {

// One SpMV (one right-hand side) with the pipelined kernel.  Plan param: bit
// 0 set -- a row's values are loaded one iteration ahead with its columns,
// else with its x gathers; bits 1-2 -- log2 of the lanes per row (1, 2, 4 or
// 8); bit 3 set -- CTAs of 1024 threads instead of 256 where the register
// budget allows four 256-thread CTAs per SM.  Sets *launched = false,
// launching nothing, when a row is longer than the kernel takes: 12
// nonzeros with one lane per row, 8 per lane with more.
// Plan slot extra_i[7] caches the longest row + 1.
template <typename V>
sspmv_status launch_csr_pipe(const sspmv_csr *A, Plan *p, V alpha, const V *x, int64_t ldx, V beta, V *y,
                             int64_t ldy, sspmv_stream_t s, bool *launched);

}  // namespace sspmv
