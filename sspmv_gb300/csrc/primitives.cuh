// primitives.cuh -- device building blocks of the GPU converters:
// exclusive scan, stable LSD radix sort of (key, value) pairs, row-length
// maximum.  All are stream ordered; the ones returning host values
// synchronize the stream.
#pragma once

#include "common.cuh"

namespace sspmv {

// out[i] = sum(in[0..i-1]); in and out may alias.  If h_total is not null the
// stream is synchronized and the grand total is stored there.
sspmv_status exclusive_scan_i64(const int64_t *in, int64_t *out, int64_t n, int64_t *h_total, sspmv_stream_t s);
sspmv_status exclusive_scan_i32(const int32_t *in, int32_t *out, int64_t n, int32_t *h_total, sspmv_stream_t s);

// Stable ascending sort of n (key, value) pairs on key bits [0, end_bit).
// Sorts in place (uses temporary device buffers of the same size).
sspmv_status radix_sort_pairs(uint64_t *keys, uint32_t *vals, int64_t n, int end_bit, sspmv_stream_t s);

// max over rows of (row_offset[i+1] - row_offset[i]); 0 when m == 0.
sspmv_status max_row_length(const int32_t *row_offset, int64_t m, int32_t *h_max, sspmv_stream_t s);

inline int bits_for(uint64_t v) {
    int b = 0;
    while (b < 64 && (v >> b) != 0) b++;
    return b;
}

}  // namespace sspmv
