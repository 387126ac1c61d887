// common.cuh -- shared internals of libsspmv: status/error plumbing, value
// type dispatch, device memory helpers and small device utilities.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>

#include "sspmv.h"

namespace sspmv {

// ---------------------------------------------------------------- errors --
void set_error(const char *fmt, ...);
sspmv_status fail(sspmv_status s, const char *fmt, ...);

#define SSPMV_CUDA_TRY(expr)                                                            \
    do {                                                                                \
        cudaError_t e_ = (expr);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            return ::sspmv::fail(e_ == cudaErrorMemoryAllocation ? SSPMV_OUT_OF_MEMORY \
                                                                 : SSPMV_CUDA_ERROR,    \
                                 "%s:%d %s: %s", __FILE__, __LINE__, #expr,             \
                                 cudaGetErrorString(e_));                               \
        }                                                                               \
    } while (0)

// Every kernel launch of the library is counted (sspmv_launch_count).
void note_launch();

#define SSPMV_LAUNCH_CHECK()                 \
    do {                                     \
        ::sspmv::note_launch();              \
        SSPMV_CUDA_TRY(cudaGetLastError());  \
    } while (0)

#define SSPMV_TRY(expr)                         \
    do {                                        \
        sspmv_status s_ = (expr);               \
        if (s_ != SSPMV_OK) return s_;          \
    } while (0)

inline cudaStream_t cu(sspmv_stream_t s) { return reinterpret_cast<cudaStream_t>(s); }

// ---------------------------------------------------------------- memory --
// Library-owned device allocations are stream ordered (cudaMallocAsync).
template <typename T>
sspmv_status dalloc(T **p, size_t count, sspmv_stream_t s) {
    *p = nullptr;
    if (count == 0) count = 1;
    SSPMV_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void **>(p), count * sizeof(T), cu(s)));
    return SSPMV_OK;
}
inline void dfree(void *p, sspmv_stream_t s) {
    if (p) cudaFreeAsync(p, cu(s));
}

// sspmv_delete_<fmt> waits for the whole device before freeing (the matrix
// may still be in use on any stream).  A caller that knows no queued work
// uses the matrix any more (the request server, after the matrix's last
// batch completed) opens this scope on its thread to skip that wait.
struct DeleteWithoutDeviceSync {
    DeleteWithoutDeviceSync();
    ~DeleteWithoutDeviceSync();
};
void delete_barrier();

inline size_t vsize(int32_t vt) { return vt == SSPMV_F64 ? 8 : 4; }
inline int default_alignment(int32_t vt) { return 64 / (int)vsize(vt); }  // SIMD_WIDTH/8/sizeof(V)

inline bool valid_vt(int32_t vt) { return vt == SSPMV_F32 || vt == SSPMV_F64; }

// Calls f.template operator()<V>() with V = float or double.
template <typename F>
sspmv_status dispatch_value(int32_t vt, F &&f) {
    if (vt == SSPMV_F64) return f((double)0);
    if (vt == SSPMV_F32) return f((float)0);
    return fail(SSPMV_INVALID_ARG, "unknown value_type %d", vt);
}

inline int num_sms() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 152;
    }
    return n;
}

inline unsigned grid_for(int64_t work, int block, int64_t cap = 0) {
    int64_t g = (work + block - 1) / block;
    if (g < 1) g = 1;
    if (cap > 0 && g > cap) g = cap;
    if (g > 0x7fffffff) g = 0x7fffffff;
    return (unsigned)g;
}

// --------------------------------------------------------- device helpers --
// Streaming (evict-first) loads for matrix arrays that are read once per SpMV.
template <typename T>
__device__ __forceinline__ T ld_stream(const T *p) { return __ldcs(p); }
// Read-only cached loads for the gathered vector.
template <typename T>
__device__ __forceinline__ T ld_x(const T *p) { return __ldg(p); }

// Row j of a row-major block X of K right-hand sides (leading dimension ldx
// values): with `vec` set, one vector load per 16 bytes of the row (8 bytes
// for FP32 with K = 2), else K scalar loads; read-only cached like ld_x.  A
// warp gathering K-wide rows this way touches each row's sector once instead
// of once per column (K scalar loads are K separate L1 lookups per lane).
template <typename V, int K>
__device__ __forceinline__ void ld_xrow(const V *__restrict__ x, int64_t j, int64_t ldx, bool vec, V (&out)[K]) {
    const V *p = x + j * ldx;
    if constexpr (K >= 2 && K * sizeof(V) >= 8) {
        if (vec) {
            if constexpr (sizeof(V) == 8) {
#pragma unroll
                for (int h = 0; h < K / 2; h++) {
                    const double2 v = __ldg(reinterpret_cast<const double2 *>(p) + h);
                    out[2 * h] = v.x;
                    out[2 * h + 1] = v.y;
                }
            } else if constexpr (K == 2) {
                const float2 v = __ldg(reinterpret_cast<const float2 *>(p));
                out[0] = v.x;
                out[1] = v.y;
            } else {
#pragma unroll
                for (int h = 0; h < K / 4; h++) {
                    const float4 v = __ldg(reinterpret_cast<const float4 *>(p) + h);
                    out[4 * h] = v.x;
                    out[4 * h + 1] = v.y;
                    out[4 * h + 2] = v.z;
                    out[4 * h + 3] = v.w;
                }
            }
            return;
        }
    }
#pragma unroll
    for (int q = 0; q < K; q++) out[q] = ld_x(p + q);
}

// Whether ld_xrow may use vector loads for X (host side): x and every row
// start aligned to the vector width (16 bytes, 8 for FP32 with k = 2).
inline int xrow_vec(const void *x, int64_t ldx, size_t value_bytes, int k) {
    if (k < 2) return 0;
    const size_t w = k * value_bytes >= 16 ? 16 : k * value_bytes;
    return ((reinterpret_cast<uintptr_t>(x) | (uintptr_t)(ldx * (int64_t)value_bytes)) % w) == 0 ? 1 : 0;
}

template <typename V>
__device__ __forceinline__ V axpby(V alpha, V sum, V beta, const V *y) {
    return beta == V(0) ? alpha * sum : alpha * sum + beta * *y;
}

// A finished row's y value where `plain` (alpha == 1 and beta == 0, the
// reference's "y = sum" case) is known per thread: the sum itself, exactly
// alpha * sum, without the FP64 multiply.  Writes of short rows are spread
// over few lanes of many warp instructions, and GB300's narrow FP64 pipe is
// paid per warp instruction.
template <typename V>
__device__ __forceinline__ V row_out(bool plain, V alpha, V sum, V beta, const V *y) {
    return plain ? sum : axpby(alpha, sum, beta, y);
}

// n / d for n >= 0 and 1 <= d < 2^31, in 32-bit arithmetic whenever n fits
// (row and nonzero indices always do: they are int32).  A 64-bit division by
// a run-time divisor is a long instruction sequence that occupies GB300's
// narrow FP64 pipe (profiled: the pipe busy well beyond a kernel's DFMA and
// DMUL counts), the pipe FP64 SpMV needs for its FMAs.
__device__ __forceinline__ int64_t div_nonneg(int64_t n, int d) {
    return n <= 0x7fffffff ? (int64_t)((unsigned)n / (unsigned)d) : n / d;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v, unsigned width = 32) {
    for (unsigned o = width / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, width);
    return v;
}

// Longest run of consecutive lanes of the warp whose flag is false (all 32
// lanes call it).  A segmented inclusive scan (Kogge-Stone, a flagged lane
// starting a segment) needs only the offsets 1, 2, 4, ... up to this run:
// offsets up to 2^s with 2^(s+1) > run carry a value across run + 1 lanes,
// the most any lane needs (itself, the unflagged lanes before it and the
// flagged lane that starts its segment).  Rows that end every few lanes (a
// few lanes per row) then take two or three scan steps instead of five;
// in FP64 each step is an add on GB300's narrow FP64 pipe.
__device__ __forceinline__ int unflagged_run(bool flag) {
    unsigned z = ~__ballot_sync(0xffffffffu, flag);
    int run = 0;
    while (z) {
        z &= z << 1;
        run++;
    }
    return run;
}

}  // namespace sspmv
