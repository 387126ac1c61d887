// calibrate.cu -- measured ceilings the SpMV kernels are set against: random
// gathers from the x vector, and FP64 FMA throughput.
//
// A third probe times a plain stream of a given read and write volume, the
// speed of light for a kernel of that size in the benchmark's cold-L2 timing.
//
// Measurement probes of the benchmark, not part of the SpMV library: built
// on their own into lib/libsspmv_probe.so (linked against libsspmv.so) and
// loaded only by the benchmark and its tests.
//
// SpMV on matrices whose column indices are spread at random (uniform,
// power-law) is bound by the x gathers, not by HBM: every gathered element
// costs one L1 line lookup (a warp's gather touches 32 distinct lines) and
// one 32-byte L2 sector, while x itself (tens of MB) stays in L2.  This kernel
// runs that access pattern alone -- indices streamed once with evict-first
// loads, 8 read-only gathers in flight per lane, one sum per thread -- so
// a kernel's gather rate can be set against what the GPU delivers for the
// same pattern.  GB300's FP64 rate is low enough (~1 FP64 FMA per 16 bytes of
// HBM bandwidth) that FP64 SpMV, one FMA per nonzero, can be bound by its FMAs
// rather than by its bytes: dfma_kernel measures that rate.
#include "common.cuh"

#include <algorithm>
#include <vector>

namespace sspmv {
namespace {

constexpr int kPerLane = 8;
constexpr int kBlockG = 256;

// Index i of the gather sequence: a 64-bit mix (splitmix64 finaliser) of i,
// reduced to [0, n).
__global__ void gather_indices(int64_t count, int64_t n, uint64_t seed, int32_t *__restrict__ idx) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t z = (uint64_t)i + seed + 0x9E3779B97F4A7C15ull;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        idx[i] = (int32_t)(z % (uint64_t)n);
    }
}

template <typename V>
__global__ void fill_x(int64_t n, V *__restrict__ x) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = V(1) + V(i % 7) * V(0.125);
}

// Warp w takes runs of 256 indices w, w + warps, ...; lane l its 8
// consecutive indices of each run.
template <typename V>
__global__ void __launch_bounds__(kBlockG) gather_kernel(const V *__restrict__ x, const int32_t *__restrict__ idx,
                                                         int64_t runs, V *__restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    V acc = V(0);
    for (int64_t w = w0; w < runs; w += nw) {
        const int4 *ip = reinterpret_cast<const int4 *>(idx + w * 32 * kPerLane + lane * kPerLane);
        const int4 a = ld_stream(ip), b = ld_stream(ip + 1);
        const int c[kPerLane] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
        V v[kPerLane];
#pragma unroll
        for (int u = 0; u < kPerLane; u++) v[u] = ld_x(x + c[u]);
#pragma unroll
        for (int u = 0; u < kPerLane; u++) acc += v[u];
    }
    out[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

// FP64 FMA throughput: eight independent chains per thread, `iters` steps.
__global__ void __launch_bounds__(kBlockG) dfma_kernel(int64_t iters, double b, double c, double *__restrict__ out) {
    double a[8];
#pragma unroll
    for (int u = 0; u < 8; u++) a[u] = 1.0 + 0.125 * u + 1e-3 * (threadIdx.x & 7);
    for (int64_t i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 8; u++) a[u] = fma(a[u], b, c);
    }
    double s = 0.0;
#pragma unroll
    for (int u = 0; u < 8; u++) s += a[u];
    out[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// A size-matched stream: reads nr and writes nw 16-byte words of separate
// buffers, grid-stride (consecutive threads, consecutive words), evict-first
// loads; what DRAM delivers to a kernel of that size and shape.
__global__ void __launch_bounds__(kBlockG) stream_kernel(const float4 *__restrict__ src, int64_t nr,
                                                         float4 *__restrict__ dst, int64_t nw, float *__restrict__ sink) {
    const int64_t n = nr > nw ? nr : nw;
    float acc = 0.f;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 v = i < nr ? ld_stream(src + i) : make_float4(0.f, 0.f, 0.f, 0.f);
        if (i < nw) dst[i] = v;
        else acc += v.x + v.y + v.z + v.w;
    }
    if (acc == 1234.5f) *sink = acc;  // keeps the reads
}

__global__ void flush_read(const float4 *__restrict__ a, int64_t n, float *__restrict__ sink) {
    float acc = 0.f;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 v = a[i];
        acc += v.x + v.y + v.z + v.w;
    }
    if (acc == 1234.5f) *sink = acc;
}

}  // namespace
}  // namespace sspmv

using namespace sspmv;

// Median time of the size-matched stream above, L2 flushed before every run
// the way the benchmark flushes (256 MiB write, then 256 MiB read): the time
// a kernel that only had to move read_bytes in and write_bytes out would
// take, cold, at this size -- short kernels do not reach the bandwidth of a
// multi-gigabyte copy.
extern "C" sspmv_status sspmv_stream_ceiling(int64_t read_bytes, int64_t write_bytes, double *ms_out,
                                             sspmv_stream_t stream) {
    if (!ms_out || read_bytes < 0 || write_bytes < 0 || read_bytes + write_bytes <= 0)
        return fail(SSPMV_INVALID_ARG, "stream ceiling: byte counts >= 0 (not both 0) and an output required");
    const int64_t nr = (read_bytes + 15) / 16, nw = (write_bytes + 15) / 16;
    const size_t kFlush = 256u << 20;
    float4 *src = nullptr, *dst = nullptr, *fr = nullptr;
    unsigned char *fw = nullptr;
    float *sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    std::vector<float> ts;
    auto body = [&]() -> sspmv_status {
        SSPMV_TRY(dalloc(&src, (size_t)std::max<int64_t>(nr, 1), stream));
        SSPMV_TRY(dalloc(&dst, (size_t)std::max<int64_t>(nw, 1), stream));
        SSPMV_TRY(dalloc(&fr, kFlush / 16, stream));
        SSPMV_TRY(dalloc(&fw, kFlush, stream));
        SSPMV_TRY(dalloc(&sink, 1, stream));
        SSPMV_CUDA_TRY(cudaMemsetAsync(src, 0, (size_t)std::max<int64_t>(nr, 1) * 16, cu(stream)));
        SSPMV_CUDA_TRY(cudaMemsetAsync(fr, 0, kFlush, cu(stream)));
        SSPMV_CUDA_TRY(cudaEventCreate(&e0));
        SSPMV_CUDA_TRY(cudaEventCreate(&e1));
        const unsigned grid = (unsigned)(num_sms() * 16);
        for (int rep = 0; rep < 10; rep++) {  // 3 warm-up runs, median of 7 timed
            SSPMV_CUDA_TRY(cudaMemsetAsync(fw, rep & 0xff, kFlush, cu(stream)));
            flush_read<<<(unsigned)(num_sms() * 8), kBlockG, 0, cu(stream)>>>(fr, (int64_t)(kFlush / 16), sink);
            SSPMV_LAUNCH_CHECK();
            SSPMV_CUDA_TRY(cudaEventRecord(e0, cu(stream)));
            stream_kernel<<<grid, kBlockG, 0, cu(stream)>>>(src, nr, dst, nw, sink);
            SSPMV_LAUNCH_CHECK();
            SSPMV_CUDA_TRY(cudaEventRecord(e1, cu(stream)));
            SSPMV_CUDA_TRY(cudaEventSynchronize(e1));
            float ms = 0.f;
            SSPMV_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
            if (rep >= 3) ts.push_back(ms);
        }
        return SSPMV_OK;
    };
    const sspmv_status st = body();
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    dfree(src, stream);
    dfree(dst, stream);
    dfree(fr, stream);
    dfree(fw, stream);
    dfree(sink, stream);
    if (st != SSPMV_OK) return st;
    cudaStreamSynchronize(cu(stream));
    std::sort(ts.begin(), ts.end());
    *ms_out = ts[ts.size() / 2];
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_fp64_ceiling(double *fmas_per_second, sspmv_stream_t stream) {
    if (!fmas_per_second) return fail(SSPMV_INVALID_ARG, "fp64 ceiling: null output");
    const unsigned grid = (unsigned)(num_sms() * 8);
    const int64_t iters = 4096;
    double *out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float best = 0.f;
    auto body = [&]() -> sspmv_status {
        SSPMV_TRY(dalloc(&out, (size_t)grid * kBlockG, stream));
        SSPMV_CUDA_TRY(cudaEventCreate(&e0));
        SSPMV_CUDA_TRY(cudaEventCreate(&e1));
        for (int rep = 0; rep < 8; rep++) {  // 3 warm-up launches, best of 5 timed
            SSPMV_CUDA_TRY(cudaEventRecord(e0, cu(stream)));
            dfma_kernel<<<grid, kBlockG, 0, cu(stream)>>>(iters, 0.999999, 1e-9, out);
            SSPMV_LAUNCH_CHECK();
            SSPMV_CUDA_TRY(cudaEventRecord(e1, cu(stream)));
            SSPMV_CUDA_TRY(cudaEventSynchronize(e1));
            float ms = 0.f;
            SSPMV_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
            if (rep >= 3 && (best == 0.f || ms < best)) best = ms;
        }
        return SSPMV_OK;
    };
    const sspmv_status st = body();
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    dfree(out, stream);
    if (st != SSPMV_OK) return st;
    cudaStreamSynchronize(cu(stream));
    *fmas_per_second = (double)grid * kBlockG * (double)iters * 8.0 / ((double)best * 1e-3);
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_gather_ceiling(int32_t value_type, int64_t num_cols, int64_t num_gathers,
                                             double *gathers_per_second, double *checksum, sspmv_stream_t stream) {
    if (!valid_vt(value_type)) return fail(SSPMV_INVALID_ARG, "unknown value_type %d", value_type);
    if (!gathers_per_second || num_cols <= 0 || num_cols > 0x7fffffff || num_gathers <= 0)
        return fail(SSPMV_INVALID_ARG, "gather ceiling: num_cols in [1, 2^31) and num_gathers > 0 required");
    const int64_t per_run = 32 * kPerLane;
    const int64_t runs = std::max<int64_t>(num_gathers / per_run, 1);
    const int64_t count = runs * per_run;
    const unsigned grid = (unsigned)(num_sms() * 8);  // 8 resident 256-thread CTAs per SM
    int32_t *idx = nullptr;
    void *x = nullptr, *out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    const size_t sv = vsize(value_type);
    sspmv_status st = SSPMV_OK;
    float best = 0.f;
    auto body = [&]() -> sspmv_status {
        SSPMV_TRY(dalloc(&idx, (size_t)count, stream));
        SSPMV_TRY(dalloc((unsigned char **)&x, (size_t)num_cols * sv, stream));
        SSPMV_TRY(dalloc((unsigned char **)&out, (size_t)grid * kBlockG * sv, stream));
        gather_indices<<<grid_for(count, 256, (int64_t)num_sms() * 32), 256, 0, cu(stream)>>>(count, num_cols, 12345,
                                                                                              idx);
        SSPMV_LAUNCH_CHECK();
        SSPMV_CUDA_TRY(cudaEventCreate(&e0));
        SSPMV_CUDA_TRY(cudaEventCreate(&e1));
        return dispatch_value(value_type, [&](auto tag) -> sspmv_status {
            using V = decltype(tag);
            fill_x<V><<<grid_for(num_cols, 256, (int64_t)num_sms() * 32), 256, 0, cu(stream)>>>(num_cols, (V *)x);
            SSPMV_LAUNCH_CHECK();
            for (int rep = 0; rep < 8; rep++) {  // 3 warm-up launches, best of 5 timed
                SSPMV_CUDA_TRY(cudaEventRecord(e0, cu(stream)));
                gather_kernel<V><<<grid, kBlockG, 0, cu(stream)>>>((const V *)x, idx, runs, (V *)out);
                SSPMV_LAUNCH_CHECK();
                SSPMV_CUDA_TRY(cudaEventRecord(e1, cu(stream)));
                SSPMV_CUDA_TRY(cudaEventSynchronize(e1));
                float ms = 0.f;
                SSPMV_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
                if (rep >= 3 && (best == 0.f || ms < best)) best = ms;
            }
            if (checksum) {
                std::vector<V> h((size_t)grid * kBlockG);
                SSPMV_CUDA_TRY(cudaMemcpyAsync(h.data(), out, h.size() * sizeof(V), cudaMemcpyDeviceToHost,
                                               cu(stream)));
                SSPMV_CUDA_TRY(cudaStreamSynchronize(cu(stream)));
                double s = 0;
                for (V v : h) s += (double)v;
                *checksum = s;
            }
            return SSPMV_OK;
        });
    };
    st = body();
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    dfree(idx, stream);
    dfree(x, stream);
    dfree(out, stream);
    if (st != SSPMV_OK) return st;
    cudaStreamSynchronize(cu(stream));
    *gathers_per_second = (double)count / ((double)best * 1e-3);
    return SSPMV_OK;
}
