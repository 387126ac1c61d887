// primitives.cu -- exclusive scan, stable LSD radix sort, row-length max.
#include "primitives.cuh"

namespace sspmv {
namespace {

constexpr int kScanBlock = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanBlock * kScanItems;

template <typename T>
__device__ T block_exclusive_scan(T v, T *s_warp, T *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        T w = lane < kScanBlock / 32 ? s_warp[lane] : T(0);
        T wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            T t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += t;
        }
        if (lane < kScanBlock / 32) s_warp[lane] = wi - w;
        if (lane == kScanBlock / 32 - 1) s_warp[kScanBlock / 32] = wi;
    }
    __syncthreads();
    T r = s_warp[warp] + inc - v;
    if (total) *total = s_warp[kScanBlock / 32];
    __syncthreads();
    return r;
}

template <typename T>
__global__ void __launch_bounds__(kScanBlock) scan_reduce(const T *__restrict__ in, int64_t n, T *__restrict__ partial) {
    __shared__ T s_warp[kScanBlock / 32 + 1];
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    T sum = 0;
#pragma unroll
    for (int u = 0; u < kScanItems; u++)
        if (base + u < n) sum += in[base + u];
    T total;
    block_exclusive_scan(sum, s_warp, &total);
    if (threadIdx.x == 0) partial[blockIdx.x] = total;
}

template <typename T>
__global__ void __launch_bounds__(kScanBlock) scan_apply(const T *in, T *out, int64_t n, const T *__restrict__ offs) {
    __shared__ T s_warp[kScanBlock / 32 + 1];
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    T v[kScanItems];
    T sum = 0;
#pragma unroll
    for (int u = 0; u < kScanItems; u++) {
        v[u] = base + u < n ? in[base + u] : T(0);
        sum += v[u];
    }
    T run = block_exclusive_scan(sum, s_warp, (T *)nullptr) + (offs ? offs[blockIdx.x] : T(0));
#pragma unroll
    for (int u = 0; u < kScanItems; u++) {
        if (base + u < n) out[base + u] = run;
        run += v[u];
    }
}

template <typename T>
sspmv_status scan_rec(const T *in, T *out, int64_t n, sspmv_stream_t s) {
    if (n <= 0) return SSPMV_OK;
    const int64_t nb = (n + kScanTile - 1) / kScanTile;
    if (nb == 1) {
        scan_apply<T><<<1, kScanBlock, 0, cu(s)>>>(in, out, n, nullptr);
        SSPMV_LAUNCH_CHECK();
        return SSPMV_OK;
    }
    T *partial = nullptr;
    SSPMV_TRY(dalloc(&partial, (size_t)nb, s));
    scan_reduce<T><<<(unsigned)nb, kScanBlock, 0, cu(s)>>>(in, n, partial);
    sspmv_status st = SSPMV_OK;
    if (cudaGetLastError() != cudaSuccess) st = fail(SSPMV_CUDA_ERROR, "scan_reduce launch failed");
    note_launch();
    if (st == SSPMV_OK) st = scan_rec<T>(partial, partial, nb, s);
    if (st == SSPMV_OK) {
        scan_apply<T><<<(unsigned)nb, kScanBlock, 0, cu(s)>>>(in, out, n, partial);
        note_launch();
        if (cudaGetLastError() != cudaSuccess) st = fail(SSPMV_CUDA_ERROR, "scan_apply launch failed");
    }
    dfree(partial, s);
    return st;
}

template <typename T>
sspmv_status exclusive_scan(const T *in, T *out, int64_t n, T *h_total, sspmv_stream_t s) {
    T last_in = 0;
    if (h_total && n > 0)  // the last input is needed after an in-place scan
        SSPMV_CUDA_TRY(cudaMemcpyAsync(&last_in, in + n - 1, sizeof(T), cudaMemcpyDeviceToHost, cu(s)));
    SSPMV_TRY(scan_rec<T>(in, out, n, s));
    if (h_total) {
        T last_out = 0;
        if (n > 0) SSPMV_CUDA_TRY(cudaMemcpyAsync(&last_out, out + n - 1, sizeof(T), cudaMemcpyDeviceToHost, cu(s)));
        SSPMV_CUDA_TRY(cudaStreamSynchronize(cu(s)));
        *h_total = n > 0 ? last_out + last_in : T(0);
    }
    return SSPMV_OK;
}

// ------------------------------------------------------------ radix sort --
constexpr int kSortBlock = 256;
constexpr int kSortRounds = 16;
constexpr int kSortTile = kSortBlock * kSortRounds;  // 4096 keys per CTA
constexpr int kSortWarps = kSortBlock / 32;

__global__ void __launch_bounds__(kSortBlock) radix_hist(const uint64_t *__restrict__ keys, int64_t n, int shift,
                                                       int32_t *__restrict__ hist, int64_t ntiles) {
    __shared__ int32_t sh[256];
    sh[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kSortTile;
    for (int r = 0; r < kSortRounds; r++) {
        int64_t i = base + (int64_t)r * kSortBlock + threadIdx.x;
        if (i < n) atomicAdd(&sh[(keys[i] >> shift) & 0xff], 1);
    }
    __syncthreads();
    hist[(int64_t)threadIdx.x * ntiles + blockIdx.x] = sh[threadIdx.x];
}

// Stable scatter: within a tile, keys keep their order (round, warp, lane).
__global__ void __launch_bounds__(kSortBlock) radix_scatter(const uint64_t *__restrict__ kin,
                                                          const uint32_t *__restrict__ vin, uint64_t *__restrict__ kout,
                                                          uint32_t *__restrict__ vout, int64_t n, int shift,
                                                          const int32_t *__restrict__ hist, int64_t ntiles) {
    __shared__ int32_t s_off[256];      // global position of the next key of digit d
    __shared__ int32_t s_cnt[kSortWarps][256];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    s_off[threadIdx.x] = hist[(int64_t)threadIdx.x * ntiles + blockIdx.x];
    const int64_t base = (int64_t)blockIdx.x * kSortTile;
    const unsigned lt_mask = (1u << lane) - 1u;
    for (int r = 0; r < kSortRounds; r++) {
#pragma unroll
        for (int w = 0; w < kSortWarps; w++) s_cnt[w][threadIdx.x] = 0;
        __syncthreads();
        const int64_t i = base + (int64_t)r * kSortBlock + threadIdx.x;
        const bool valid = i < n;
        uint64_t k = valid ? kin[i] : 0;
        uint32_t v = valid ? vin[i] : 0;
        const int d = valid ? (int)((k >> shift) & 0xff) : 256;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int rank = __popc(peers & lt_mask);
        const int leader = __ffs(peers) - 1;
        if (valid && lane == leader) s_cnt[warp][d] = __popc(peers);
        __syncthreads();
        int pos = 0;
        if (valid) {
            int before = 0;
            for (int w = 0; w < warp; w++) before += s_cnt[w][d];
            pos = s_off[d] + before + rank;
        }
        __syncthreads();
        {
            int tot = 0;
#pragma unroll
            for (int w = 0; w < kSortWarps; w++) tot += s_cnt[w][threadIdx.x];
            s_off[threadIdx.x] += tot;
        }
        if (valid) {
            kout[pos] = k;
            vout[pos] = v;
        }
        __syncthreads();
    }
}

__global__ void row_len_max(const int32_t *__restrict__ rp, int64_t m, int32_t *out) {
    int32_t best = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        best = max(best, rp[i + 1] - rp[i]);
    for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, best);
}

}  // namespace

sspmv_status exclusive_scan_i64(const int64_t *in, int64_t *out, int64_t n, int64_t *h_total, sspmv_stream_t s) {
    return exclusive_scan<int64_t>(in, out, n, h_total, s);
}
sspmv_status exclusive_scan_i32(const int32_t *in, int32_t *out, int64_t n, int32_t *h_total, sspmv_stream_t s) {
    return exclusive_scan<int32_t>(in, out, n, h_total, s);
}

sspmv_status radix_sort_pairs(uint64_t *keys, uint32_t *vals, int64_t n, int end_bit, sspmv_stream_t s) {
    if (n <= 1 || end_bit <= 0) return SSPMV_OK;
    const int64_t ntiles = (n + kSortTile - 1) / kSortTile;
    uint64_t *k2 = nullptr;
    uint32_t *v2 = nullptr;
    int32_t *hist = nullptr;
    sspmv_status st = dalloc(&k2, (size_t)n, s);
    if (st == SSPMV_OK) st = dalloc(&v2, (size_t)n, s);
    if (st == SSPMV_OK) st = dalloc(&hist, (size_t)ntiles * 256, s);
    uint64_t *ka = keys, *kb = k2;
    uint32_t *va = vals, *vb = v2;
    for (int shift = 0; st == SSPMV_OK && shift < end_bit; shift += 8) {
        radix_hist<<<(unsigned)ntiles, kSortBlock, 0, cu(s)>>>(ka, n, shift, hist, ntiles);
        note_launch();
        if (cudaGetLastError() != cudaSuccess) { st = fail(SSPMV_CUDA_ERROR, "radix_hist launch failed"); break; }
        st = exclusive_scan_i32(hist, hist, ntiles * 256, nullptr, s);
        if (st != SSPMV_OK) break;
        radix_scatter<<<(unsigned)ntiles, kSortBlock, 0, cu(s)>>>(ka, va, kb, vb, n, shift, hist, ntiles);
        note_launch();
        if (cudaGetLastError() != cudaSuccess) { st = fail(SSPMV_CUDA_ERROR, "radix_scatter launch failed"); break; }
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    if (st == SSPMV_OK && ka != keys) {
        cudaError_t e = cudaMemcpyAsync(keys, ka, (size_t)n * 8, cudaMemcpyDeviceToDevice, cu(s));
        if (e == cudaSuccess) e = cudaMemcpyAsync(vals, va, (size_t)n * 4, cudaMemcpyDeviceToDevice, cu(s));
        if (e != cudaSuccess) st = fail(SSPMV_CUDA_ERROR, "radix copy back: %s", cudaGetErrorString(e));
    }
    dfree(k2, s);
    dfree(v2, s);
    dfree(hist, s);
    return st;
}

sspmv_status max_row_length(const int32_t *row_offset, int64_t m, int32_t *h_max, sspmv_stream_t s) {
    *h_max = 0;
    if (m <= 0) return SSPMV_OK;
    int32_t *d = nullptr;
    SSPMV_TRY(dalloc(&d, 1, s));
    cudaMemsetAsync(d, 0, 4, cu(s));
    row_len_max<<<grid_for(m, 256, (int64_t)num_sms() * 8), 256, 0, cu(s)>>>(row_offset, m, d);
    note_launch();
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_max, d, 4, cudaMemcpyDeviceToHost, cu(s));
    if (e == cudaSuccess) e = cudaStreamSynchronize(cu(s));
    dfree(d, s);
    if (e != cudaSuccess) return fail(SSPMV_CUDA_ERROR, "max_row_length: %s", cudaGetErrorString(e));
    return SSPMV_OK;
}

}  // namespace sspmv
