// bsr.cu -- BSR format on sm_103a: GPU converter, SpMV / SpMM, export.
//
// Converter (csr_to_bsr, include/sparse_conversion.h:769-926): the distinct
// (block row, block column) pairs of the nonzeros, block columns ascending in
// each block row, blocks stored row-major (r x c) and zero filled.  On the GPU
// every nonzero contributes the key block_row*nb + block_col, the keys are
// radix sorted and made unique, and values are written row by row in CSR
// order (a duplicated (row, col) keeps its last value, as the reference's
// overwrite).  r = c = 1 copies the CSR arrays, as the reference does.
//
// SpMV (LeSpMV_bsr, src/spmv_bsr.cpp:215-233): the block-stream kernel (below)
// for SpMV with r a power of two <= 32 and c <= 16 a power of two; otherwise,
// for SpMM and for kernel_flag 1, one thread per matrix row.  There the r
// threads of a block row read the r consecutive c-wide rows of each block,
// so a block (r*c values) is one contiguous read; x[bc*c .. bc*c+c) is one
// c-wide read shared by the r threads.  Columns past num_cols (the ragged
// last block column) are skipped.
#include <algorithm>
#include <vector>

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

__global__ void bsr_keys(int64_t m, int32_t r, int32_t c, int64_t nb, const int32_t *__restrict__ rp,
                         const int32_t *__restrict__ ci, uint64_t *__restrict__ keys, uint32_t *__restrict__ vals) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t br = (uint64_t)div_nonneg(i, r);
        for (int32_t jj = rp[i]; jj < rp[i + 1]; jj++) {
            keys[jj] = br * (uint64_t)nb + (uint64_t)(ci[jj] / c);
            vals[jj] = (uint32_t)jj;
        }
    }
}

__global__ void unique_flags(int64_t n, const uint64_t *__restrict__ keys, int32_t *__restrict__ flags) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        flags[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1 : 0;
}

__global__ void unique_scatter(int64_t n, const uint64_t *__restrict__ keys, const int32_t *__restrict__ pos,
                               int64_t nb, uint64_t *__restrict__ ukeys, int32_t *__restrict__ bcol) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (i == 0 || keys[i] != keys[i - 1]) {
            ukeys[pos[i]] = keys[i];
            bcol[pos[i]] = (int32_t)(keys[i] % (uint64_t)nb);
        }
}

// row_ptr[b] = first unique block with block row >= b
__global__ void bsr_row_ptr(int64_t mb, int64_t nb, int64_t nnzb, const uint64_t *__restrict__ ukeys,
                            int32_t *__restrict__ row_ptr) {
    for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b <= mb; b += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t key = (uint64_t)b * (uint64_t)nb;
        int64_t lo = 0, hi = nnzb;
        while (lo < hi) {
            int64_t mid = (lo + hi) >> 1;
            if (ukeys[mid] < key) lo = mid + 1;
            else hi = mid;
        }
        row_ptr[b] = (int32_t)lo;
    }
}

template <typename V>
__global__ void bsr_fill(int64_t m, int32_t r, int32_t c, const int32_t *__restrict__ rp, const int32_t *__restrict__ ci,
                         const V *__restrict__ cv, const int32_t *__restrict__ row_ptr, const int32_t *__restrict__ bcol,
                         V *__restrict__ data) {
    const int64_t rc = (int64_t)r * c;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t br = div_nonneg(i, r), q = i - br * r;
        const int32_t b0 = row_ptr[br], b1 = row_ptr[br + 1];
        for (int32_t jj = rp[i]; jj < rp[i + 1]; jj++) {
            const int32_t col = ci[jj], bc = col / c;
            int32_t lo = b0, hi = b1;
            while (lo < hi) {
                int32_t mid = (lo + hi) >> 1;
                if (bcol[mid] < bc) lo = mid + 1;
                else hi = mid;
            }
            data[(int64_t)lo * rc + q * c + (col - bc * c)] = cv[jj];
        }
    }
}

template <typename V, int K, int CB, bool PLAIN = false>
__global__ void __launch_bounds__(kBlock) bsr_spmv_kernel(int m, int n, int r, int cr,
                                                        const int32_t *__restrict__ row_ptr,
                                                        const int32_t *__restrict__ bcol, const V *__restrict__ data,
                                                        const V *__restrict__ x, int64_t ldx, int xvec, V alpha,
                                                        V beta, V *__restrict__ y, int64_t ldy) {
    const int c = CB > 0 ? CB : cr;
    const int64_t rc = (int64_t)r * c;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t br = div_nonneg(i, r), q = i - br * r;
        const int32_t k0 = ld_stream(row_ptr + br), k1 = ld_stream(row_ptr + br + 1);
        V s[K];
#pragma unroll
        for (int t = 0; t < K; t++) s[t] = V(0);
        for (int32_t k = k0; k < k1; k++) {
            const int64_t x0 = (int64_t)ld_x(bcol + k) * c;
            const V *blk = data + k * rc + q * c;
            if (CB > 0 && x0 + c <= n) {
                V a[CB > 0 ? CB : 1];
#pragma unroll
                for (int e = 0; e < (CB > 0 ? CB : 1); e++) a[e] = ld_stream(blk + e);
#pragma unroll
                for (int e = 0; e < (CB > 0 ? CB : 1); e++) {
                    V xr[K];
                    ld_xrow<V, K>(x, x0 + e, ldx, xvec != 0, xr);
#pragma unroll
                    for (int t = 0; t < K; t++) s[t] += a[e] * xr[t];
                }
            } else {
                for (int e = 0; e < c; e++) {
                    if (x0 + e >= n) break;
                    const V a = ld_stream(blk + e);
                    V xr[K];
                    ld_xrow<V, K>(x, x0 + e, ldx, xvec != 0, xr);
#pragma unroll
                    for (int t = 0; t < K; t++) s[t] += a * xr[t];
                }
            }
        }
        V *yp = y + i * ldy;
#pragma unroll
        for (int t = 0; t < K; t++) yp[t] = row_out(PLAIN, alpha, s[t], beta, yp + t);
    }
}

// ------------------------------------------------------- block stream --
// The thread-per-row kernel above leaves lanes idle wherever the block rows of
// a warp hold different numbers of blocks, and GB300's narrow FP64 pipe is
// paid per warp instruction, however few lanes are active (profiled on 4x4
// FP64 blocks, about one block per block row: the pipe 75-84% busy with a
// third of its lanes doing FMAs).  This kernel streams blocks instead: lane
// (g, q), g = lane / r, q = lane % r, multiplies row q of block kb + g by its
// x segment, so each step of G = 32 / r blocks keeps all 32 lanes on FMAs.
// Partial sums of one block row are joined by a segmented scan over the
// groups (lanes q, q + r, q + 2r, ...; block_row[k] keys the segments), and a
// block row running past the step carries into the next step.  Each warp owns
// whole block rows (warp_row[w] .. warp_row[w + 1], cut every `per_warp`
// blocks), so no partial sum leaves its warp: one launch, and the summation
// order is fixed by the matrix alone.  r must be a power of two <= 32.
template <typename V, int CB>
__global__ void __launch_bounds__(kBlock) bsr_stream_kernel(
    int64_t nwarps, int m, int n, int lr, const int32_t *__restrict__ warp_row, const int32_t *__restrict__ row_ptr,
    const int32_t *__restrict__ block_row, const int32_t *__restrict__ bcol, const V *__restrict__ data,
    const V *__restrict__ x, V alpha, V beta, V *__restrict__ y) {
    const int r = 1 << lr, G = 32 >> lr;
    const int lane = threadIdx.x & 31, g = lane >> lr, q = lane & (r - 1);
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (w >= nwarps) return;  // warp-uniform
    const int64_t rc = (int64_t)r * CB;
    const int rb0 = warp_row[w], rb1 = warp_row[w + 1];
    const int k0 = row_ptr[rb0], k1 = row_ptr[rb1];
    V carry = V(0);
    int carry_row = -2;
    const bool plain = alpha == V(1) && beta == V(0);  // y = sum, exactly alpha * sum
    for (int kb = k0; kb < k1; kb += G) {
        const int k = kb + g;
        const bool valid = k < k1;
        const int br = valid ? ld_stream(block_row + k) : -1;
        V s = V(0);
        if (valid) {
            const int64_t x0 = (int64_t)ld_stream(bcol + k) * CB;
            const V *blk = data + (int64_t)k * rc + q * CB;
            if (x0 + CB <= n) {
                V a[CB];
#pragma unroll
                for (int e = 0; e < CB; e++) a[e] = ld_stream(blk + e);
#pragma unroll
                for (int e = 0; e < CB; e++) s += a[e] * ld_x(x + x0 + e);
            } else {
                for (int e = 0; e < CB && x0 + e < n; e++) s += ld_stream(blk + e) * ld_x(x + x0 + e);
            }
        }
        // FP64 adds run on the same narrow pipe as the FMAs: the carry is
        // added only when a row goes on from the previous step, and the scan
        // runs only as deep as the longest segment of this step.
        if (__shfl_sync(0xffffffffu, br, 0) == carry_row) {
            if (g == 0) s += carry;
        }
        const int prev = __shfl_up_sync(0xffffffffu, br, r);
        const unsigned heads = __ballot_sync(0xffffffffu, g == 0 || prev != br);  // lanes of segment heads
        const int head_g = (31 - __clz(heads & (0xffffffffu >> (31 - lane)))) >> lr;
        const int depth = __reduce_max_sync(0xffffffffu, (unsigned)(valid ? g - head_g : 0));
        for (int off = 1; off <= depth; off <<= 1) {  // segmented inclusive scan over g
            const int obr = __shfl_up_sync(0xffffffffu, br, off << lr);
            const V os = __shfl_up_sync(0xffffffffu, s, off << lr);
            if (g >= off && obr == br) s += os;
        }
        int next = __shfl_down_sync(0xffffffffu, br, r);  // block row of block k + 1
        if (g == G - 1) next = (k + 1 < k1) ? ld_stream(block_row + k + 1) : -1;
        if (valid && next != br) {  // last block of row br
            const int64_t row = ((int64_t)br << lr) + q;
            if (row < m) y[row] = row_out(plain, alpha, s, beta, y + row);
        }
        carry_row = __shfl_sync(0xffffffffu, br, (G - 1) << lr);
        carry = __shfl_sync(0xffffffffu, s, ((G - 1) << lr) + q);
    }
    for (int b = rb0 + g; b < rb1; b += G) {  // empty block rows: y = beta * y
        if (ld_stream(row_ptr + b) == ld_stream(row_ptr + b + 1)) {
            const int64_t row = ((int64_t)b << lr) + q;
            if (row < m) y[row] = axpby(alpha, V(0), beta, y + row);
        }
    }
}

__global__ void bsr_block_rows(int64_t mb, const int32_t *__restrict__ row_ptr, int32_t *__restrict__ block_row) {
    for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < mb; b += (int64_t)gridDim.x * blockDim.x)
        for (int32_t k = row_ptr[b]; k < row_ptr[b + 1]; k++) block_row[k] = (int32_t)b;
}

// warp_row[w] = the block row holding block w * per_warp (the last block row
// starting at or before it); warp_row[0] = 0, warp_row[nwarps] = mb.
__global__ void bsr_warp_rows(int64_t nwarps, int64_t mb, int64_t per_warp, const int32_t *__restrict__ row_ptr,
                              int32_t *__restrict__ warp_row) {
    for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w <= nwarps; w += (int64_t)gridDim.x * blockDim.x) {
        if (w == 0 || w == nwarps) {
            warp_row[w] = w == 0 ? 0 : (int32_t)mb;
            continue;
        }
        const int64_t k = w * per_warp;
        int64_t lo = 0, hi = mb - 1;
        while (lo < hi) {
            const int64_t mid = (lo + hi + 1) >> 1;
            if (row_ptr[mid] <= k) lo = mid;
            else hi = mid - 1;
        }
        warp_row[w] = (int32_t)lo;
    }
}

// Lane slots the thread-per-row kernel spends: every warp of 32 rows (32 / r
// block rows) runs as many block iterations as its longest block row.
__global__ void bsr_row_kernel_slots(int64_t mb, int lr, const int32_t *__restrict__ row_ptr,
                                     unsigned long long *__restrict__ slots) {
    const int64_t per = 32 >> lr;
    const int64_t groups = (mb + per - 1) / per;
    unsigned long long acc = 0;
    for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < groups; w += (int64_t)gridDim.x * blockDim.x) {
        int32_t mx = 0;
        const int64_t b1 = min(mb, (w + 1) * per);
        for (int64_t b = w * per; b < b1; b++) mx = max(mx, row_ptr[b + 1] - row_ptr[b]);
        acc += (unsigned long long)mx * (unsigned long long)per;
    }
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0 && acc) atomicAdd(slots, acc);
}

int log2_exact(int64_t v) {
    int l = 0;
    while ((int64_t(1) << l) < v) l++;
    return (int64_t(1) << l) == v ? l : -1;
}

// The block-stream kernel pays a segmented scan per step (about twice the
// FP64 work of a thread whose lanes are all busy, measured); the thread-per-
// row kernel pays for its idle lanes.  The stream kernel is chosen when the
// thread kernel's lane slots exceed the blocks' by this factor.
constexpr double kStreamWaste = 2.0;

// extra_i[2]: 1 = block-stream kernel, 2 = thread-per-row kernel (decided once).
sspmv_status choose_bsr_kernel(const sspmv_bsr *A, Plan *p, sspmv_stream_t s) {
    if (p->extra_i[2]) return SSPMV_OK;
    std::lock_guard<PlanMutex> guard(plan_mutex());
    if (p->extra_i[2]) return SSPMV_OK;
    const int lr = log2_exact(A->blockDim_r);
    unsigned long long *d = nullptr, h = 0;
    SSPMV_TRY(dalloc(&d, 1, s));
    auto body = [&]() -> sspmv_status {
        SSPMV_CUDA_TRY(cudaMemsetAsync(d, 0, sizeof(h), cu(s)));
        const int64_t groups = (A->mb + (32 >> lr) - 1) / (32 >> lr);
        bsr_row_kernel_slots<<<grid_for(groups, 256, (int64_t)num_sms() * 16), 256, 0, cu(s)>>>(A->mb, lr, A->row_ptr,
                                                                                              d);
        SSPMV_LAUNCH_CHECK();
        SSPMV_CUDA_TRY(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, cu(s)));
        SSPMV_CUDA_TRY(cudaStreamSynchronize(cu(s)));
        return SSPMV_OK;
    };
    const sspmv_status st = body();
    dfree(d, s);
    if (st != SSPMV_OK) return st;
    p->extra_i[2] = (double)h > kStreamWaste * (double)A->nnzb ? 1 : 2;
    return SSPMV_OK;
}

// Plan of the block-stream kernel: extra[0] = warp_row, extra[1] = block_row,
// extra_i[0] = warps, extra_i[1] = blocks per warp.
sspmv_status ensure_bsr_stream_plan(const sspmv_bsr *A, Plan *p, sspmv_stream_t s) {
    if (p->extra[0]) return SSPMV_OK;
    std::lock_guard<PlanMutex> guard(plan_mutex());
    if (p->extra[0]) return SSPMV_OK;
    const int lr = log2_exact(A->blockDim_r);
    const int64_t G = 32 >> lr, nnzb = A->nnzb, mb = A->mb;
    // enough warps to fill the GPU (48 per SM), at most 16 steps per warp
    const int64_t steps = std::min<int64_t>(16, std::max<int64_t>(1, nnzb / (G * num_sms() * 48)));
    const int64_t per_warp = G * steps;
    const int64_t nwarps = std::max<int64_t>(1, (nnzb + per_warp - 1) / per_warp);
    int32_t *wr = nullptr, *brow = nullptr;
    SSPMV_TRY(dalloc(&wr, (size_t)nwarps + 1, s));
    sspmv_status st = dalloc(&brow, (size_t)nnzb, s);
    if (st != SSPMV_OK) {
        dfree(wr, s);
        return st;
    }
    bsr_warp_rows<<<grid_for(nwarps + 1, 256, (int64_t)num_sms() * 16), 256, 0, cu(s)>>>(nwarps, mb, per_warp,
                                                                                      A->row_ptr, wr);
    note_launch();
    if (mb > 0) {
        bsr_block_rows<<<grid_for(mb, 256, (int64_t)num_sms() * 16), 256, 0, cu(s)>>>(mb, A->row_ptr, brow);
        note_launch();
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        dfree(wr, s);
        dfree(brow, s);
        return fail(SSPMV_CUDA_ERROR, "bsr plan: %s", cudaGetErrorString(e));
    }
    p->extra_i[0] = nwarps;
    p->extra_i[1] = per_warp;
    p->extra[1] = brow;
    p->extra[0] = wr;  // published last
    return SSPMV_OK;
}

template <typename V, int CB>
sspmv_status launch_bsr_stream(const sspmv_bsr *A, Plan *p, V alpha, const V *x, V beta, V *y, sspmv_stream_t s) {
    SSPMV_TRY(ensure_bsr_stream_plan(A, p, s));
    const int64_t nwarps = p->extra_i[0];
    const unsigned grid = (unsigned)((nwarps * 32 + kBlock - 1) / kBlock);
    bsr_stream_kernel<V, CB><<<grid, kBlock, 0, cu(s)>>>(
        nwarps, (int)A->f.num_rows, (int)A->f.num_cols, log2_exact(A->blockDim_r), (const int32_t *)p->extra[0],
        A->row_ptr, (const int32_t *)p->extra[1], A->block_colindex, (const V *)A->block_data, x, alpha, beta, y);
    SSPMV_LAUNCH_CHECK();
    return SSPMV_OK;
}

// The block-stream kernel takes SpMV (k = 1, unit strides) for r a power of
// two <= 32 and c in {1, 2, 4, 8, 16}: with kernel_flag 2 always, with
// kernel_flag 0 when the block rows are uneven enough (choose_bsr_kernel);
// kernel_flag 1 is the thread-per-row kernel.
template <typename V>
bool try_bsr_stream(const sspmv_bsr *A, V alpha, const V *x, V beta, V *y, sspmv_stream_t s, sspmv_status *st) {
    if (A->f.kernel_flag == 1 || A->nnzb > 0x7fffffff) return false;
    const int lr = log2_exact(A->blockDim_r);
    if (lr < 0 || lr > 5) return false;
    if (A->blockDim_c != 1 && A->blockDim_c != 2 && A->blockDim_c != 4 && A->blockDim_c != 8 && A->blockDim_c != 16)
        return false;
    Plan *p = get_plan(&A->f);
    if (!p) {
        *st = fail(SSPMV_OUT_OF_MEMORY, "plan allocation failed");
        return true;
    }
    if (A->f.kernel_flag != 2) {
        *st = choose_bsr_kernel(A, p, s);
        if (*st != SSPMV_OK) return true;
        if (p->extra_i[2] != 1) return false;
    }
    switch (A->blockDim_c) {
    case 1: *st = launch_bsr_stream<V, 1>(A, p, alpha, x, beta, y, s); return true;
    case 2: *st = launch_bsr_stream<V, 2>(A, p, alpha, x, beta, y, s); return true;
    case 4: *st = launch_bsr_stream<V, 4>(A, p, alpha, x, beta, y, s); return true;
    case 8: *st = launch_bsr_stream<V, 8>(A, p, alpha, x, beta, y, s); return true;
    case 16: *st = launch_bsr_stream<V, 16>(A, p, alpha, x, beta, y, s); return true;
    default: return false;
    }
}

template <typename V, int K, int CB>
sspmv_status launch_bsr_c(const sspmv_bsr *A, V alpha, const V *x, int64_t ldx, V beta, V *y, int64_t ldy,
                          sspmv_stream_t s) {
    const unsigned grid = grid_for(A->f.num_rows, kBlock, (int64_t)num_sms() * 16);
    auto go = [&](auto kernel) {
        kernel<<<grid, kBlock, 0, cu(s)>>>((int)A->f.num_rows, (int)A->f.num_cols, (int)A->blockDim_r,
                                           (int)A->blockDim_c, A->row_ptr, A->block_colindex,
                                           (const V *)A->block_data, x, ldx, xrow_vec(x, ldx, sizeof(V), K), alpha,
                                           beta, y, ldy);
    };
    if (K == 1 && alpha == V(1) && beta == V(0)) go(bsr_spmv_kernel<V, K, CB, K == 1>);  // y = sum
    else go(bsr_spmv_kernel<V, K, CB>);
    SSPMV_LAUNCH_CHECK();
    return SSPMV_OK;
}

template <typename V, int K>
sspmv_status launch_bsr(const sspmv_bsr *A, V alpha, const V *x, int64_t ldx, V beta, V *y, int64_t ldy,
                        sspmv_stream_t s) {
    switch (A->blockDim_c) {
    case 1: return launch_bsr_c<V, K, 1>(A, alpha, x, ldx, beta, y, ldy, s);
    case 2: return launch_bsr_c<V, K, 2>(A, alpha, x, ldx, beta, y, ldy, s);
    case 4: return launch_bsr_c<V, K, 4>(A, alpha, x, ldx, beta, y, ldy, s);
    case 8: return launch_bsr_c<V, K, 8>(A, alpha, x, ldx, beta, y, ldy, s);
    case 16: return launch_bsr_c<V, K, 16>(A, alpha, x, ldx, beta, y, ldy, s);
    default: return launch_bsr_c<V, K, 0>(A, alpha, x, ldx, beta, y, ldy, s);
    }
}

}  // namespace

extern "C" sspmv_status sspmv_csr_to_bsr(const sspmv_csr *csr, int32_t r, int32_t c, sspmv_bsr *out,
                                         sspmv_stream_t s) {
    if (!csr || !out) return fail(SSPMV_INVALID_ARG, "null argument");
    SSPMV_TRY(check_dims(csr->f.value_type, csr->f.num_rows, csr->f.num_cols, csr->f.num_nnzs));
    if (r == 0) r = 16;
    if (c == 0) c = default_alignment(csr->f.value_type);
    if (r < 1 || c < 1) return fail(SSPMV_INVALID_ARG, "block dimensions must be >= 1");
    const int64_t m = csr->f.num_rows, n = csr->f.num_cols, nnz = csr->f.num_nnzs;
    const int32_t vt = csr->f.value_type;
    const size_t sv = vsize(vt);
    sspmv_bsr A;
    init_features(&A.f, vt, m, n, nnz, 1);
    A.blockDim_r = r;
    A.blockDim_c = c;
    A.blockNNZ = (int64_t)r * c;
    A.mb = (m + r - 1) / r;
    A.nb = (n + c - 1) / c;
    A.row_ptr = nullptr;
    A.block_colindex = nullptr;
    A.block_data = nullptr;
    const unsigned g = grid_for(std::max<int64_t>(m, 1), 256, (int64_t)num_sms() * 16);
    sspmv_status st = SSPMV_OK;
    if (r == 1 && c == 1) {  // include/sparse_conversion.h:784-815: copies of the CSR arrays
        A.nnzb = nnz;
        st = dalloc(&A.row_ptr, (size_t)m + 1, s);
        if (st == SSPMV_OK) st = dalloc(&A.block_colindex, (size_t)nnz, s);
        if (st == SSPMV_OK) st = dalloc((unsigned char **)&A.block_data, (size_t)nnz * sv, s);
        if (st == SSPMV_OK) {
            cudaError_t e = cudaMemcpyAsync(A.row_ptr, csr->row_offset, ((size_t)m + 1) * 4, cudaMemcpyDeviceToDevice, cu(s));
            if (e == cudaSuccess && nnz)
                e = cudaMemcpyAsync(A.block_colindex, csr->col_index, (size_t)nnz * 4, cudaMemcpyDeviceToDevice, cu(s));
            if (e == cudaSuccess && nnz)
                e = cudaMemcpyAsync(A.block_data, csr->values, (size_t)nnz * sv, cudaMemcpyDeviceToDevice, cu(s));
            if (e == cudaSuccess) e = cudaStreamSynchronize(cu(s));
            if (e != cudaSuccess) st = fail(SSPMV_CUDA_ERROR, "csr_to_bsr copy: %s", cudaGetErrorString(e));
        }
    } else {
        uint64_t *keys = nullptr, *ukeys = nullptr;
        uint32_t *vals = nullptr;
        int32_t *pos = nullptr;
        int32_t nnzb = 0;
        st = dalloc(&keys, (size_t)nnz, s);
        if (st == SSPMV_OK) st = dalloc(&vals, (size_t)nnz, s);
        if (st == SSPMV_OK) st = dalloc(&pos, (size_t)nnz, s);
        if (st == SSPMV_OK && nnz > 0) {
            bsr_keys<<<g, 256, 0, cu(s)>>>(m, r, c, A.nb, csr->row_offset, csr->col_index, keys, vals);
            note_launch();
            st = radix_sort_pairs(keys, vals, nnz, bits_for((uint64_t)(A.mb * A.nb)), s);
            if (st == SSPMV_OK) {
                unique_flags<<<grid_for(nnz, 256, (int64_t)num_sms() * 16), 256, 0, cu(s)>>>(nnz, keys, pos);
                note_launch();
                st = exclusive_scan_i32(pos, pos, nnz, &nnzb, s);
            }
        }
        A.nnzb = nnzb;
        if (st == SSPMV_OK) st = dalloc(&ukeys, (size_t)nnzb, s);
        if (st == SSPMV_OK) st = dalloc(&A.block_colindex, (size_t)nnzb, s);
        if (st == SSPMV_OK) st = dalloc(&A.row_ptr, (size_t)A.mb + 1, s);
        if (st == SSPMV_OK) st = dalloc((unsigned char **)&A.block_data, (size_t)nnzb * A.blockNNZ * sv, s);
        if (st == SSPMV_OK) {
            cudaMemsetAsync(A.block_data, 0, (size_t)nnzb * A.blockNNZ * sv, cu(s));
            if (nnz > 0) {
                unique_scatter<<<grid_for(nnz, 256, (int64_t)num_sms() * 16), 256, 0, cu(s)>>>(nnz, keys, pos, A.nb,
                                                                                            ukeys, A.block_colindex);
                note_launch();
            }
            bsr_row_ptr<<<grid_for(A.mb + 1, 256), 256, 0, cu(s)>>>(A.mb, A.nb, nnzb, ukeys, A.row_ptr);
            note_launch();
            if (m > 0)
                st = dispatch_value(vt, [&](auto tag) -> sspmv_status {
                    using V = decltype(tag);
                    bsr_fill<V><<<g, 256, 0, cu(s)>>>(m, r, c, csr->row_offset, csr->col_index, (const V *)csr->values,
                                                      A.row_ptr, A.block_colindex, (V *)A.block_data);
                    SSPMV_LAUNCH_CHECK();
                    return SSPMV_OK;
                });
            cudaError_t e = cudaStreamSynchronize(cu(s));
            if (st == SSPMV_OK && e != cudaSuccess) st = fail(SSPMV_CUDA_ERROR, "csr_to_bsr: %s", cudaGetErrorString(e));
        }
        dfree(keys, s);
        dfree(vals, s);
        dfree(pos, s);
        dfree(ukeys, s);
    }
    if (st != SSPMV_OK) {
        dfree(A.row_ptr, s);
        dfree(A.block_colindex, s);
        dfree(A.block_data, s);
        return st;
    }
    *out = A;
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_csr_count_blocks(const sspmv_csr *csr, int32_t r, int32_t c, int64_t *nnzb,
                                               sspmv_stream_t s) {
    if (!csr || !nnzb) return fail(SSPMV_INVALID_ARG, "null argument");
    if (r < 1 || c < 1) return fail(SSPMV_INVALID_ARG, "block dimensions must be >= 1");
    const int64_t m = csr->f.num_rows, n = csr->f.num_cols, nnz = csr->f.num_nnzs;
    *nnzb = 0;
    if (nnz == 0) return SSPMV_OK;
    const int64_t mb = (m + r - 1) / r, nb = (n + c - 1) / c;
    uint64_t *keys = nullptr;
    uint32_t *vals = nullptr;
    int32_t *pos = nullptr;
    sspmv_status st = dalloc(&keys, (size_t)nnz, s);
    if (st == SSPMV_OK) st = dalloc(&vals, (size_t)nnz, s);
    if (st == SSPMV_OK) st = dalloc(&pos, (size_t)nnz, s);
    if (st == SSPMV_OK) {
        bsr_keys<<<grid_for(m, 256, (int64_t)num_sms() * 16), 256, 0, cu(s)>>>(m, r, c, nb, csr->row_offset,
                                                                                csr->col_index, keys, vals);
        note_launch();
        st = radix_sort_pairs(keys, vals, nnz, bits_for((uint64_t)(mb * nb)), s);
    }
    int32_t total = 0;
    if (st == SSPMV_OK) {
        unique_flags<<<grid_for(nnz, 256, (int64_t)num_sms() * 16), 256, 0, cu(s)>>>(nnz, keys, pos);
        note_launch();
        st = exclusive_scan_i32(pos, pos, nnz, &total, s);
    }
    dfree(keys, s);
    dfree(vals, s);
    dfree(pos, s);
    if (st == SSPMV_OK) *nnzb = total;
    return st;
}

extern "C" sspmv_status sspmv_spmm_bsr(double alpha, const sspmv_bsr *A, int32_t k, const void *X, int64_t ldx,
                                       double beta, void *Y, int64_t ldy, sspmv_stream_t s) {
    if (!A) return fail(SSPMV_INVALID_ARG, "null matrix");
    SSPMV_TRY(check_spmm_args(&A->f, k, X, ldx, Y, ldy));
    if (A->f.num_rows == 0) return SSPMV_OK;
    return dispatch_value(A->f.value_type, [&](auto tag) -> sspmv_status {
        using V = decltype(tag);
        return for_rhs_chunks<V>(k, (const V *)X, (V *)Y, [&](int32_t step, const V *xs, V *ys) {
            const V a = (V)alpha, b = (V)beta;
            if (step == 1 && ldx == 1 && ldy == 1) {
                sspmv_status st = SSPMV_OK;
                if (try_bsr_stream<V>(A, a, xs, b, ys, s, &st)) return st;
            }
            switch (step) {
            case 8: return launch_bsr<V, 8>(A, a, xs, ldx, b, ys, ldy, s);
            case 4: return launch_bsr<V, 4>(A, a, xs, ldx, b, ys, ldy, s);
            case 2: return launch_bsr<V, 2>(A, a, xs, ldx, b, ys, ldy, s);
            default: return launch_bsr<V, 1>(A, a, xs, ldx, b, ys, ldy, s);
            }
        });
    });
}

extern "C" sspmv_status sspmv_LeSpMV_bsr(double alpha, const sspmv_bsr *A, const void *x, double beta, void *y,
                                         sspmv_stream_t s) {
    return sspmv_spmm_bsr(alpha, A, 1, x, 1, beta, y, 1, s);
}

extern "C" sspmv_status sspmv_bsr_export(const sspmv_bsr *A, int32_t *row_ptr, int32_t *block_colindex,
                                         void *block_data, sspmv_stream_t s) {
    if (!A) return fail(SSPMV_INVALID_ARG, "null matrix");
    const bool one = A->blockDim_r == 1 && A->blockDim_c == 1;
    const size_t nrp = (size_t)(one ? A->f.num_rows : A->mb) + 1;
    if (row_ptr) SSPMV_CUDA_TRY(cudaMemcpyAsync(row_ptr, A->row_ptr, nrp * 4, cudaMemcpyDeviceToHost, cu(s)));
    if (block_colindex && A->nnzb)
        SSPMV_CUDA_TRY(cudaMemcpyAsync(block_colindex, A->block_colindex, (size_t)A->nnzb * 4, cudaMemcpyDeviceToHost, cu(s)));
    if (block_data && A->nnzb)
        SSPMV_CUDA_TRY(cudaMemcpyAsync(block_data, A->block_data, (size_t)A->nnzb * A->blockNNZ * vsize(A->f.value_type),
                                       cudaMemcpyDeviceToHost, cu(s)));
    SSPMV_CUDA_TRY(cudaStreamSynchronize(cu(s)));
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_delete_bsr(sspmv_bsr *A) {
    if (!A) return SSPMV_OK;
    delete_barrier();
    free_plan(&A->f, nullptr);
    if (A->f.owns) {
        dfree(A->row_ptr, nullptr);
        dfree(A->block_colindex, nullptr);
        dfree(A->block_data, nullptr);
    }
    A->row_ptr = A->block_colindex = nullptr;
    A->block_data = nullptr;
    return SSPMV_OK;
}

extern "C" double sspmv_algorithmic_bytes_bsr(const sspmv_bsr *A, int32_t k, int32_t beta_nonzero) {
    const double sv = (double)vsize(A->f.value_type);
    return (double)A->f.num_nnzs * sv + (double)A->nnzb * 4.0 + (double)(A->mb + 1) * 4.0 +
           (double)k * (double)A->f.num_cols * sv + (double)k * (double)A->f.num_rows * sv * (beta_nonzero ? 2.0 : 1.0);
}
