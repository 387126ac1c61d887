// bytes_model.cu -- the reference benchmark's byte count per SpMV
// (include/spmv_benchmark.h:26-150, bytes_per_spmv), the numerator of the
// GB/s that its benchmark programs print (src/spmv_benchmark.cpp:68).
//
// That model differs from sspmv_algorithmic_bytes_<fmt> (structural bytes
// without padding, x once, y once) in several ways, each kept here as the
// reference has it: x is charged once per nonzero (a gather, not a read of
// the vector), y twice per row, CSR / BSR / CSR5 charge two row-pointer reads
// per row, ELL and the sliced formats charge their padded slots, the sliced
// formats charge values at sizeof(IndexType) (4 bytes, also for FP64), COO
// charges y only for rows that hold a nonzero, and DIA charges its nonzeros
// and rows only.  Index and UIndexType are 4-byte here, as in the reference's
// int build.
#include "common.cuh"

#include <algorithm>

namespace sspmv {
namespace {

constexpr double kIdx = 4.0;  // sizeof(IndexType) == sizeof(UIndexType)

__global__ void mark_rows(int64_t nnz, const int32_t *__restrict__ ri, int64_t m, uint8_t *__restrict__ flag) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t r = ri[i];
        if (r >= 0 && r < m) flag[r] = 1;
    }
}

__global__ void count_flags(int64_t m, const uint8_t *__restrict__ flag, unsigned long long *__restrict__ count) {
    unsigned long long c = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        c += flag[i];
    c = warp_sum(c);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

// Rows of the COO matrix that hold at least one nonzero (one pass over
// row_index; the matrix may be unsorted).
sspmv_status occupied_rows(const sspmv_coo *A, int64_t *out) {
    const int64_t m = A->f.num_rows, nnz = A->f.num_nnzs;
    *out = 0;
    if (m == 0 || nnz == 0) return SSPMV_OK;
    cudaStream_t s = nullptr;
    uint8_t *flag = nullptr;
    unsigned long long *cnt = nullptr;
    auto body = [&]() -> sspmv_status {
        SSPMV_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        const sspmv_stream_t ss = reinterpret_cast<sspmv_stream_t>(s);
        SSPMV_TRY(dalloc(&flag, (size_t)m, ss));
        SSPMV_TRY(dalloc(&cnt, 1, ss));
        SSPMV_CUDA_TRY(cudaMemsetAsync(flag, 0, (size_t)m, s));
        SSPMV_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), s));
        mark_rows<<<grid_for(nnz, 256, (int64_t)num_sms() * 16), 256, 0, s>>>(nnz, A->row_index, m, flag);
        SSPMV_LAUNCH_CHECK();
        count_flags<<<grid_for(m, 256, (int64_t)num_sms() * 16), 256, 0, s>>>(m, flag, cnt);
        SSPMV_LAUNCH_CHECK();
        unsigned long long h = 0;
        SSPMV_CUDA_TRY(cudaMemcpyAsync(&h, cnt, sizeof(h), cudaMemcpyDeviceToHost, s));
        SSPMV_CUDA_TRY(cudaStreamSynchronize(s));
        *out = (int64_t)h;
        return SSPMV_OK;
    };
    const sspmv_status st = body();
    if (s) {
        dfree(flag, reinterpret_cast<sspmv_stream_t>(s));
        dfree(cnt, reinterpret_cast<sspmv_stream_t>(s));
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
    }
    return st;
}

double sv_of(const sspmv_features &f) { return (double)vsize(f.value_type); }

}  // namespace
}  // namespace sspmv

using namespace sspmv;

extern "C" double sspmv_reference_bytes_coo(const sspmv_coo *A) {
    if (!A || !valid_vt(A->f.value_type)) return -1.0;
    int64_t occ = 0;
    if (occupied_rows(A, &occ) != SSPMV_OK) return -1.0;
    const double sv = sv_of(A->f), nnz = (double)A->f.num_nnzs;
    return 2 * kIdx * nnz + 2 * sv * nnz + 2 * sv * (double)occ;
}

extern "C" double sspmv_reference_bytes_csr(const sspmv_csr *A) {
    if (!A || !valid_vt(A->f.value_type)) return -1.0;
    const double sv = sv_of(A->f), m = (double)A->f.num_rows, nnz = (double)A->f.num_nnzs;
    return 2 * kIdx * m + kIdx * nnz + 2 * sv * nnz + 2 * sv * m;
}

extern "C" double sspmv_reference_bytes_bsr(const sspmv_bsr *A) {
    if (!A || !valid_vt(A->f.value_type)) return -1.0;
    const double sv = sv_of(A->f), nnzb = (double)A->nnzb;
    return 2 * kIdx * (double)A->mb + kIdx * nnzb + 2 * sv * nnzb * (double)A->blockDim_r * (double)A->blockDim_c +
           2 * sv * (double)A->f.num_rows;
}

extern "C" double sspmv_reference_bytes_csr5(const sspmv_csr5 *A) {
    if (!A || !valid_vt(A->f.value_type)) return -1.0;
    const double sv = sv_of(A->f), m = (double)A->f.num_rows, nnz = (double)A->f.num_nnzs;
    return 2 * kIdx * m + kIdx * nnz + 2 * sv * nnz + 2 * sv * m + kIdx * (double)A->_p + kIdx;
}

extern "C" double sspmv_reference_bytes_ell(const sspmv_ell *A) {
    if (!A || !valid_vt(A->f.value_type)) return -1.0;
    const double sv = sv_of(A->f), m = (double)A->f.num_rows;
    const double slots = m * (double)A->max_row_width;
    return kIdx * slots + sv * slots + sv * (double)A->f.num_nnzs + 2 * sv * m;
}

extern "C" double sspmv_reference_bytes_sell(const sspmv_s_ell *A) {
    if (!A || !valid_vt(A->f.value_type)) return -1.0;
    const double sv = sv_of(A->f);
    return kIdx * (double)A->chunk_num + 2 * kIdx * (double)A->total_slots + sv * (double)A->f.num_nnzs +
           2 * sv * (double)A->f.num_rows;
}

extern "C" double sspmv_reference_bytes_sell_c_sigma(const sspmv_sell_c_sigma *A) {
    if (!A || !valid_vt(A->f.value_type)) return -1.0;
    const double sv = sv_of(A->f), m = (double)A->f.num_rows;
    return kIdx * (double)A->validchunkNum + kIdx * m + 2 * kIdx * (double)A->total_slots +
           sv * (double)A->f.num_nnzs + 2 * sv * m;
}

extern "C" double sspmv_reference_bytes_sell_c_R(const sspmv_sell_c_R *A) {
    if (!A || !valid_vt(A->f.value_type)) return -1.0;
    const double sv = sv_of(A->f), m = (double)A->f.num_rows;
    return kIdx * (double)A->validchunkNum + kIdx * m + 2 * kIdx * (double)A->total_slots +
           sv * (double)A->f.num_nnzs + 2 * sv * m;
}

extern "C" double sspmv_reference_bytes_dia(const sspmv_dia *A) {
    if (!A || !valid_vt(A->f.value_type)) return -1.0;
    const double sv = sv_of(A->f);
    return 2 * sv * (double)A->f.num_nnzs + 2 * sv * (double)A->f.num_rows;
}
