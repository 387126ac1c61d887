// api_core.cu -- status strings, error text, plan bookkeeping and the CSR
// container entry points (create / wrap / export / delete).
#include <atomic>
#include <cstdarg>
#include <cstring>

#include "common.cuh"
#include "plan.cuh"

namespace sspmv {

static thread_local char g_last_error[1024] = "";
static std::atomic<long long> g_launches{0};

void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

static thread_local int g_delete_nosync = 0;
DeleteWithoutDeviceSync::DeleteWithoutDeviceSync() { g_delete_nosync++; }
DeleteWithoutDeviceSync::~DeleteWithoutDeviceSync() { g_delete_nosync--; }
void delete_barrier() {
    if (g_delete_nosync == 0) cudaDeviceSynchronize();
}

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
}

sspmv_status fail(sspmv_status s, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    return s;
}

PlanMutex &plan_mutex() {
    static PlanMutex m;
    return m;
}

Plan *get_plan(const sspmv_features *f) {
    if (f->priv) return reinterpret_cast<Plan *>(f->priv);
    std::lock_guard<PlanMutex> g(plan_mutex());
    if (!f->priv) const_cast<sspmv_features *>(f)->priv = new (std::nothrow) Plan();
    return reinterpret_cast<Plan *>(f->priv);
}

void free_plan(sspmv_features *f, sspmv_stream_t s) {
    Plan *p = reinterpret_cast<Plan *>(f->priv);
    if (!p) return;
    for (auto &mp : p->merge) {
        dfree(mp.coords, s);
        dfree(mp.carry_row, s);
        dfree(mp.has_end, s);
        dfree(mp.carry_val, s);
        dfree(mp.head_val, s);
    }
    if (p->sub) {
        free_plan(&p->sub->f, s);
        delete p->sub;
    }
    for (void *e : p->extra) dfree(e, s);
    delete p;
    f->priv = nullptr;
}

void init_features(sspmv_features *f, int32_t vt, int64_t m, int64_t n, int64_t nnz, int32_t owns) {
    std::memset(f, 0, sizeof(*f));
    f->num_rows = m;
    f->num_cols = n;
    f->num_nnzs = nnz;
    f->sparsity = (m > 0 && n > 0) ? (double)nnz / ((double)m * (double)n) : 0.0;
    f->value_type = vt;
    f->owns = owns;
}

sspmv_status check_dims(int32_t vt, int64_t m, int64_t n, int64_t nnz) {
    if (!valid_vt(vt)) return fail(SSPMV_INVALID_ARG, "value_type must be SSPMV_F32 or SSPMV_F64");
    if (m < 0 || n < 0 || nnz < 0) return fail(SSPMV_INVALID_ARG, "negative dimension");
    if (m > 0x7fffffff || n > 0x7fffffff || nnz > 0x7fffffff)
        return fail(SSPMV_NOT_SUPPORTED, "int32 index instantiation: dimensions must be < 2^31");
    return SSPMV_OK;
}

}  // namespace sspmv

using namespace sspmv;

extern "C" const char *sspmv_status_string(sspmv_status s) {
    switch (s) {
    case SSPMV_OK: return "SSPMV_OK";
    case SSPMV_INVALID_ARG: return "SSPMV_INVALID_ARG";
    case SSPMV_INFEASIBLE: return "SSPMV_INFEASIBLE";
    case SSPMV_OUT_OF_MEMORY: return "SSPMV_OUT_OF_MEMORY";
    case SSPMV_BUDGET_EXCEEDED: return "SSPMV_BUDGET_EXCEEDED";
    case SSPMV_DEVICE_TIMEOUT: return "SSPMV_DEVICE_TIMEOUT";
    case SSPMV_CUDA_ERROR: return "SSPMV_CUDA_ERROR";
    case SSPMV_NOT_SUPPORTED: return "SSPMV_NOT_SUPPORTED";
    }
    return "SSPMV_UNKNOWN";
}

extern "C" const char *sspmv_last_error(void) { return g_last_error; }

extern "C" const char *sspmv_version(void) { return "sspmv-gb300 0.1 (sm_103a)"; }

extern "C" int64_t sspmv_launch_count(void) { return (int64_t)g_launches.load(); }

extern "C" sspmv_status sspmv_release_plan(sspmv_features *f, sspmv_stream_t s) {
    if (!f) return fail(SSPMV_INVALID_ARG, "null matrix");
    int param = 0;
    if (f->priv) param = reinterpret_cast<Plan *>(f->priv)->param;
    free_plan(f, s);  // f->kernel_flag stays
    if (param != 0) {  // keep the kernel parameter (a host-side record; no device memory)
        Plan *p = get_plan(f);
        if (!p) return fail(SSPMV_OUT_OF_MEMORY, "plan allocation failed");
        p->param = param;
    }
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_set_kernel(sspmv_features *f, int32_t kernel_flag, int32_t param) {
    if (!f) return fail(SSPMV_INVALID_ARG, "null matrix");
    if (kernel_flag < 0 || param < 0) return fail(SSPMV_INVALID_ARG, "negative kernel_flag or param");
    Plan *p = get_plan(f);
    if (!p) return fail(SSPMV_OUT_OF_MEMORY, "plan allocation failed");
    f->kernel_flag = kernel_flag;
    p->param = param;
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_csr_create(sspmv_csr *out, int32_t vt, int64_t m, int64_t n, int64_t nnz,
                                         const int32_t *row_offset, const int32_t *col_index, const void *values,
                                         int32_t from_host, sspmv_stream_t s) {
    if (!out) return fail(SSPMV_INVALID_ARG, "null output");
    SSPMV_TRY(check_dims(vt, m, n, nnz));
    if (!row_offset || (nnz > 0 && (!col_index || !values))) return fail(SSPMV_INVALID_ARG, "null array");
    if (from_host) {
        // Kernels index x by col_index and y by row: reject malformed input
        // before it reaches the device.
        if (row_offset[0] != 0 || row_offset[m] != nnz) return fail(SSPMV_INVALID_ARG, "row_offset[0] != 0 or row_offset[m] != nnz");
        long long bad = 0;
#pragma omp parallel for reduction(+ : bad)
        for (int64_t i = 0; i < m; i++) bad += row_offset[i + 1] < row_offset[i];
#pragma omp parallel for reduction(+ : bad)
        for (int64_t j = 0; j < nnz; j++) bad += (col_index[j] < 0 || col_index[j] >= n);
        if (bad) return fail(SSPMV_INVALID_ARG, "row_offset not monotone or column index out of [0, num_cols)");
    }
    sspmv_csr A;
    init_features(&A.f, vt, m, n, nnz, 1);
    A.row_offset = nullptr;
    A.col_index = nullptr;
    A.values = nullptr;
    const size_t sv = vsize(vt);
    sspmv_status st = dalloc(&A.row_offset, (size_t)m + 1, s);
    if (st == SSPMV_OK) st = dalloc(&A.col_index, (size_t)nnz, s);
    if (st == SSPMV_OK) st = dalloc((unsigned char **)&A.values, (size_t)nnz * sv, s);
    if (st != SSPMV_OK) {
        dfree(A.row_offset, s);
        dfree(A.col_index, s);
        dfree(A.values, s);
        return st;
    }
    cudaMemcpyKind kind = from_host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    cudaError_t e = cudaMemcpyAsync(A.row_offset, row_offset, ((size_t)m + 1) * 4, kind, cu(s));
    if (e == cudaSuccess && nnz > 0) e = cudaMemcpyAsync(A.col_index, col_index, (size_t)nnz * 4, kind, cu(s));
    if (e == cudaSuccess && nnz > 0) e = cudaMemcpyAsync(A.values, values, (size_t)nnz * sv, kind, cu(s));
    if (e == cudaSuccess && from_host) e = cudaStreamSynchronize(cu(s));
    if (e != cudaSuccess) {
        dfree(A.row_offset, s);
        dfree(A.col_index, s);
        dfree(A.values, s);
        return fail(SSPMV_CUDA_ERROR, "csr_create copy: %s", cudaGetErrorString(e));
    }
    *out = A;
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_csr_wrap(sspmv_csr *out, int32_t vt, int64_t m, int64_t n, int64_t nnz,
                                       int32_t *row_offset, int32_t *col_index, void *values) {
    if (!out) return fail(SSPMV_INVALID_ARG, "null output");
    SSPMV_TRY(check_dims(vt, m, n, nnz));
    if (!row_offset || (nnz > 0 && (!col_index || !values))) return fail(SSPMV_INVALID_ARG, "null array");
    init_features(&out->f, vt, m, n, nnz, 0);
    out->row_offset = row_offset;
    out->col_index = col_index;
    out->values = values;
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_csr_export(const sspmv_csr *A, int32_t *row_offset, int32_t *col_index,
                                         void *values, sspmv_stream_t s) {
    if (!A) return fail(SSPMV_INVALID_ARG, "null matrix");
    const int64_t m = A->f.num_rows, nnz = A->f.num_nnzs;
    if (row_offset) SSPMV_CUDA_TRY(cudaMemcpyAsync(row_offset, A->row_offset, (size_t)(m + 1) * 4, cudaMemcpyDeviceToHost, cu(s)));
    if (col_index && nnz) SSPMV_CUDA_TRY(cudaMemcpyAsync(col_index, A->col_index, (size_t)nnz * 4, cudaMemcpyDeviceToHost, cu(s)));
    if (values && nnz) SSPMV_CUDA_TRY(cudaMemcpyAsync(values, A->values, (size_t)nnz * vsize(A->f.value_type), cudaMemcpyDeviceToHost, cu(s)));
    SSPMV_CUDA_TRY(cudaStreamSynchronize(cu(s)));
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_delete_csr(sspmv_csr *A) {
    if (!A) return SSPMV_OK;
    // The matrix may still be in use on any stream: wait for the device
    // before returning its memory.
    delete_barrier();
    free_plan(&A->f, nullptr);
    if (A->f.owns) {
        dfree(A->row_offset, nullptr);
        dfree(A->col_index, nullptr);
        dfree(A->values, nullptr);
    }
    A->row_offset = nullptr;
    A->col_index = nullptr;
    A->values = nullptr;
    A->f.num_rows = A->f.num_cols = A->f.num_nnzs = 0;
    return SSPMV_OK;
}
