// mtx_io.cpp -- Matrix Market coordinate reader and writer (host).
//
// Reader semantics follow the reference's read_csr_matrix
// (utils/sparse_io.cpp:27-204, banner parsing utils/mmio.cpp:144-258):
//   - coordinate format; real, integer or pattern (pattern -> 1.0);
//   - 1-based indices converted to 0-based;
//   - values parsed as double and rounded to the value type;
//   - symmetric files: every off-diagonal entry (r,c) is followed by its
//     mirror (c,r) in the expanded triplet list;
//   - CSR built by a stable counting sort on rows (duplicates kept, column
//     order within a row = triplet order), as coo_to_csr
//     (include/sparse_conversion.h:30-91).
// Unlike the reference it returns a status instead of exiting, and does not
// parse inside assert() (so a release build still reads the file).
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "sspmv.h"

namespace sspmv {
sspmv_status fail(sspmv_status s, const char *fmt, ...);
}
using sspmv::fail;

namespace {

struct Triplets {
    int64_t m = 0, n = 0;
    std::vector<int32_t> r, c;
    std::vector<double> v;
};

std::string lower(std::string s) {
    for (auto &ch : s) ch = (char)std::tolower((unsigned char)ch);
    return s;
}

sspmv_status read_triplets(const char *path, Triplets &t) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return fail(SSPMV_INVALID_ARG, "cannot open %s", path);
    std::fseek(f, 0, SEEK_END);
    long sz = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    std::vector<char> buf((size_t)(sz > 0 ? sz : 0) + 1, 0);
    size_t got = std::fread(buf.data(), 1, (size_t)(sz > 0 ? sz : 0), f);
    std::fclose(f);
    buf[got] = 0;
    char *p = buf.data();
    char *end = p + got;

    // banner
    char *eol = (char *)std::memchr(p, '\n', (size_t)(end - p));
    if (!eol) return fail(SSPMV_INVALID_ARG, "%s: missing Matrix Market banner", path);
    std::string banner(p, eol);
    char b0[64] = {0}, b1[64] = {0}, b2[64] = {0}, b3[64] = {0}, b4[64] = {0};
    if (std::sscanf(banner.c_str(), "%63s %63s %63s %63s %63s", b0, b1, b2, b3, b4) != 5 ||
        lower(b0) != "%%matrixmarket")
        return fail(SSPMV_INVALID_ARG, "%s: could not process Matrix Market banner", path);
    std::string obj = lower(b1), fmt = lower(b2), field = lower(b3), sym = lower(b4);
    if (obj != "matrix" || fmt != "coordinate")
        return fail(SSPMV_NOT_SUPPORTED, "%s: only sparse coordinate matrices are supported", path);
    bool pattern = field == "pattern";
    if (!(pattern || field == "real" || field == "integer"))
        return fail(SSPMV_NOT_SUPPORTED, "%s: field '%s' not supported (real, integer, pattern)", path, b3);
    bool symmetric = sym == "symmetric";
    if (!(symmetric || sym == "general"))
        return fail(SSPMV_NOT_SUPPORTED, "%s: symmetry '%s' not supported (general, symmetric)", path, b4);
    p = eol + 1;

    // comments, then the size line
    while (p < end && (*p == '%' || *p == '\n' || *p == '\r')) {
        char *e2 = (char *)std::memchr(p, '\n', (size_t)(end - p));
        p = e2 ? e2 + 1 : end;
    }
    char *q;
    long long m = std::strtoll(p, &q, 10);
    if (q == p) return fail(SSPMV_INVALID_ARG, "%s: bad size line", path);
    p = q;
    long long n = std::strtoll(p, &q, 10);
    if (q == p) return fail(SSPMV_INVALID_ARG, "%s: bad size line", path);
    p = q;
    long long nz = std::strtoll(p, &q, 10);
    if (q == p) return fail(SSPMV_INVALID_ARG, "%s: bad size line", path);
    p = q;
    if (m < 0 || n < 0 || nz < 0 || m > 0x7fffffff || n > 0x7fffffff || nz > 0x3fffffff)
        return fail(SSPMV_NOT_SUPPORTED, "%s: sizes out of int32 range", path);
    t.m = m;
    t.n = n;
    t.r.reserve((size_t)nz * (symmetric ? 2 : 1));
    t.c.reserve((size_t)nz * (symmetric ? 2 : 1));
    t.v.reserve((size_t)nz * (symmetric ? 2 : 1));
    for (long long k = 0; k < nz; k++) {
        long long ri = std::strtoll(p, &q, 10);
        if (q == p) return fail(SSPMV_INVALID_ARG, "%s: entry %lld malformed", path, k + 1);
        p = q;
        long long ci = std::strtoll(p, &q, 10);
        if (q == p) return fail(SSPMV_INVALID_ARG, "%s: entry %lld malformed", path, k + 1);
        p = q;
        double v = 1.0;
        if (!pattern) {
            v = std::strtod(p, &q);
            if (q == p) return fail(SSPMV_INVALID_ARG, "%s: entry %lld malformed", path, k + 1);
            p = q;
        }
        if (ri < 1 || ri > m || ci < 1 || ci > n)
            return fail(SSPMV_INVALID_ARG, "%s: entry %lld index out of range", path, k + 1);
        t.r.push_back((int32_t)(ri - 1));
        t.c.push_back((int32_t)(ci - 1));
        t.v.push_back(v);
        if (symmetric && ri != ci) {
            t.r.push_back((int32_t)(ci - 1));
            t.c.push_back((int32_t)(ri - 1));
            t.v.push_back(v);
        }
    }
    if (t.r.size() > 0x7fffffffull) return fail(SSPMV_NOT_SUPPORTED, "%s: too many entries", path);
    return SSPMV_OK;
}

}  // namespace

extern "C" sspmv_status sspmv_read_mtx(const char *path, int32_t value_type, int64_t *num_rows, int64_t *num_cols,
                                       int64_t *num_nnzs, int32_t *row_offset, int32_t *col_index, void *values) {
    if (!path || !num_rows || !num_cols || !num_nnzs) return fail(SSPMV_INVALID_ARG, "null argument");
    if (value_type != SSPMV_F32 && value_type != SSPMV_F64) return fail(SSPMV_INVALID_ARG, "bad value_type");
    Triplets t;
    sspmv_status st = read_triplets(path, t);
    if (st != SSPMV_OK) return st;
    const int64_t nnz = (int64_t)t.r.size();
    *num_rows = t.m;
    *num_cols = t.n;
    *num_nnzs = nnz;
    if (!row_offset) return SSPMV_OK;  // size query
    if (nnz > 0 && (!col_index || !values)) return fail(SSPMV_INVALID_ARG, "null output array");
    // stable counting sort by row
    std::vector<int64_t> cnt((size_t)t.m + 1, 0);
    for (int32_t r : t.r) cnt[(size_t)r + 1]++;
    for (int64_t i = 0; i < t.m; i++) cnt[(size_t)i + 1] += cnt[(size_t)i];
    for (int64_t i = 0; i <= t.m; i++) row_offset[i] = (int32_t)cnt[(size_t)i];
    for (int64_t k = 0; k < nnz; k++) {
        int64_t d = cnt[(size_t)t.r[(size_t)k]]++;
        col_index[d] = t.c[(size_t)k];
        if (value_type == SSPMV_F64) ((double *)values)[d] = t.v[(size_t)k];
        else ((float *)values)[d] = (float)t.v[(size_t)k];
    }
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_read_mtx_coo(const char *path, int32_t value_type, int64_t *num_rows,
                                           int64_t *num_cols, int64_t *num_nnzs, int32_t *row_index,
                                           int32_t *col_index, void *values) {
    if (!path || !num_rows || !num_cols || !num_nnzs) return fail(SSPMV_INVALID_ARG, "null argument");
    if (value_type != SSPMV_F32 && value_type != SSPMV_F64) return fail(SSPMV_INVALID_ARG, "bad value_type");
    Triplets t;
    sspmv_status st = read_triplets(path, t);
    if (st != SSPMV_OK) return st;
    const int64_t nnz = (int64_t)t.r.size();
    *num_rows = t.m;
    *num_cols = t.n;
    *num_nnzs = nnz;
    if (!row_index) return SSPMV_OK;  // size query
    if (nnz > 0 && (!col_index || !values)) return fail(SSPMV_INVALID_ARG, "null output array");
    for (int64_t k = 0; k < nnz; k++) {  // file order, mirrors right after their entries
        row_index[k] = t.r[(size_t)k];
        col_index[k] = t.c[(size_t)k];
        if (value_type == SSPMV_F64) ((double *)values)[k] = t.v[(size_t)k];
        else ((float *)values)[k] = (float)t.v[(size_t)k];
    }
    return SSPMV_OK;
}

// sum_csr_duplicates (include/sparse_operation.h:22-73), the compact step of
// coo_to_csr (include/sparse_conversion.h:82-87): per row, entries of equal
// column summed; the row's columns come out in the reverse order of their
// first appearance (the reference chains them head-first) and sums equal to
// zero are dropped.  In place on host arrays; row_offset is rewritten.
template <typename V>
static void sum_duplicates(int64_t m, int64_t n, int32_t *rp, int32_t *ci, V *cv) {
    std::vector<int32_t> next((size_t)n, -1);
    std::vector<V> sums((size_t)n, V(0));
    int64_t nnz = 0, row_end = 0;
    for (int64_t i = 0; i < m; i++) {
        int32_t head = -2;
        const int64_t row_start = row_end;
        row_end = rp[i + 1];
        for (int64_t jj = row_start; jj < row_end; jj++) {
            const int32_t j = ci[jj];
            sums[(size_t)j] += cv[jj];
            if (next[(size_t)j] == -1) {
                next[(size_t)j] = head;
                head = j;
            }
        }
        while (head != -2) {
            const int32_t cur = head;
            head = next[(size_t)cur];
            if (sums[(size_t)cur] != V(0)) {
                ci[nnz] = cur;
                cv[nnz] = sums[(size_t)cur];
                nnz++;
            }
            next[(size_t)cur] = -1;
            sums[(size_t)cur] = V(0);
        }
        rp[i + 1] = (int32_t)nnz;
    }
}

extern "C" sspmv_status sspmv_sum_csr_duplicates(int32_t value_type, int64_t num_rows, int64_t num_cols,
                                                 int32_t *row_offset, int32_t *col_index, void *values,
                                                 int64_t *num_nnzs) {
    if (!row_offset || num_rows < 0 || num_cols < 0) return fail(SSPMV_INVALID_ARG, "bad arguments");
    if (row_offset[num_rows] > 0 && (!col_index || !values)) return fail(SSPMV_INVALID_ARG, "null array");
    for (int64_t k = 0; k < row_offset[num_rows]; k++)
        if (col_index[k] < 0 || col_index[k] >= num_cols) return fail(SSPMV_INVALID_ARG, "column out of range");
    if (value_type == SSPMV_F64) sum_duplicates(num_rows, num_cols, row_offset, col_index, (double *)values);
    else if (value_type == SSPMV_F32) sum_duplicates(num_rows, num_cols, row_offset, col_index, (float *)values);
    else return fail(SSPMV_INVALID_ARG, "bad value_type");
    if (num_nnzs) *num_nnzs = row_offset[num_rows];
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_write_mtx(const char *path, int64_t num_rows, int64_t num_cols,
                                        const int32_t *row_offset, const int32_t *col_index, const double *values) {
    if (!path || !row_offset) return fail(SSPMV_INVALID_ARG, "null argument");
    FILE *f = std::fopen(path, "wb");
    if (!f) return fail(SSPMV_INVALID_ARG, "cannot create %s", path);
    const int64_t nnz = row_offset[num_rows];
    std::fprintf(f, "%%%%MatrixMarket matrix coordinate real general\n");
    std::fprintf(f, "%lld %lld %lld\n", (long long)num_rows, (long long)num_cols, (long long)nnz);
    for (int64_t i = 0; i < num_rows; i++)
        for (int32_t j = row_offset[i]; j < row_offset[i + 1]; j++)
            std::fprintf(f, "%lld %d %.17g\n", (long long)i + 1, col_index[j] + 1, values[j]);
    if (std::fclose(f) != 0) return fail(SSPMV_INVALID_ARG, "write failed: %s", path);
    return SSPMV_OK;
}
