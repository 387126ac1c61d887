// features.cu -- matrix feature extraction on the GPU.
//
// Replaces the reference's MTX class (src/sparse_features.cpp:122-968:
// MtxLoad, CalculateFeatures, CalculateTilesFeatures, P_ratioAndGini,
// CalculateTilesExtraFeatures) for a general CSR matrix already on the device.
// The reference parses the Matrix Market file and keeps N x T count tables
// (Rows_cnt / Cols_cnt, 2 GB each at N = 2M, T = 256); here:
//   - one pass over the rows counts per column, per diagonal, per T x T tile
//     (block-local histograms for the T row and column blocks), and gathers
//     each row's triangle counts, diagonal dominance, log10 value range and
//     column-step distance;
//   - distinct (row, tile column) and (column, tile row) pairs -- the
//     reference's uniq_RB / uniq_CB, kept with flag tables -- come from a
//     radix sort of 64-bit keys;
//   - P-ratio and Gini of a count vector come from its sorted copy: the
//     trapezoid area is sum_k o_k (L - k) - nnz/2 in exact integers, the
//     P-ratio is the smallest top fraction p with p + share >= 1;
//   - pattern symmetry looks every (i, j) up as (j, i) in the sorted keys.
// Integer counts are exact; floating features are computed in double.  The
// reference's quirks are kept: accumulators of t_var_* and t_nz_ratio_* start
// at -1, the tile grid gives the first T_mod blocks one extra row, a row's
// log10 minimum starts at 0.  Values are compared exactly for value symmetry
// (the reference compares "%lf" strings).  GrX features are -1, as the
// reference leaves them (its BSR_ANA block does not build).
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "primitives.cuh"

namespace sspmv {
sspmv_status check_dims(int32_t vt, int64_t m, int64_t n, int64_t nnz);
}

using namespace sspmv;

namespace {

constexpr int kBlock = 256;
constexpr int kMaxSmemBlocks = 4096;  // RB/CB histograms kept in shared memory up to this T

struct TileMap {
    int64_t T, tn_rb, tm_rb, tn_cb, tm_cb;
    __host__ __device__ int64_t row_tile(int64_t i) const {
        const int64_t thr = tm_rb * (tn_rb + 1);
        return i < thr ? i / (tn_rb + 1) : tm_rb + (tn_rb ? (i - thr) / tn_rb : 0);
    }
    __host__ __device__ int64_t col_tile(int64_t j) const {
        const int64_t thr = tm_cb * (tn_cb + 1);
        return j < thr ? j / (tn_cb + 1) : tm_cb + (tn_cb ? (j - thr) / tn_cb : 0);
    }
};

struct RowPartial {
    long long lower, upper, ondiag, dominance, nz_rows;
    double max_off, max_diag, row_div, dist;
};

__device__ void atomic_max_double(double *addr, double v) {
    unsigned long long *p = (unsigned long long *)addr, old = *p, assumed;
    while (__longlong_as_double(old) < v) {
        assumed = old;
        old = atomicCAS(p, assumed, (unsigned long long)__double_as_longlong(v));
        if (old == assumed) break;
    }
}

__device__ void atomic_min_double(double *addr, double v) {
    unsigned long long *p = (unsigned long long *)addr, old = *p, assumed;
    while (__longlong_as_double(old) > v) {
        assumed = old;
        old = atomicCAS(p, assumed, (unsigned long long)__double_as_longlong(v));
        if (old == assumed) break;
    }
}

template <typename V>
__global__ void __launch_bounds__(kBlock) feat_rows(int64_t m, TileMap tm, const int32_t *__restrict__ rp,
                                                  const int32_t *__restrict__ ci, const V *__restrict__ cv,
                                                  int32_t *__restrict__ col_cnt, int32_t *__restrict__ diag_cnt,
                                                  int32_t *__restrict__ tiles, int32_t *__restrict__ rb,
                                                  int32_t *__restrict__ cb, double *__restrict__ maxc,
                                                  double *__restrict__ minc, RowPartial *__restrict__ part) {
    extern __shared__ int32_t s_hist[];  // [T] row blocks, [T] column blocks
    const int64_t T = tm.T;
    const bool smem = T <= kMaxSmemBlocks;
    if (smem) {
        for (int64_t t = threadIdx.x; t < 2 * T; t += blockDim.x) s_hist[t] = 0;
        __syncthreads();
    }
    RowPartial p{0, 0, 0, 0, 0, -1.79769313486231570e308, -1.79769313486231570e308, -1.0, 0.0};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = rp[i], e = rp[i + 1];
        const int64_t tr = tm.row_tile(i);
        double dom = 0.0, maxr = 0.0, minr = 0.0;
        long long dsum = 0;
        for (int64_t jj = s; jj < e; jj++) {
            const int64_t j = ci[jj];
            const double a = fabs((double)cv[jj]);
            atomicAdd(col_cnt + j, 1);
            atomicAdd(diag_cnt + (j - i + m), 1);
            const int64_t tc = tm.col_tile(j);
            atomicAdd(tiles + tr * T + tc, 1);
            if (smem) {
                atomicAdd(s_hist + tr, 1);
                atomicAdd(s_hist + T + tc, 1);
            } else {
                atomicAdd(rb + tr, 1);
                atomicAdd(cb + tc, 1);
            }
            if (i == j) {
                p.ondiag++;
                p.max_diag = fmax(p.max_diag, a);
                dom += a;
            } else {
                if (i > j) p.lower++;
                else p.upper++;
                p.max_off = fmax(p.max_off, a);
                dom -= a;
            }
            const double lg = log10(a);
            if (maxr < lg) maxr = lg;
            if (a > 0.0 && minr > lg) minr = lg;
            atomic_max_double(maxc + j, lg);  // columns start at 0, as rows
            if (a > 0.0) atomic_min_double(minc + j, lg);
            if (jj + 1 < e) dsum += (long long)ci[jj + 1] - j;
        }
        if (e > s) {
            p.nz_rows++;
            p.dist += (double)dsum / (double)(e - s);
        }
        if (dom > 0) p.dominance++;
        if (minr != 0.0) p.row_div = fmax(p.row_div, maxr - minr);
    }
    if (smem) {
        __syncthreads();
        for (int64_t t = threadIdx.x; t < T; t += blockDim.x) {
            if (s_hist[t]) atomicAdd(rb + t, s_hist[t]);
            if (s_hist[T + t]) atomicAdd(cb + t, s_hist[T + t]);
        }
    }
    part[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = p;
}

// (row, tile column) and (column, tile row) keys of every nonzero
__global__ void feat_uniq_keys(int64_t m, int64_t T, TileMap tm, const int32_t *__restrict__ rp,
                               const int32_t *__restrict__ ci, uint64_t *__restrict__ krow,
                               uint64_t *__restrict__ kcol, uint32_t *__restrict__ v1, uint32_t *__restrict__ v2) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t tr = tm.row_tile(i);
        for (int64_t jj = rp[i]; jj < rp[i + 1]; jj++) {
            krow[jj] = (uint64_t)i * (uint64_t)T + (uint64_t)tm.col_tile(ci[jj]);
            kcol[jj] = (uint64_t)ci[jj] * (uint64_t)T + (uint64_t)tr;
            v1[jj] = v2[jj] = (uint32_t)jj;
        }
    }
}

// distinct keys add one to their tile: rows == 1 for (row, tcol) keys
__global__ void feat_uniq_count(int64_t nnz, int64_t T, TileMap tm, int rows, const uint64_t *__restrict__ k,
                                int32_t *__restrict__ out) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nnz; q += (int64_t)gridDim.x * blockDim.x) {
        if (q > 0 && k[q] == k[q - 1]) continue;
        const int64_t a = (int64_t)(k[q] / (uint64_t)T), b = (int64_t)(k[q] % (uint64_t)T);
        if (rows) atomicAdd(out + tm.row_tile(a) * T + b, 1);
        else atomicAdd(out + b * T + tm.col_tile(a), 1);
    }
}

__global__ void feat_sym_keys(int64_t m, int64_t n, const int32_t *__restrict__ rp, const int32_t *__restrict__ ci,
                              uint64_t *__restrict__ k, uint32_t *__restrict__ v) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        for (int64_t jj = rp[i]; jj < rp[i + 1]; jj++) {
            k[jj] = (uint64_t)i * (uint64_t)n + (uint64_t)ci[jj];
            v[jj] = (uint32_t)jj;
        }
}

__device__ int64_t lower_bound_u64(const uint64_t *a, int64_t len, uint64_t key) {
    int64_t lo = 0, hi = len;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

template <typename V>
__global__ void feat_symmetry(int64_t m, int64_t n, int64_t nnz, const int32_t *__restrict__ rp,
                              const int32_t *__restrict__ ci, const V *__restrict__ cv,
                              const uint64_t *__restrict__ k, const uint32_t *__restrict__ perm,
                              unsigned long long *__restrict__ counts) {
    unsigned long long sp = 0, sv = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        for (int64_t jj = rp[i]; jj < rp[i + 1]; jj++) {
            const int64_t j = ci[jj];
            if (i == j) continue;
            const uint64_t kt = (uint64_t)j * (uint64_t)n + (uint64_t)i;
            const int64_t q = lower_bound_u64(k, nnz, kt);
            if (q < nnz && k[q] == kt) {
                sp++;
                const int64_t q2 = lower_bound_u64(k, nnz, (uint64_t)i * (uint64_t)n + (uint64_t)j);
                if (cv[perm[q]] == cv[perm[q2]]) sv++;  // first values of (j,i) and (i,j)
            }
        }
    atomicAdd(counts, sp);
    atomicAdd(counts + 1, sv);
}

// min / max / nonzero count / sum of squared deviations of an int vector
struct IntStats {
    long long mn, mx, nz;
    double sq;
};

__global__ void feat_int_stats(int64_t len, const int32_t *__restrict__ a, double mean, IntStats *__restrict__ part) {
    IntStats s{100000000LL, 0, 0, 0.0};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (int64_t)gridDim.x * blockDim.x) {
        const long long v = a[i];
        s.mn = min(s.mn, v);
        s.mx = max(s.mx, v);
        s.nz += v != 0;
        const double d = (double)v - mean;
        s.sq += d * d;
    }
    part[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void row_lengths(int64_t m, const int32_t *__restrict__ rp, int32_t *__restrict__ out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = rp[i + 1] - rp[i];
}

__global__ void col_range(int64_t n, const double *__restrict__ maxc, const double *__restrict__ minc,
                          double *__restrict__ part) {
    double best = -1.0;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x)
        if (minc[j] != 0.0) best = fmax(best, maxc[j] - minc[j]);
    part[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = best;
}

template <typename T>
sspmv_status d2h_vec(std::vector<T> &v, const T *d, size_t n, sspmv_stream_t s) {
    v.resize(n);
    if (n) SSPMV_CUDA_TRY(cudaMemcpyAsync(v.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost, cu(s)));
    SSPMV_CUDA_TRY(cudaStreamSynchronize(cu(s)));
    return SSPMV_OK;
}

__global__ void widen_counts(int64_t n, const int32_t *__restrict__ a, uint64_t *__restrict__ k,
                             uint32_t *__restrict__ v) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        k[i] = (uint64_t)(uint32_t)a[i];
        v[i] = (uint32_t)i;
    }
}

__global__ void keys_to_i64(int64_t n, const uint64_t *__restrict__ k, int64_t *__restrict__ w) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        w[i] = (int64_t)k[i];
}

// Sorted counts o (ascending) with exclusive prefix ex: the largest k whose
// top part o[k..L-1] satisfies (L-k)/L + share >= 1 (stored as k+1), and the
// trapezoid sum  sum_k o_k (L - k).
__global__ void feat_pg(int64_t len, int64_t total, const uint64_t *__restrict__ o, const int64_t *__restrict__ ex,
                        unsigned long long *__restrict__ out) {
    unsigned long long a = 0, bk = 0;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < len; k += (int64_t)gridDim.x * blockDim.x) {
        a += (unsigned long long)o[k] * (unsigned long long)(len - k);
        const double p = (double)(len - k) / (double)len, q = (double)(total - ex[k]) / (double)total;
        if (!(p + q < 1.0)) bk = max(bk, (unsigned long long)k + 1);
    }
    atomicAdd(out, a);
    atomicMax(out + 1, bk);
}

// P_ratioAndGini (src/sparse_features.cpp:612-640) of a device count vector
// whose entries sum to `total`.
sspmv_status p_ratio_gini(const int32_t *d_vec, int64_t len, int64_t total, double *p_ratio, double *gini,
                          sspmv_stream_t s) {
    *p_ratio = -1.0;
    *gini = -1.0;
    if (len <= 0 || total <= 0) return SSPMV_OK;
    uint64_t *keys = nullptr;
    uint32_t *vals = nullptr;
    int64_t *ex = nullptr;
    unsigned long long *out = nullptr;
    sspmv_status st = dalloc(&keys, (size_t)len, s);
    if (st == SSPMV_OK) st = dalloc(&vals, (size_t)len, s);
    if (st == SSPMV_OK) st = dalloc(&ex, (size_t)len, s);
    if (st == SSPMV_OK) st = dalloc(&out, 2, s);
    const unsigned g = grid_for(len, 256, (int64_t)num_sms() * 8);
    if (st == SSPMV_OK) {
        widen_counts<<<g, 256, 0, cu(s)>>>(len, d_vec, keys, vals);
        note_launch();
        st = radix_sort_pairs(keys, vals, len, 32, s);
    }
    if (st == SSPMV_OK) {
        keys_to_i64<<<g, 256, 0, cu(s)>>>(len, keys, ex);
        note_launch();
        st = exclusive_scan_i64(ex, ex, len, nullptr, s);
    }
    unsigned long long h[2] = {0, 0};
    if (st == SSPMV_OK) {
        cudaMemsetAsync(out, 0, 16, cu(s));
        feat_pg<<<g, 256, 0, cu(s)>>>(len, total, keys, ex, out);
        note_launch();
        cudaError_t e = cudaMemcpyAsync(h, out, 16, cudaMemcpyDeviceToHost, cu(s));
        if (e == cudaSuccess) e = cudaStreamSynchronize(cu(s));
        if (e != cudaSuccess) st = fail(SSPMV_CUDA_ERROR, "p_ratio_gini: %s", cudaGetErrorString(e));
    }
    if (st == SSPMV_OK) {
        const int64_t kbest = (int64_t)h[1] - 1;  // k = 0 always qualifies
        *p_ratio = (double)(len - kbest) / (double)len;
        const double area = (double)h[0] - (double)total / 2.0;
        const double whole = (double)total * (double)len / 2.0;
        *gini = (whole - area) / whole;
    }
    dfree(keys, s);
    dfree(vals, s);
    dfree(ex, s);
    dfree(out, s);
    return st;
}

struct VecStats {
    int64_t mn = 100000000, mx = 0, nz = 0;
    double sq = 0;
};

sspmv_status int_stats(const int32_t *d, int64_t len, double mean, VecStats *r, sspmv_stream_t s) {
    *r = VecStats();
    if (len <= 0) return SSPMV_OK;
    const int64_t blocks = std::min<int64_t>((len + 255) / 256, (int64_t)num_sms() * 8);
    IntStats *part = nullptr;
    SSPMV_TRY(dalloc(&part, (size_t)blocks * 256, s));
    feat_int_stats<<<(unsigned)blocks, 256, 0, cu(s)>>>(len, d, mean, part);
    note_launch();
    std::vector<IntStats> h;
    sspmv_status st = d2h_vec(h, part, (size_t)blocks * 256, s);
    dfree(part, s);
    SSPMV_TRY(st);
    for (const IntStats &p : h) {  // fixed order: deterministic
        r->mn = std::min<int64_t>(r->mn, p.mn);
        r->mx = std::max<int64_t>(r->mx, p.mx);
        r->nz += p.nz;
        r->sq += p.sq;
    }
    return SSPMV_OK;
}

}  // namespace

// ------------------------------------------------------------ GrX features --
// The tile group analysis the reference specifies but does not build
// (CalculateTilesExtraFeatures under BSR_ANA and AnalyzeTile_Group,
// src/sparse_features.cpp:884-1065): tiles are R x Cd blocks with R =
// BestDimForBSR(num_rows, T), Cd = BestDimForBSR(num_cols, T); an entry is
// present when its value is nonzero.
//   GrX_uniqC: inside each tile, each row is scanned left to right; at a
//     present column p with p + X <= Cd the scan counts a group when columns
//     p .. p+X-1 are all present and resumes at p + step + 1.  For a run of L
//     consecutive present columns inside one tile this counts
//     (L >= X) ? (L - X) / (X + 1) + 1 : 0 groups.  GrX_uniqR likewise down
//     each column.  Both are divided by num_nnzs.
//   GrX_potReuseR: number of (X-row group of a tile row, tile column) pairs
//     holding a present entry, divided by mb * ceil(R / X); GrX_potReuseC
//     likewise with column groups and tile rows.
// A feature stays -1 when the tile is smaller than X in its direction.
namespace {

int64_t best_dim_for_tiles(int64_t nums, int64_t target) {
    // BestDimForBSR (src/sparse_features.cpp:858-880): the first Dim whose
    // block count ceil(nums / Dim) is closest to target.
    int64_t best = 0, best_diff = 10000;
    for (int64_t dim = 1; dim < nums; dim++) {
        const int64_t mb = (nums + dim - 1) / dim;
        const int64_t diff = mb > target ? mb - target : target - mb;
        if (diff < best_diff) {
            best_diff = diff;
            best = dim;
        }
        if (diff == 0) break;
        if (mb < target && diff >= best_diff) break;  // block counts only fall from here on
    }
    return best > 0 ? best : 1;
}

template <typename V>
__global__ void grx_keys(int64_t m, int64_t n, const int32_t *__restrict__ rp, const int32_t *__restrict__ ci,
                         const V *__restrict__ val, uint64_t sentinel, uint64_t *__restrict__ k_rc,
                         uint64_t *__restrict__ k_cr, uint32_t *__restrict__ v1, uint32_t *__restrict__ v2) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        for (int64_t jj = rp[i]; jj < rp[i + 1]; jj++) {
            const bool present = val[jj] != V(0);
            const uint64_t c = (uint64_t)ci[jj];
            k_rc[jj] = present ? (uint64_t)i * (uint64_t)n + c : sentinel;
            k_cr[jj] = present ? c * (uint64_t)m + (uint64_t)i : sentinel;
            v1[jj] = v2[jj] = 0;
        }
}

// Groups in runs of consecutive minor indices (keys sorted, major * minor_n + minor).
__global__ void grx_runs(int64_t cnt, const uint64_t *__restrict__ k, uint64_t sentinel, uint64_t minor_n,
                         uint64_t tile, int64_t X, unsigned long long *__restrict__ total) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < cnt; q += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t key = k[q];
        if (key == sentinel || (q > 0 && k[q - 1] == key)) continue;
        if (q > 0 && (key % minor_n) % tile != 0 && k[q - 1] == key - 1) continue;  // not the start of a run
        int64_t L = 1;
        uint64_t last = key;
        for (int64_t j = q + 1; j < cnt; j++) {
            const uint64_t kj = k[j];
            if (kj == last) continue;
            if (kj == sentinel || kj != last + 1 || (kj % minor_n) % tile == 0) break;
            last = kj;
            L++;
        }
        if (L >= X) atomicAdd(total, (unsigned long long)((L - X) / (X + 1) + 1));
    }
}

// (group of X majors inside its tile, tile of the minor index) keys.
__global__ void grx_pot_keys(int64_t cnt, const uint64_t *__restrict__ k, uint64_t sentinel, uint64_t minor_n,
                             uint64_t tile_major, uint64_t tile_minor, uint64_t X, uint64_t groups_per_tile,
                             uint64_t ntiles_minor, uint64_t out_sentinel, uint64_t *__restrict__ out) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < cnt; q += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t key = k[q];
        if (key == sentinel) {
            out[q] = out_sentinel;
            continue;
        }
        const uint64_t maj = key / minor_n, mnr = key % minor_n;
        const uint64_t group = (maj / tile_major) * groups_per_tile + (maj % tile_major) / X;
        out[q] = group * ntiles_minor + mnr / tile_minor;
    }
}

__global__ void count_distinct(int64_t cnt, const uint64_t *__restrict__ k, uint64_t sentinel,
                               unsigned long long *__restrict__ total) {
    unsigned long long c = 0;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < cnt; q += (int64_t)gridDim.x * blockDim.x)
        c += k[q] != sentinel && (q == 0 || k[q - 1] != k[q]);
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(total, c);
}

}  // namespace

extern "C" sspmv_status sspmv_csr_grx_features(const sspmv_csr *A, int32_t tile_blocks, int32_t group, double *out,
                                               sspmv_stream_t s) {
    if (!A || !out) return fail(SSPMV_INVALID_ARG, "null argument");
    SSPMV_TRY(check_dims(A->f.value_type, A->f.num_rows, A->f.num_cols, A->f.num_nnzs));
    const int64_t m = A->f.num_rows, n = A->f.num_cols, nnz = A->f.num_nnzs;
    if (m == 0 || n == 0 || nnz == 0) return fail(SSPMV_INVALID_ARG, "features need a nonempty matrix");
    if (tile_blocks < 0 || group < 0) return fail(SSPMV_INVALID_ARG, "negative tile_blocks or group");
    const int64_t T = tile_blocks > 0 ? tile_blocks : 256;
    const int64_t X = group > 0 ? group : 64 / (int64_t)vsize(A->f.value_type);
    const int64_t R = best_dim_for_tiles(m, T), Cd = best_dim_for_tiles(n, T);
    const int64_t mb = (m + R - 1) / R, nb = (n + Cd - 1) / Cd;
    const bool do_r = R >= X, do_c = Cd >= X;
    for (int i = 0; i < 4; i++) out[i] = -1.0;
    if (!do_r && !do_c) return SSPMV_OK;
    uint64_t *k_rc = nullptr, *k_cr = nullptr, *k_pot = nullptr;
    uint32_t *v1 = nullptr, *v2 = nullptr, *v3 = nullptr;
    unsigned long long *cnt = nullptr;
    auto release = [&]() {
        dfree(k_rc, s); dfree(k_cr, s); dfree(k_pot, s); dfree(v1, s); dfree(v2, s); dfree(v3, s); dfree(cnt, s);
    };
    sspmv_status st = SSPMV_OK;
#define GTRY(x)                          \
    do {                                 \
        st = (x);                        \
        if (st != SSPMV_OK) {            \
            release();                   \
            return st;                   \
        }                                \
    } while (0)
    GTRY(dalloc(&k_rc, (size_t)nnz, s));
    GTRY(dalloc(&k_cr, (size_t)nnz, s));
    GTRY(dalloc(&k_pot, (size_t)nnz, s));
    GTRY(dalloc(&v1, (size_t)nnz, s));
    GTRY(dalloc(&v2, (size_t)nnz, s));
    GTRY(dalloc(&v3, (size_t)nnz, s));
    GTRY(dalloc(&cnt, 4, s));
    cudaMemsetAsync(cnt, 0, 32, cu(s));
    const uint64_t sentinel = (uint64_t)m * (uint64_t)n;
    const unsigned gm = grid_for(m, 256, (int64_t)num_sms() * 8), gz = grid_for(nnz, 256, (int64_t)num_sms() * 16);
    GTRY(dispatch_value(A->f.value_type, [&](auto tag) -> sspmv_status {
        using V = decltype(tag);
        grx_keys<V><<<gm, 256, 0, cu(s)>>>(m, n, A->row_offset, A->col_index, (const V *)A->values, sentinel, k_rc, k_cr,
                                           v1, v2);
        SSPMV_LAUNCH_CHECK();
        return SSPMV_OK;
    }));
    const int kbits = bits_for(sentinel);
    GTRY(radix_sort_pairs(k_rc, v1, nnz, kbits, s));
    GTRY(radix_sort_pairs(k_cr, v2, nnz, kbits, s));
    const uint64_t gpr = (uint64_t)((R + X - 1) / X), gpc = (uint64_t)((Cd + X - 1) / X);
    if (do_c) {  // groups along columns: row-major keys, tiles of Cd columns
        grx_runs<<<gz, 256, 0, cu(s)>>>(nnz, k_rc, sentinel, (uint64_t)n, (uint64_t)Cd, X, cnt + 1);
        note_launch();
    }
    if (do_r) {
        grx_runs<<<gz, 256, 0, cu(s)>>>(nnz, k_cr, sentinel, (uint64_t)m, (uint64_t)R, X, cnt + 0);
        note_launch();
        const uint64_t ps = (uint64_t)mb * gpr * (uint64_t)nb;
        grx_pot_keys<<<gz, 256, 0, cu(s)>>>(nnz, k_rc, sentinel, (uint64_t)n, (uint64_t)R, (uint64_t)Cd, (uint64_t)X,
                                            gpr, (uint64_t)nb, ps, k_pot);
        note_launch();
        GTRY(radix_sort_pairs(k_pot, v3, nnz, bits_for(ps), s));
        count_distinct<<<gz, 256, 0, cu(s)>>>(nnz, k_pot, ps, cnt + 2);
        note_launch();
    }
    if (do_c) {
        const uint64_t ps = (uint64_t)nb * gpc * (uint64_t)mb;
        grx_pot_keys<<<gz, 256, 0, cu(s)>>>(nnz, k_cr, sentinel, (uint64_t)m, (uint64_t)Cd, (uint64_t)R, (uint64_t)X,
                                            gpc, (uint64_t)mb, ps, k_pot);
        note_launch();
        GTRY(radix_sort_pairs(k_pot, v3, nnz, bits_for(ps), s));
        count_distinct<<<gz, 256, 0, cu(s)>>>(nnz, k_pot, ps, cnt + 3);
        note_launch();
    }
    unsigned long long h[4] = {0, 0, 0, 0};
    cudaError_t e = cudaMemcpyAsync(h, cnt, 32, cudaMemcpyDeviceToHost, cu(s));
    if (e == cudaSuccess) e = cudaStreamSynchronize(cu(s));
    release();
#undef GTRY
    if (e != cudaSuccess) return fail(SSPMV_CUDA_ERROR, "grx features: %s", cudaGetErrorString(e));
    if (do_r) {
        out[0] = (double)h[0] / (double)nnz;
        out[2] = (double)h[2] / (double)((uint64_t)mb * gpr);
    }
    if (do_c) {
        out[1] = (double)h[1] / (double)nnz;
        out[3] = (double)h[3] / (double)((uint64_t)nb * gpc);
    }
    return SSPMV_OK;
}

static const char *kFeatureNames[SSPMV_NUM_FEATURES] = {
    "num_rows", "num_cols", "num_nnz", "nnz_ratio", "nnz_on_maindiag_ratio", "nnz_row_distance_ratio",
    "nz_row_ratio", "max_nnz_each_row", "ave_nnz_each_row", "standard_dev_row", "P-ratio_row", "Gini_coeff_row",
    "nz_col_ratio", "max_nnz_each_col", "ave_nnz_each_col", "standard_dev_col", "P-ratio_col", "Gini_coeff_col",
    "nz_tiles_ratio", "max_nnz_each_tiles", "ave_nnz_each_tiles", "standard_dev_tiles", "P-ratio_tiles",
    "Gini_coeff_tiles", "nz_ratio_RB", "max_nnz_each_RB", "ave_nnz_each_RB", "standard_dev_RB", "P-ratio_RB",
    "Gini_coeff_RB", "nz_ratio_CB", "max_nnz_each_CB", "ave_nnz_each_CB", "standard_dev_CB", "P-ratio_CB",
    "Gini_coeff_CB", "uniq_R", "uniq_C", "potReuseR", "potReuseC", "nnz_lower", "nnz_upper", "nnz_diagonal",
    "num_diags", "min_nnz_each_row", "min_nnz_each_col", "diagonal_dominant_ratio", "max_value_offdiag",
    "max_value_diagonal", "row_variability", "col_variability", "pattern_symm", "value_symm", "min_nnz_each_tiles",
    "min_nnz_each_RB", "min_nnz_each_CB", "var_nnz_each_row", "var_nnz_each_col", "GrX_uniqR", "GrX_uniqC",
    "GrX_potReuseR", "GrX_potReuseC"};

extern "C" const char *sspmv_feature_name(int32_t i) {
    return (i >= 0 && i < SSPMV_NUM_FEATURES) ? kFeatureNames[i] : nullptr;
}

extern "C" sspmv_status sspmv_csr_features(const sspmv_csr *A, int32_t tile_blocks, double *F, int32_t *nnz_by_tiles,
                                           int32_t *uniq_rb, int32_t *uniq_cb, sspmv_stream_t s) {
    if (!A || !F) return fail(SSPMV_INVALID_ARG, "null argument");
    SSPMV_TRY(check_dims(A->f.value_type, A->f.num_rows, A->f.num_cols, A->f.num_nnzs));
    const int64_t m = A->f.num_rows, n = A->f.num_cols, nnz = A->f.num_nnzs;
    if (m == 0 || n == 0 || nnz == 0) return fail(SSPMV_INVALID_ARG, "features need a nonempty matrix");
    const int64_t T = tile_blocks > 0 ? tile_blocks : 256;
    const int64_t TT = T * T;
    TileMap tm{T, m / T, m % T, n / T, n % T};
    int32_t *col_cnt = nullptr, *diag_cnt = nullptr, *tiles = nullptr, *rb = nullptr, *cb = nullptr;
    int32_t *urb = nullptr, *ucb = nullptr, *rows = nullptr;
    double *maxc = nullptr, *minc = nullptr, *crange = nullptr;
    RowPartial *part = nullptr;
    uint64_t *k1 = nullptr, *k2 = nullptr;
    uint32_t *v1 = nullptr, *v2 = nullptr;
    unsigned long long *sym = nullptr;
    const int64_t blocks = std::min<int64_t>((m + 255) / 256, (int64_t)num_sms() * 8);
    auto release = [&]() {
        dfree(col_cnt, s); dfree(diag_cnt, s); dfree(tiles, s); dfree(rb, s); dfree(cb, s);
        dfree(urb, s); dfree(ucb, s); dfree(rows, s); dfree(maxc, s); dfree(minc, s); dfree(crange, s);
        dfree(part, s); dfree(k1, s); dfree(k2, s); dfree(v1, s); dfree(v2, s); dfree(sym, s);
    };
    sspmv_status st = SSPMV_OK;
#define FTRY(x)                          \
    do {                                 \
        st = (x);                        \
        if (st != SSPMV_OK) {            \
            release();                   \
            return st;                   \
        }                                \
    } while (0)
    FTRY(dalloc(&col_cnt, (size_t)n, s));
    FTRY(dalloc(&diag_cnt, (size_t)(m + n), s));
    FTRY(dalloc(&tiles, (size_t)TT, s));
    FTRY(dalloc(&rb, (size_t)T, s));
    FTRY(dalloc(&cb, (size_t)T, s));
    FTRY(dalloc(&urb, (size_t)TT, s));
    FTRY(dalloc(&ucb, (size_t)TT, s));
    FTRY(dalloc(&rows, (size_t)m, s));
    FTRY(dalloc(&maxc, (size_t)n, s));
    FTRY(dalloc(&minc, (size_t)n, s));
    FTRY(dalloc(&part, (size_t)blocks * 256, s));
    cudaMemsetAsync(col_cnt, 0, (size_t)n * 4, cu(s));
    cudaMemsetAsync(diag_cnt, 0, (size_t)(m + n) * 4, cu(s));
    cudaMemsetAsync(tiles, 0, (size_t)TT * 4, cu(s));
    cudaMemsetAsync(rb, 0, (size_t)T * 4, cu(s));
    cudaMemsetAsync(cb, 0, (size_t)T * 4, cu(s));
    cudaMemsetAsync(urb, 0, (size_t)TT * 4, cu(s));
    cudaMemsetAsync(ucb, 0, (size_t)TT * 4, cu(s));
    cudaMemsetAsync(maxc, 0, (size_t)n * 8, cu(s));
    cudaMemsetAsync(minc, 0, (size_t)n * 8, cu(s));
    const size_t smem = T <= kMaxSmemBlocks ? (size_t)2 * T * 4 : 0;
    FTRY(dispatch_value(A->f.value_type, [&](auto tag) -> sspmv_status {
        using V = decltype(tag);
        feat_rows<V><<<(unsigned)blocks, 256, smem, cu(s)>>>(m, tm, A->row_offset, A->col_index, (const V *)A->values,
                                                             col_cnt, diag_cnt, tiles, rb, cb, maxc, minc, part);
        SSPMV_LAUNCH_CHECK();
        return SSPMV_OK;
    }));
    // distinct rows / columns per tile
    FTRY(dalloc(&k1, (size_t)nnz, s));
    FTRY(dalloc(&k2, (size_t)nnz, s));
    FTRY(dalloc(&v1, (size_t)nnz, s));
    FTRY(dalloc(&v2, (size_t)nnz, s));
    const unsigned gz = grid_for(nnz, 256, (int64_t)num_sms() * 16);
    feat_uniq_keys<<<(unsigned)blocks, 256, 0, cu(s)>>>(m, T, tm, A->row_offset, A->col_index, k1, k2, v1, v2);
    note_launch();
    FTRY(radix_sort_pairs(k1, v1, nnz, bits_for((uint64_t)m * (uint64_t)T), s));
    feat_uniq_count<<<gz, 256, 0, cu(s)>>>(nnz, T, tm, 1, k1, urb);
    note_launch();
    FTRY(radix_sort_pairs(k2, v2, nnz, bits_for((uint64_t)n * (uint64_t)T), s));
    feat_uniq_count<<<gz, 256, 0, cu(s)>>>(nnz, T, tm, 0, k2, ucb);
    note_launch();
    // pattern / value symmetry (square matrices)
    unsigned long long hsym[2] = {0, 0};
    if (m == n) {
        FTRY(dalloc(&sym, 2, s));
        cudaMemsetAsync(sym, 0, 16, cu(s));
        feat_sym_keys<<<(unsigned)blocks, 256, 0, cu(s)>>>(m, n, A->row_offset, A->col_index, k1, v1);
        note_launch();
        FTRY(radix_sort_pairs(k1, v1, nnz, bits_for((uint64_t)m * (uint64_t)n), s));
        FTRY(dispatch_value(A->f.value_type, [&](auto tag) -> sspmv_status {
            using V = decltype(tag);
            feat_symmetry<V><<<(unsigned)blocks, 256, 0, cu(s)>>>(m, n, nnz, A->row_offset, A->col_index,
                                                                  (const V *)A->values, k1, v1, sym);
            SSPMV_LAUNCH_CHECK();
            return SSPMV_OK;
        }));
        cudaMemcpyAsync(hsym, sym, 16, cudaMemcpyDeviceToHost, cu(s));
    }
    // row partials (fixed order)
    std::vector<RowPartial> hp;
    FTRY(d2h_vec(hp, part, (size_t)blocks * 256, s));
    RowPartial P{0, 0, 0, 0, 0, -1.79769313486231570e308, -1.79769313486231570e308, -1.0, 0.0};
    for (const RowPartial &q : hp) {
        P.lower += q.lower; P.upper += q.upper; P.ondiag += q.ondiag; P.dominance += q.dominance; P.nz_rows += q.nz_rows;
        P.max_off = std::max(P.max_off, q.max_off); P.max_diag = std::max(P.max_diag, q.max_diag);
        P.row_div = std::max(P.row_div, q.row_div); P.dist += q.dist;
    }
    // column value range
    FTRY(dalloc(&crange, (size_t)blocks * 256, s));
    col_range<<<(unsigned)blocks, 256, 0, cu(s)>>>(n, maxc, minc, crange);
    note_launch();
    std::vector<double> hcr;
    FTRY(d2h_vec(hcr, crange, (size_t)blocks * 256, s));
    double col_div = -1.0;
    for (double v : hcr) col_div = std::max(col_div, v);
    // diagonals: count and the ones within 5% of the main diagonal
    std::vector<int32_t> hdiag;
    FTRY(d2h_vec(hdiag, diag_cnt, (size_t)(m + n), s));
    int64_t ndiags = 0, close = 0;
    const int64_t close_thr = (m + n - 1) / 20;
    for (int64_t t = 0; t < m + n; t++)
        if (hdiag[(size_t)t]) {
            ndiags++;
            if (std::llabs(t - m) <= close_thr) close += hdiag[(size_t)t];
        }
    // count-vector statistics
    row_lengths<<<(unsigned)blocks, 256, 0, cu(s)>>>(m, A->row_offset, rows);
    note_launch();
    const double ave_r = (double)nnz / m, ave_c = (double)nnz / n;
    const double ave_t = (double)nnz / ((double)T * T), ave_b = (double)nnz / T;
    VecStats sr, sc, st_t, sb, scb;
    FTRY(int_stats(rows, m, ave_r, &sr, s));
    FTRY(int_stats(col_cnt, n, ave_c, &sc, s));
    FTRY(int_stats(tiles, TT, ave_t, &st_t, s));
    FTRY(int_stats(rb, T, ave_b, &sb, s));
    FTRY(int_stats(cb, T, ave_b, &scb, s));
    double pr_r, g_r, pr_c, g_c, pr_t, g_t, pr_rb, g_rb, pr_cb, g_cb;
    FTRY(p_ratio_gini(rows, m, nnz, &pr_r, &g_r, s));
    FTRY(p_ratio_gini(col_cnt, n, nnz, &pr_c, &g_c, s));
    FTRY(p_ratio_gini(tiles, TT, nnz, &pr_t, &g_t, s));
    FTRY(p_ratio_gini(rb, T, nnz, &pr_rb, &g_rb, s));
    FTRY(p_ratio_gini(cb, T, nnz, &pr_cb, &g_cb, s));
    // uniq sums and optional arrays
    std::vector<int32_t> hurb, hucb;
    FTRY(d2h_vec(hurb, urb, (size_t)TT, s));
    FTRY(d2h_vec(hucb, ucb, (size_t)TT, s));
    long long sum_urb = 0, sum_ucb = 0;
    for (int64_t i = 0; i < TT; i++) {
        sum_urb += hurb[(size_t)i];
        sum_ucb += hucb[(size_t)i];
    }
    if (uniq_rb) std::copy(hurb.begin(), hurb.end(), uniq_rb);
    if (uniq_cb) std::copy(hucb.begin(), hucb.end(), uniq_cb);
    if (nnz_by_tiles) {
        std::vector<int32_t> ht;
        FTRY(d2h_vec(ht, tiles, (size_t)TT, s));
        std::copy(ht.begin(), ht.end(), nnz_by_tiles);
    }
    release();
#undef FTRY
    // CalculateTilesFeatures accumulators start at -1 (include/sparse_features.h:242-244,293-295)
    const double var_t = (-1.0 + st_t.sq) / (double)TT, var_rb = (-1.0 + sb.sq) / T, var_cb = (-1.0 + scb.sq) / T;
    const double var_r = sr.sq / m, var_c = sc.sq / n;
    double v[SSPMV_NUM_FEATURES] = {
        (double)m, (double)n, (double)nnz, (double)nnz / ((double)m * n), (double)close / nnz,
        P.dist / m / n, (double)P.nz_rows / m, (double)sr.mx, ave_r, std::sqrt(var_r), pr_r, g_r,
        (double)sc.nz / n, (double)sc.mx, ave_c, std::sqrt(var_c), pr_c, g_c,
        (-1.0 + st_t.nz) / (double)TT, (double)st_t.mx, ave_t, std::sqrt(std::max(var_t, 0.0)), pr_t, g_t,
        (-1.0 + sb.nz) / T, (double)sb.mx, ave_b, std::sqrt(std::max(var_rb, 0.0)), pr_rb, g_rb,
        (-1.0 + scb.nz) / T, (double)scb.mx, ave_b, std::sqrt(std::max(var_cb, 0.0)), pr_cb, g_cb,
        (double)sum_urb / nnz, (double)sum_ucb / nnz, (double)sum_urb / m, (double)sum_ucb / n,
        (double)P.lower, (double)P.upper, (double)P.ondiag, (double)ndiags, (double)sr.mn, (double)sc.mn,
        (double)P.dominance / (double)std::min(m, n), P.max_off, P.max_diag, P.row_div, col_div,
        m == n ? (double)hsym[0] / (double)(nnz - P.ondiag) : 0.0,
        m == n ? (double)hsym[1] / (double)(nnz - P.ondiag) : 0.0,
        (double)st_t.mn, (double)sb.mn, (double)scb.mn, var_r, var_c, -1.0, -1.0, -1.0, -1.0};
    std::copy(v, v + SSPMV_NUM_FEATURES, F);
    return SSPMV_OK;
}
