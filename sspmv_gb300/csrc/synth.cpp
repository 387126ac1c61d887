// synth.cpp -- seeded synthetic CSR matrices and vectors (host, OpenMP).
//
// Every random draw is a pure function of (seed, stream, a, b) through a
// splitmix64-style mixer, so a matrix is identical whatever the thread count
// and on any host (x86_64 or aarch64).  Rows are column-sorted and free of
// duplicates, which is what the reference's converters need for bit-exact
// comparison (DIA and BSR overwrite duplicates while CSR sums them).
//
// Families (the synthetic workloads the SpMV benchmark suite is quoted on):
//   LAPLACIAN2D  5-point stencil on a g x g grid, diagonal 4, off-diagonals -1
//   BANDED       fixed diagonal offsets, values U[-1,1)
//   POWERLAW     row lengths from a truncated Zipf law scaled to a target
//                mean, uniform random distinct columns, values U[-1,1)
//   BLOCK        distinct dense b x b blocks at uniform random block positions
//   UNIFORM      a fixed number of distinct uniform random columns per row
#include "sspmv.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

enum : uint64_t { ST_LEN = 1, ST_COL = 2, ST_VAL = 3, ST_EMPTY = 4, ST_BLOCK = 5, ST_VEC = 6, ST_ROUND = 7 };

inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline uint64_t hash4(uint64_t seed, uint64_t stream, uint64_t a, uint64_t b) {
    uint64_t h = mix64(seed ^ (stream * 0xD6E8FEB86659FD93ull));
    h = mix64(h ^ a);
    return mix64(h ^ (b * 0x9E3779B97F4A7C15ull));
}
inline double u01(uint64_t h) { return (double)(h >> 11) * (1.0 / 9007199254740992.0); }
inline double value_at(uint64_t seed, int64_t row, int64_t col) {
    return 2.0 * u01(hash4(seed, ST_VAL, (uint64_t)row, (uint64_t)col)) - 1.0;
}

// Zipf(alpha) on [1, cap] sampled by inverse CDF; rows are scaled to `mean`.
struct PowerLaw {
    std::vector<double> cdf;
    double scale = 1.0;
    int64_t cap = 1;
    void init(double alpha, double mean, int64_t cap_) {
        cap = cap_ < 1 ? 1 : cap_;
        cdf.resize((size_t)cap);
        double acc = 0, m1 = 0;
        for (int64_t k = 1; k <= cap; k++) {
            double w = std::pow((double)k, -alpha);
            acc += w;
            m1 += w * (double)k;
            cdf[(size_t)k - 1] = acc;
        }
        for (auto &c : cdf) c /= acc;
        double ez = m1 / acc;
        scale = mean > 0 ? mean / ez : 1.0;
    }
    int64_t draw(uint64_t seed, int64_t row) const {
        double u = u01(hash4(seed, ST_LEN, (uint64_t)row, 0));
        int64_t z = (int64_t)(std::lower_bound(cdf.begin(), cdf.end(), u) - cdf.begin()) + 1;
        double v = u01(hash4(seed, ST_ROUND, (uint64_t)row, 0));
        int64_t l = (int64_t)std::floor(scale * (double)z + v);
        if (l < 1) l = 1;
        if (l > cap) l = cap;
        return l;
    }
};

// L distinct columns in [0, ncols), ascending, drawn from row-keyed streams.
void distinct_cols(uint64_t seed, int64_t row, int64_t L, int64_t ncols, int32_t *out) {
    if (L >= ncols) {
        for (int64_t j = 0; j < ncols; j++) out[j] = (int32_t)j;
        return;
    }
    if (2 * L > ncols) {  // dense rows: partial Fisher-Yates over all columns
        std::vector<int32_t> all((size_t)ncols);
        for (int64_t j = 0; j < ncols; j++) all[(size_t)j] = (int32_t)j;
        for (int64_t j = 0; j < L; j++) {
            int64_t k = j + (int64_t)(u01(hash4(seed, ST_COL, (uint64_t)row, (uint64_t)j)) * (double)(ncols - j));
            std::swap(all[(size_t)j], all[(size_t)k]);
        }
        std::sort(all.begin(), all.begin() + L);
        std::memcpy(out, all.data(), sizeof(int32_t) * (size_t)L);
        return;
    }
    std::vector<int32_t> c;
    c.reserve((size_t)L + 8);
    uint64_t draw = 0;
    while ((int64_t)c.size() < L) {
        int64_t need = L - (int64_t)c.size();
        for (int64_t t = 0; t < need; t++, draw++)
            c.push_back((int32_t)(u01(hash4(seed, ST_COL, (uint64_t)row, draw)) * (double)ncols));
        std::sort(c.begin(), c.end());
        c.erase(std::unique(c.begin(), c.end()), c.end());
    }
    std::memcpy(out, c.data(), sizeof(int32_t) * (size_t)L);
}

bool row_is_empty(const sspmv_synth_params *p, uint64_t seed, int64_t row) {
    return p->empty_row_frac > 0 && u01(hash4(seed, ST_EMPTY, (uint64_t)row, 0)) < p->empty_row_frac;
}

struct BlockSet {
    std::vector<uint64_t> keys;  // br * nbc + bc, ascending, distinct
    std::vector<int64_t> start;  // per block row, into keys
};

void build_blocks(const sspmv_synth_params *p, uint64_t seed, int64_t m, int64_t n, BlockSet &bs) {
    int64_t b = p->block_dim > 0 ? p->block_dim : 4;
    int64_t nbr = (m + b - 1) / b, nbc = (n + b - 1) / b;
    int64_t want = p->num_blocks;
    if (want > nbr * nbc) want = nbr * nbc;
    uint64_t draw = 0;
    bs.keys.clear();
    while ((int64_t)bs.keys.size() < want) {
        int64_t need = want - (int64_t)bs.keys.size();
        size_t old = bs.keys.size();
        bs.keys.resize(old + (size_t)need);
#pragma omp parallel for schedule(static)
        for (int64_t t = 0; t < need; t++) {
            uint64_t h1 = hash4(seed, ST_BLOCK, draw + (uint64_t)t, 0);
            uint64_t h2 = hash4(seed, ST_BLOCK, draw + (uint64_t)t, 1);
            uint64_t br = (uint64_t)(u01(h1) * (double)nbr), bc = (uint64_t)(u01(h2) * (double)nbc);
            bs.keys[old + (size_t)t] = br * (uint64_t)nbc + bc;
        }
        draw += (uint64_t)need;
        std::sort(bs.keys.begin(), bs.keys.end());
        bs.keys.erase(std::unique(bs.keys.begin(), bs.keys.end()), bs.keys.end());
    }
    bs.start.assign((size_t)nbr + 1, 0);
    for (uint64_t k : bs.keys) bs.start[(size_t)(k / (uint64_t)nbc) + 1]++;
    for (int64_t r = 0; r < nbr; r++) bs.start[(size_t)r + 1] += bs.start[(size_t)r];
}

int64_t row_len(const sspmv_synth_params *p, const PowerLaw &pl, const BlockSet &bs, uint64_t seed,
                int64_t m, int64_t n, int64_t i) {
    switch (p->family) {
    case SSPMV_SYNTH_LAPLACIAN2D: {
        int64_t g = p->grid, gy = i / g, gx = i % g;
        return 1 + (gy > 0) + (gx > 0) + (gx < g - 1) + (gy < g - 1);
    }
    case SSPMV_SYNTH_BANDED: {
        int64_t l = 0;
        for (int d = 0; d < p->num_offsets; d++) {
            int64_t j = i + p->offsets[d];
            l += (j >= 0 && j < n);
        }
        return l;
    }
    case SSPMV_SYNTH_POWERLAW:
        return row_is_empty(p, seed, i) ? 0 : pl.draw(seed, i);
    case SSPMV_SYNTH_BLOCK: {
        int64_t b = p->block_dim > 0 ? p->block_dim : 4, br = i / b;
        int64_t nbc = (n + b - 1) / b, l = 0;
        for (int64_t k = bs.start[(size_t)br]; k < bs.start[(size_t)br + 1]; k++) {
            int64_t bc = (int64_t)(bs.keys[(size_t)k] % (uint64_t)nbc);
            int64_t c0 = bc * b, c1 = std::min(n, c0 + b);
            l += c1 - c0;
        }
        return l;
    }
    case SSPMV_SYNTH_UNIFORM:
        return row_is_empty(p, seed, i) ? 0 : std::min<int64_t>(p->per_row, n);
    }
    (void)m;
    return 0;
}

void fill_row(const sspmv_synth_params *p, const BlockSet &bs, uint64_t seed, int64_t n, int64_t i,
              int64_t len, int32_t *cols, double *vals) {
    switch (p->family) {
    case SSPMV_SYNTH_LAPLACIAN2D: {
        int64_t g = p->grid, gy = i / g, gx = i % g, k = 0;
        if (gy > 0) { cols[k] = (int32_t)(i - g); vals[k++] = -1.0; }
        if (gx > 0) { cols[k] = (int32_t)(i - 1); vals[k++] = -1.0; }
        cols[k] = (int32_t)i; vals[k++] = 4.0;
        if (gx < g - 1) { cols[k] = (int32_t)(i + 1); vals[k++] = -1.0; }
        if (gy < g - 1) { cols[k] = (int32_t)(i + g); vals[k++] = -1.0; }
        return;
    }
    case SSPMV_SYNTH_BANDED: {
        std::vector<int64_t> off(p->offsets, p->offsets + p->num_offsets);
        std::sort(off.begin(), off.end());
        int64_t k = 0;
        for (int64_t o : off) {
            int64_t j = i + o;
            if (j >= 0 && j < n) cols[k++] = (int32_t)j;
        }
        break;
    }
    case SSPMV_SYNTH_POWERLAW:
    case SSPMV_SYNTH_UNIFORM:
        if (len > 0) distinct_cols(seed, i, len, n, cols);
        break;
    case SSPMV_SYNTH_BLOCK: {
        int64_t b = p->block_dim > 0 ? p->block_dim : 4, br = i / b;
        int64_t nbc = (n + b - 1) / b, k = 0;
        for (int64_t q = bs.start[(size_t)br]; q < bs.start[(size_t)br + 1]; q++) {
            int64_t bc = (int64_t)(bs.keys[(size_t)q] % (uint64_t)nbc);
            for (int64_t c = bc * b; c < std::min(n, bc * b + b); c++) cols[k++] = (int32_t)c;
        }
        break;
    }
    }
    for (int64_t k = 0; k < len; k++) vals[k] = value_at(seed, i, cols[k]);
}

int64_t ncols_of(const sspmv_synth_params *p, int64_t m) { return p->num_cols > 0 ? p->num_cols : m; }

int64_t nrows_of(const sspmv_synth_params *p) {
    if (p->family == SSPMV_SYNTH_LAPLACIAN2D) return p->grid * p->grid;
    return p->num_rows;
}

}  // namespace

extern "C" {

int64_t sspmv_synth_row_offsets(const sspmv_synth_params *p, uint64_t seed, int32_t *row_offset) {
    int64_t m = nrows_of(p), n = ncols_of(p, m);
    if (m < 0 || n < 0) return -1;
    PowerLaw pl;
    if (p->family == SSPMV_SYNTH_POWERLAW) pl.init(p->alpha, p->mean, std::min<int64_t>(p->cap, n));
    BlockSet bs;
    if (p->family == SSPMV_SYNTH_BLOCK) build_blocks(p, seed, m, n, bs);
    std::vector<int64_t> len((size_t)m);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < m; i++) len[(size_t)i] = row_len(p, pl, bs, seed, m, n, i);
    int64_t acc = 0;
    row_offset[0] = 0;
    for (int64_t i = 0; i < m; i++) {
        acc += len[(size_t)i];
        if (acc > 2147483647LL) return -1;  // int32 index space
        row_offset[i + 1] = (int32_t)acc;
    }
    return acc;
}

static int synth_fill(const sspmv_synth_params *p, uint64_t seed, const int32_t *row_offset, int32_t *col,
                      double *vd, float *vf) {
    int64_t m = nrows_of(p), n = ncols_of(p, m);
    BlockSet bs;
    if (p->family == SSPMV_SYNTH_BLOCK) build_blocks(p, seed, m, n, bs);
#pragma omp parallel
    {
        std::vector<double> tmp;
#pragma omp for schedule(dynamic, 1024)
        for (int64_t i = 0; i < m; i++) {
            int64_t s = row_offset[i], l = row_offset[i + 1] - s;
            tmp.resize((size_t)std::max<int64_t>(l, 1));
            fill_row(p, bs, seed, n, i, l, col + s, tmp.data());
            if (vd) std::memcpy(vd + s, tmp.data(), sizeof(double) * (size_t)l);
            if (vf)
                for (int64_t k = 0; k < l; k++) vf[s + k] = (float)tmp[(size_t)k];
        }
    }
    return 0;
}

int sspmv_synth_fill_f64(const sspmv_synth_params *p, uint64_t seed, const int32_t *row_offset,
                         int32_t *col_index, double *values) {
    return synth_fill(p, seed, row_offset, col_index, values, nullptr);
}

int sspmv_synth_fill_f32(const sspmv_synth_params *p, uint64_t seed, const int32_t *row_offset,
                         int32_t *col_index, float *values) {
    return synth_fill(p, seed, row_offset, col_index, nullptr, values);
}

void sspmv_synth_vector_f64(int64_t n, uint64_t seed, double *out) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) out[i] = 2.0 * u01(hash4(seed, ST_VEC, (uint64_t)i, 0)) - 1.0;
}

void sspmv_synth_vector_f32(int64_t n, uint64_t seed, float *out) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) out[i] = (float)(2.0 * u01(hash4(seed, ST_VEC, (uint64_t)i, 0)) - 1.0);
}

}  // extern "C"
