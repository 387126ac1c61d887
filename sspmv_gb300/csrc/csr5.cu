// csr5.cu -- CSR5 format on sm_103a: GPU converter, SpMV / SpMM, export.
//
// Format (Liu & Vinter, ICS'15; reference struct include/sparse_format.h:141-
// 166): the nonzeros are cut into tiles of sigma x omega; tile t's elements
// are stored transposed (element of lane x, position i at t*sigma*omega +
// i*omega + x) unless the tile lies inside one row ("fast track", tile_ptr
// words equal) or is the last tile.  tile_ptr[t] = row holding the tile's
// first nonzero, bit 31 set when the tile meets an empty row.  Each lane's
// first descriptor word holds y_offset (rows started in earlier lanes),
// seg_offset and one bit per position where a row starts; tiles with empty
// rows map segment numbers to rows through tile_desc_offset.
//
// Converter (csr_to_csr5, include/sparse_conversion.h:939-1379, csr5_utils.h):
// every step runs per tile or per row on the GPU and reproduces the
// reference's arrays bit for bit (tile_ptr[_p] left 0 as the reference does;
// tile_desc_offset slots the reference never writes are 0).
//
// SpMV (LeSpMV_csr5, src/spmv_csr5.cpp:439-457, which the reference builds for
// double with AVX-512 only): one warp covers 32/omega tiles, a lane per tile
// column.  Each lane sums its sigma products, closing a row segment at every
// start bit; segments that run across lanes are joined with a segmented
// shuffle scan keyed by segment number.  A tile's first and last rows can
// cross tile boundaries: their pieces go to per-tile carries that a fix-up
// kernel adds in tile order, so results are deterministic.  A row pass handles
// the last tile (as CSR rows) and sets y = beta*y on empty rows.  Unlike the
// reference, beta is applied to every row (the reference drops it on rows that
// lie inside one tile, src/spmv_csr5.cpp:287-288).
#include <algorithm>
#include <cstring>
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

struct Geom {
    int32_t sigma, omega, byo, bso, np, p;
};

// ------------------------------------------------------------ converter --
__global__ void c5_tile_ptr(int32_t p, int32_t tile, int32_t m, int32_t nnz, const int32_t *__restrict__ rp,
                            uint32_t *__restrict__ tp) {
    int32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= p) return;
    int64_t b = (int64_t)t * tile;
    if (b > nnz) b = nnz;
    int32_t start = 0, stop = m;
    while (stop >= start) {
        int32_t med = (stop + start) / 2;
        if (b >= rp[med]) start = med + 1;
        else stop = med - 1;
    }
    tp[t] = (uint32_t)(start - 1);
}

__global__ void c5_dirty(int32_t p, const int32_t *__restrict__ rp, const uint32_t *__restrict__ tin,
                         uint32_t *__restrict__ tout) {
    int32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= p) return;
    uint32_t start = tin[t] & 0x7FFFFFFFu, stop = tin[t + 1] & 0x7FFFFFFFu;
    uint32_t v = tin[t];
    if (start != stop) {
        for (uint32_t r = start; r <= stop; r++)
            if (rp[r] == rp[r + 1]) {
                v = start | 0x80000000u;
                break;
            }
    }
    tout[t] = v;
}

__global__ void c5_bits(int32_t m, int32_t p, Geom g, const int32_t *__restrict__ rp, uint32_t *__restrict__ td) {
    const int32_t tile = g.sigma * g.omega, bao = g.byo + g.bso;
    for (int32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x) {
        const int32_t ptr = rp[r];
        const int32_t pid = ptr / tile;
        if (pid < p - 1) {
            const int32_t lx = (ptr / g.sigma) % g.omega;
            const int32_t glid = ptr % g.sigma + bao;
            atomicOr(td + (size_t)pid * g.omega * g.np + (size_t)(glid / 32) * g.omega + lx, 1u << (31 - glid % 32));
        }
    }
}

// include/sparse_conversion.h:1113-1213, one thread per tile
__global__ void c5_offsets_pack(int32_t p, Geom g, const uint32_t *__restrict__ tp, uint32_t *__restrict__ td,
                                int32_t *__restrict__ tdo_ptr) {
    int32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= p - 1) return;
    const bool with_empty = (tp[t] >> 31) & 1u;
    const uint32_t rs = tp[t] & 0x7FFFFFFFu, re = tp[t + 1] & 0x7FFFFFFFu;
    if (rs == re) return;
    const int32_t bao = g.byo + g.bso, omega = g.omega, sigma = g.sigma;
    uint32_t *d = td + (size_t)t * omega * g.np;
    int32_t segn[33], present[33];
    for (int32_t l = 0; l <= omega; l++) {
        segn[l] = 0;
        present[l] = 0;
    }
    present[omega] = 1;
    for (int32_t lane = 0; lane < omega; lane++) {
        int32_t stop = 0, ly = 0, pres = lane == 0;
        uint32_t bitflag = (d[lane] << bao) | ((uint32_t)pres << 31);
        const int32_t start = !((bitflag >> 31) & 1u);
        pres |= (int32_t)((bitflag >> 31) & 1u);
        for (int32_t i = 1; i < sigma; i++) {
            if ((!ly && i == 32 - bao) || (ly && (i - (32 - bao)) % 32 == 0)) {
                ly++;
                bitflag = d[(size_t)ly * omega + lane];
            }
            const int32_t ni = !ly ? i : i - (32 - bao);
            stop += (int32_t)((bitflag >> (31 - ni % 32)) & 1u);
            pres |= (int32_t)((bitflag >> (31 - ni % 32)) & 1u);
        }
        const int32_t sg = stop - start + pres;
        segn[lane] = sg > 0 ? sg : 0;
        present[lane] = pres;
    }
    int32_t run = 0;
    for (int32_t l = 0; l <= omega; l++) {
        const int32_t v = segn[l];
        segn[l] = run;
        run += v;
    }
    if (with_empty) tdo_ptr[t] = segn[omega];
    for (int32_t lane = 0; lane < omega; lane++) {
        int32_t yo = segn[lane], ss = 0, nx = lane + 1;
        if (present[lane])
            while (!present[nx] && nx < omega) {
                ss++;
                nx++;
            }
        yo = lane ? yo - 1 : 0;
        d[lane] = d[lane] | ((uint32_t)yo << (32 - g.byo)) | ((uint32_t)ss << (32 - bao));
    }
}

__device__ int32_t c5_rel_row(const int32_t *rp, int32_t rs, int32_t re, int32_t idx) {
    int32_t start = 0, stop = re - rs - 1;
    while (stop >= start) {
        const int32_t med = (stop + start) / 2;
        if (idx >= rp[rs + 1 + med]) start = med + 1;
        else stop = med - 1;
    }
    return start - 1;
}

// include/sparse_conversion.h:1254-1358, one thread per tile with empty rows
__global__ void c5_desc_offsets(int32_t p, Geom g, const int32_t *__restrict__ rp, const uint32_t *__restrict__ tp,
                                const uint32_t *__restrict__ td, const int32_t *__restrict__ tdo_ptr,
                                int32_t *__restrict__ tdo) {
    int32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= p - 1 || !((tp[t] >> 31) & 1u)) return;
    const int32_t rs = (int32_t)(tp[t] & 0x7FFFFFFFu), re = (int32_t)(tp[t + 1] & 0x7FFFFFFFu);
    const int32_t omega = g.omega, sigma = g.sigma, bao = g.byo + g.bso, bbf = 32 - bao;
    const int32_t optr = tdo_ptr[t];
    const uint32_t *d0 = td + (size_t)t * omega * g.np;
    for (int32_t lane = 0; lane < omega; lane++) {
        int32_t ly = 0;
        uint32_t d = d0[lane];
        int32_t yo = (int32_t)(d >> (32 - g.byo));
        d <<= bao;
        d = lane ? d : (d | 0x80000000u);
        if (((d >> 31) & 1u) && lane) {
            tdo[optr + yo] = c5_rel_row(rp, rs, re, t * omega * sigma + lane * sigma);
            yo++;
        }
        for (int32_t i = 1; i < sigma; i++) {
            if ((!ly && i == bbf) || (ly && !(31 & (i - bbf)))) {
                ly++;
                d = d0[(size_t)ly * omega + lane];
            }
            const int32_t ni = 31 & (!ly ? i : i - bbf);
            if ((d >> (31 - ni)) & 1u) {
                tdo[optr + yo] = c5_rel_row(rp, rs, re, t * omega * sigma + lane * sigma + i);
                yo++;
            }
        }
    }
}

template <typename T>
__global__ void c5_transpose(int64_t nnz, int32_t p, int32_t sigma, int32_t omega, const uint32_t *__restrict__ tp,
                             const T *__restrict__ in, T *__restrict__ out) {
    const int64_t tile = (int64_t)sigma * omega;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t = div_nonneg(k, (int)tile);
        if (t >= p - 1 || tp[t] == tp[t + 1]) {
            out[k] = in[k];
        } else {
            const int64_t q = k - t * tile, y = div_nonneg(q, omega), x = q - y * omega;  // destination (y, x)
            out[k] = in[t * tile + x * sigma + y];
        }
    }
}

// ------------------------------------------------------------------ SpMV --
struct C5View {
    int32_t m, n, p, sigma, byo, bao, np;
    int32_t xvec;  // X rows aligned for vector loads (xrow_vec), set per call
    const int32_t *rp, *col;
    const void *val;
    const uint32_t *tp, *td;
    const int32_t *tdo_ptr, *tdo;
};

template <int OMEGA>
__device__ __forceinline__ uint32_t c5_bit(const uint32_t *d, int lane, int i, int bao, uint32_t d0) {
    // bit for position i of this lane (packet 0 holds positions 0..31-bao)
    const int glid = i + bao;
    const uint32_t w = glid < 32 ? d0 : d[(glid / 32) * OMEGA + lane];
    return (w >> (31 - glid % 32)) & 1u;
}

// SIG > 0: sigma known at compile time (16 or 32, descriptors of at most two
// packets), so a lane's loop over its sigma nonzeros unrolls fully.
template <typename V, int K, int OMEGA, int SIG, bool PLAIN = false>
__global__ void __launch_bounds__(kBlock) csr5_tile_kernel(C5View A, const V *__restrict__ x, int64_t ldx, V alpha,
                                                         V beta, V *__restrict__ y, int64_t ldy,
                                                         int32_t *__restrict__ carry_row, int32_t *__restrict__ has_end,
                                                         V *__restrict__ carry_val, V *__restrict__ head_val) {
    constexpr int kGroups = 32 / OMEGA;
    const int lane = threadIdx.x & 31;
    const int g = lane / OMEGA, xl = lane % OMEGA;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t t = warp * kGroups + g;
    const bool active = t < (int64_t)A.p - 1;
    const V *val = (const V *)A.val;
    const int sigma = SIG > 0 ? SIG : A.sigma;
    const int64_t tile = (int64_t)sigma * OMEGA;
    const int64_t base = t * tile;

    uint32_t tp0 = 0, tp1 = 0, d0 = 0;
    int32_t yoff = 0;
    if (active) {
        tp0 = A.tp[t];
        tp1 = A.tp[t + 1];
        d0 = A.td[(size_t)t * OMEGA * A.np + xl];
        yoff = (int32_t)(d0 >> (32 - A.byo));
        if (xl == 0) yoff = 0;
    }
    const bool fast = tp0 == tp1;
    const bool dirty = (tp0 >> 31) & 1u;
    const int32_t row_start = (int32_t)(tp0 & 0x7FFFFFFFu);
    const uint32_t *dl = A.td + (size_t)t * OMEGA * A.np;
    const int32_t optr = (active && dirty) ? A.tdo_ptr[t] : 0;
    // segment rel >= 1 of a tile with empty rows: tile_desc_offset holds its
    // row counted from row_start + 1 (include/sparse_conversion.h:1290-1305)
    auto map_row = [&](int32_t rel) -> int64_t {
        if (rel == 0) return row_start;
        return (int64_t)row_start + (dirty ? 1 + A.tdo[optr + rel - 1] : rel);
    };

    V sum[K], head[K];
#pragma unroll
    for (int q = 0; q < K; q++) sum[q] = head[q] = V(0);
    bool seen = false;
    int32_t rel = yoff;
    // With at most two descriptor packets the lane's flags for positions
    // 0..sigma-1 fit one 64-bit window: position i at bit 63 - i.
    const bool window = SIG > 0 || A.np <= 2;
    uint64_t bits = 0;
    if (active && window)
        bits = ((uint64_t)d0 << 32 | (A.np > 1 ? dl[OMEGA + xl] : 0u)) << A.bao;
    auto bit_at = [&](int i) -> uint32_t {
        if (window) return (uint32_t)(bits >> (63 - i)) & 1u;
        return c5_bit<OMEGA>(dl, xl, i, A.bao, d0);
    };
    const uint32_t bit0 = active ? bit_at(0) : 0u;
    if (active) {
        // lane xl's i-th nonzero: p0 + i * step (tiles inside one row are
        // stored untransposed)
        const int64_t p0 = fast ? base + (int64_t)xl * sigma : base + xl;
        const int64_t step = fast ? 1 : OMEGA;
        // nonzeros whose loads (and x gathers) are in flight together: 8 for
        // f32 at k = 1; 4 otherwise (deeper prefetch measured slower for f64)
        constexpr int kU = (sizeof(V) == 4 && K == 1) ? 8 : 4;
#pragma unroll
        for (int i0 = 0; i0 < sigma; i0 += kU) {
            int cc[kU];
            V aa[kU], xv[kU][K];
#pragma unroll
            for (int u = 0; u < kU; u++) {
                const int i = i0 + u;
                cc[u] = 0;
                aa[u] = V(0);
                if (i < sigma) {
                    const int64_t idx = p0 + (int64_t)i * step;
                    cc[u] = ld_stream(A.col + idx);
                    aa[u] = ld_stream(val + idx);
                }
            }
#pragma unroll
            for (int u = 0; u < kU; u++) {
                if (i0 + u < sigma) {
                    ld_xrow<V, K>(x, cc[u], ldx, A.xvec != 0, xv[u]);
                } else {
#pragma unroll
                    for (int q = 0; q < K; q++) xv[u][q] = V(0);
                }
            }
#pragma unroll
            for (int u = 0; u < kU; u++) {
                const int i = i0 + u;
                if (i >= sigma) break;
                const uint32_t b = (xl == 0 && i == 0) ? 0u : (i == 0 ? bit0 : bit_at(i));
                if (b) {
                    if (!seen) {
#pragma unroll
                        for (int q = 0; q < K; q++) head[q] = sum[q];
                        seen = true;
                    } else {
                        V *yp = y + map_row(rel) * ldy;
#pragma unroll
                        for (int q = 0; q < K; q++) yp[q] = row_out(PLAIN, alpha, sum[q], beta, yp + q);
                    }
                    rel++;
#pragma unroll
                    for (int q = 0; q < K; q++) sum[q] = V(0);
                }
#pragma unroll
                for (int q = 0; q < K; q++) sum[q] += aa[u] * xv[u][q];
            }
        }
    }
    // segmented inclusive scan of the lanes' trailing runs, keyed by segment
    int32_t key = rel;
    // runs of equal keys never cross a tile's lanes (its first lane is flagged)
    const int32_t key_up = __shfl_up_sync(0xffffffffu, key, 1, OMEGA);  // every lane shuffles (full mask)
    const int span = unflagged_run(xl == 0 || key_up != key);
#pragma unroll
    for (int o = 1; o < OMEGA; o <<= 1) {
        if (o > span) break;  // warp-uniform
        const int32_t k2 = __shfl_up_sync(0xffffffffu, key, o, OMEGA);
        V v2[K];
#pragma unroll
        for (int q = 0; q < K; q++) v2[q] = __shfl_up_sync(0xffffffffu, sum[q], o, OMEGA);
        if (xl >= o && k2 == key) {
#pragma unroll
            for (int q = 0; q < K; q++) sum[q] += v2[q];
        }
    }
    const int32_t kprev = __shfl_up_sync(0xffffffffu, key, 1, OMEGA);
    V sprev[K];
#pragma unroll
    for (int q = 0; q < K; q++) sprev[q] = __shfl_up_sync(0xffffffffu, sum[q], 1, OMEGA);
    const uint32_t tile_bit0 = __shfl_sync(0xffffffffu, bit0, g * OMEGA, 32);
    const bool carry = xl > 0 && kprev == yoff;
    if (active && seen) {  // the segment numbered yoff closes at this lane's first start bit
        V tot[K];
#pragma unroll
        for (int q = 0; q < K; q++) tot[q] = head[q] + (carry ? sprev[q] : V(0));
        if (yoff == 0 && !tile_bit0) {
            V *hp = head_val + t * kMaxK;  // the tile's first row began in an earlier tile
#pragma unroll
            for (int q = 0; q < K; q++) hp[q] = tot[q];
        } else {
            V *yp = y + map_row(yoff) * ldy;
#pragma unroll
            for (int q = 0; q < K; q++) yp[q] = row_out(PLAIN, alpha, tot[q], beta, yp + q);
        }
    }
    if (active && xl == OMEGA - 1) {  // the tile's last run
        const int64_t r = map_row(key);
        const int64_t tile_end = base + tile;
        const bool continues = (int64_t)A.rp[r + 1] > tile_end;
        has_end[t] = (key > 0 || !continues) ? 1 : 0;
        if (continues) {
            carry_row[t] = (int32_t)r;
            V *cp = carry_val + t * kMaxK;
#pragma unroll
            for (int q = 0; q < K; q++) cp[q] = sum[q];
        } else {
            carry_row[t] = -1;
            if (key == 0 && !tile_bit0) {
                V *hp = head_val + t * kMaxK;
#pragma unroll
                for (int q = 0; q < K; q++) hp[q] = sum[q];
            } else {
                V *yp = y + r * ldy;
#pragma unroll
                for (int q = 0; q < K; q++) yp[q] = row_out(PLAIN, alpha, sum[q], beta, yp + q);
            }
        }
    }
}

__global__ void count_empty_rows(int64_t rows, const int32_t *__restrict__ rp, unsigned long long *out) {
    unsigned long long c = 0;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x)
        c += rp[r] == rp[r + 1];
    c = warp_sum(c);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

// y = beta*y on the empty rows before the tail tile (thread per row).
template <typename V, int K>
__global__ void __launch_bounds__(kBlock) csr5_empty_rows(int64_t rows, const int32_t *__restrict__ rp, V beta,
                                                        V *__restrict__ y, int64_t ldy) {
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x)
        if (ld_stream(rp + r) == ld_stream(rp + r + 1)) {
            V *yp = y + r * ldy;
#pragma unroll
            for (int q = 0; q < K; q++) yp[q] = beta == V(0) ? V(0) : beta * yp[q];
        }
}

// Rows from the tail tile on (CSR dot products, warp per row; the first one is
// clipped to the tail when it began earlier).
template <typename V, int K>
__global__ void __launch_bounds__(kBlock) csr5_rows_kernel(C5View A, int32_t tail_row, int64_t tail_start,
                                                         const V *__restrict__ x, int64_t ldx, V alpha, V beta,
                                                         V *__restrict__ y, int64_t ldy, int32_t *__restrict__ has_end,
                                                         V *__restrict__ head_val) {
    const int lane = threadIdx.x & 31;
    const V *val = (const V *)A.val;
    for (int64_t r = tail_row + (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5); r < A.m;
         r += ((int64_t)gridDim.x * blockDim.x) >> 5) {
        const int32_t rs = A.rp[r], re = A.rp[r + 1];
        const bool clipped = r == tail_row && rs < tail_start;
        const int64_t s0 = clipped ? tail_start : rs;
        V s[K];
#pragma unroll
        for (int q = 0; q < K; q++) s[q] = V(0);
        for (int64_t j = s0 + lane; j < re; j += 32) {
            const V a = ld_stream(val + j);
            V xr[K];
            ld_xrow<V, K>(x, ld_stream(A.col + j), ldx, A.xvec != 0, xr);
#pragma unroll
            for (int q = 0; q < K; q++) s[q] += a * xr[q];
        }
#pragma unroll
        for (int q = 0; q < K; q++) s[q] = warp_sum(s[q]);
        if (lane == 0) {
            if (clipped) {
                V *hp = head_val + (int64_t)(A.p - 1) * kMaxK;
#pragma unroll
                for (int q = 0; q < K; q++) hp[q] = s[q];
                has_end[A.p - 1] = 1;
            } else {
                V *yp = y + r * ldy;
#pragma unroll
                for (int q = 0; q < K; q++) yp[q] = axpby(alpha, s[q], beta, yp + q);
            }
        }
    }
}

// Tiles 0..p-2 may leave a carry; the walk may reach the tail tile p-1, whose
// head piece the row pass stored.
template <typename V, int K>
__global__ void csr5_fixup(int32_t ntiles, int64_t tile, const int32_t *__restrict__ rp,
                           const int32_t *__restrict__ carry_row, const int32_t *__restrict__ has_end,
                           const V *__restrict__ carry_val, const V *__restrict__ head_val, V alpha, V beta,
                           V *__restrict__ y, int64_t ldy) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t - (threadIdx.x & 31) >= ntiles - 1) return;  // whole warp past the last full tile
    const int32_t r = t < ntiles - 1 ? carry_row[t] : -1;
    const bool mine = r >= 0 && (int64_t)rp[r] >= t * tile;  // open here and began in tile t
    V tot[K];
    chain_sum<V, K>(mine, t, ntiles, 0, has_end, carry_val, head_val, tot);
    if (mine) {
        V *yp = y + (int64_t)r * ldy;
#pragma unroll
        for (int q = 0; q < K; q++) yp[q] = axpby(alpha, tot[q], beta, yp + q);
    }
}

C5View view_of(const sspmv_csr5 *A) {
    C5View v;
    v.xvec = 0;
    v.m = (int32_t)A->f.num_rows;
    v.n = (int32_t)A->f.num_cols;
    v.p = A->_p;
    v.sigma = A->sigma;
    v.byo = A->bit_y_offset;
    v.bao = A->bit_y_offset + A->bit_scansum_offset;
    v.np = A->num_packets;
    v.rp = A->row_offset;
    v.col = A->col_index;
    v.val = A->values;
    v.tp = A->tile_ptr;
    v.td = A->tile_desc;
    v.tdo_ptr = A->tile_desc_offset_ptr;
    v.tdo = A->tile_desc_offset;
    return v;
}

// plan: extra[0] carry_row+has_end ints (2p), extra[1] carry_val, extra[2] head_val
sspmv_status ensure_c5_plan(const sspmv_csr5 *A, Plan *pl, sspmv_stream_t s) {
    if (pl->extra[0]) return SSPMV_OK;
    std::lock_guard<PlanMutex> g(plan_mutex());
    if (pl->extra[0]) return SSPMV_OK;
    const int64_t p = std::max<int64_t>(A->_p, 1);
    const size_t sv = vsize(A->f.value_type);
    int32_t *ints = nullptr;
    unsigned char *cv = nullptr, *hv = nullptr;
    SSPMV_TRY(dalloc(&ints, (size_t)p * 2, s));
    SSPMV_TRY(dalloc(&cv, (size_t)p * kMaxK * sv, s));
    SSPMV_TRY(dalloc(&hv, (size_t)p * kMaxK * sv, s));
    SSPMV_CUDA_TRY(cudaMemsetAsync(ints, 0, (size_t)p * 8, cu(s)));
    // empty rows before the tail tile (they get y = beta*y in a separate pass)
    const int64_t tail_row = A->_p > 0 ? A->tail_partition_start : 0;
    unsigned long long *cnt = nullptr, h = 0;
    SSPMV_TRY(dalloc(&cnt, 1, s));
    SSPMV_CUDA_TRY(cudaMemsetAsync(cnt, 0, 8, cu(s)));
    if (tail_row > 0) {
        count_empty_rows<<<grid_for(tail_row, 256, (int64_t)num_sms() * 16), 256, 0, cu(s)>>>(tail_row, A->row_offset,
                                                                                             cnt);
        note_launch();
    }
    SSPMV_CUDA_TRY(cudaMemcpyAsync(&h, cnt, 8, cudaMemcpyDeviceToHost, cu(s)));
    SSPMV_CUDA_TRY(cudaStreamSynchronize(cu(s)));
    dfree(cnt, s);
    pl->extra_i[3] = (int64_t)h;
    pl->extra[1] = cv;
    pl->extra[2] = hv;
    pl->extra[0] = ints;
    return SSPMV_OK;
}

template <typename V, int K, int OMEGA>
sspmv_status launch_c5_tiles(const C5View &v, V alpha, const V *x, int64_t ldx, V beta, V *y, int64_t ldy,
                             int32_t *cr, int32_t *he, V *cv, V *hv, sspmv_stream_t s) {
    const int64_t tiles = v.p - 1;
    const int64_t warps = (tiles + (32 / OMEGA) - 1) / (32 / OMEGA);
    const unsigned grid = grid_for(warps * 32, kBlock);
    const int sig = (v.np <= 2 && (v.sigma == 16 || v.sigma == 32)) ? v.sigma : 0;
    if constexpr (K == 1) {  // one right-hand side: sigma-specialised kernels
        if (sig == 16) {
            if (alpha == V(1) && beta == V(0))
                csr5_tile_kernel<V, K, OMEGA, 16, true><<<grid, kBlock, 0, cu(s)>>>(v, x, ldx, alpha, beta, y, ldy, cr,
                                                                                   he, cv, hv);
            else
                csr5_tile_kernel<V, K, OMEGA, 16><<<grid, kBlock, 0, cu(s)>>>(v, x, ldx, alpha, beta, y, ldy, cr, he,
                                                                              cv, hv);
            SSPMV_LAUNCH_CHECK();
            return SSPMV_OK;
        }
        if (sig == 32) {
            if (alpha == V(1) && beta == V(0))
                csr5_tile_kernel<V, K, OMEGA, 32, true><<<grid, kBlock, 0, cu(s)>>>(v, x, ldx, alpha, beta, y, ldy, cr,
                                                                                   he, cv, hv);
            else
                csr5_tile_kernel<V, K, OMEGA, 32><<<grid, kBlock, 0, cu(s)>>>(v, x, ldx, alpha, beta, y, ldy, cr, he,
                                                                              cv, hv);
            SSPMV_LAUNCH_CHECK();
            return SSPMV_OK;
        }
    }
    csr5_tile_kernel<V, K, OMEGA, 0><<<grid, kBlock, 0, cu(s)>>>(v, x, ldx, alpha, beta, y, ldy, cr, he, cv, hv);
    SSPMV_LAUNCH_CHECK();
    return SSPMV_OK;
}

template <typename V, int K>
sspmv_status csr5_pass(const sspmv_csr5 *A, Plan *pl, V alpha, const V *x, int64_t ldx, V beta, V *y, int64_t ldy,
                       sspmv_stream_t s) {
    SSPMV_TRY(ensure_c5_plan(A, pl, s));
    C5View v = view_of(A);
    v.xvec = xrow_vec(x, ldx, sizeof(V), K);
    const int64_t p = std::max<int64_t>(A->_p, 1);
    int32_t *cr = (int32_t *)pl->extra[0], *he = cr + p;
    V *cv = (V *)pl->extra[1], *hv = (V *)pl->extra[2];
    if (A->_p > 1) {
        switch (A->omega) {
        case 4: SSPMV_TRY((launch_c5_tiles<V, K, 4>(v, alpha, x, ldx, beta, y, ldy, cr, he, cv, hv, s))); break;
        case 8: SSPMV_TRY((launch_c5_tiles<V, K, 8>(v, alpha, x, ldx, beta, y, ldy, cr, he, cv, hv, s))); break;
        case 16: SSPMV_TRY((launch_c5_tiles<V, K, 16>(v, alpha, x, ldx, beta, y, ldy, cr, he, cv, hv, s))); break;
        case 32: SSPMV_TRY((launch_c5_tiles<V, K, 32>(v, alpha, x, ldx, beta, y, ldy, cr, he, cv, hv, s))); break;
        default: return fail(SSPMV_NOT_SUPPORTED, "CSR5 SpMV supports omega in {4, 8, 16, 32}");
        }
    }
    const int64_t tail_start = A->_p > 0 ? (int64_t)(A->_p - 1) * A->sigma * A->omega : 0;
    const int32_t tail_row = A->_p > 0 ? A->tail_partition_start : 0;
    if (pl->extra_i[3] > 0) {  // empty rows before the tail tile
        csr5_empty_rows<V, K><<<grid_for(tail_row, kBlock, (int64_t)num_sms() * 16), kBlock, 0, cu(s)>>>(
            tail_row, A->row_offset, beta, y, ldy);
        SSPMV_LAUNCH_CHECK();
    }
    csr5_rows_kernel<V, K><<<grid_for((A->f.num_rows - tail_row) * 32, kBlock, (int64_t)num_sms() * 32), kBlock, 0,
                             cu(s)>>>(v, tail_row, tail_start, x, ldx, alpha, beta, y, ldy, he, hv);
    SSPMV_LAUNCH_CHECK();
    if (A->_p > 1) {
        csr5_fixup<V, K><<<grid_for(A->_p - 1, 256), 256, 0, cu(s)>>>(A->_p, (int64_t)A->sigma * A->omega,
                                                                     A->row_offset, cr, he, cv, hv, alpha, beta, y,
                                                                     ldy);
        SSPMV_LAUNCH_CHECK();
    }
    return SSPMV_OK;
}

}  // namespace

extern "C" sspmv_status sspmv_csr_to_csr5(const sspmv_csr *csr, int32_t sigma, int32_t omega, sspmv_csr5 *out,
                                          sspmv_stream_t s) {
    if (!csr || !out) return fail(SSPMV_INVALID_ARG, "null argument");
    SSPMV_TRY(check_dims(csr->f.value_type, csr->f.num_rows, csr->f.num_cols, csr->f.num_nnzs));
    if (sigma == 0) sigma = 16;
    if (omega == 0) omega = default_alignment(csr->f.value_type);
    if (sigma < 1 || omega < 1 || omega > 32) return fail(SSPMV_INVALID_ARG, "sigma >= 1, 1 <= omega <= 32 required");
    const int64_t m = csr->f.num_rows, nnz = csr->f.num_nnzs;
    const int32_t vt = csr->f.value_type;
    const size_t sv = vsize(vt);
    sspmv_csr5 A;
    std::memset(&A, 0, sizeof(A));
    init_features(&A.f, vt, m, csr->f.num_cols, nnz, 1);
    A.sigma = sigma;
    A.omega = omega;
    // include/sparse_conversion.h:977-996
    int32_t base = 2;
    A.bit_y_offset = 1;
    while (base < sigma * omega) { base *= 2; A.bit_y_offset++; }
    base = 2;
    A.bit_scansum_offset = 1;
    while (base < omega) { base *= 2; A.bit_scansum_offset++; }
    if (A.bit_y_offset + A.bit_scansum_offset > 31) return fail(SSPMV_INVALID_ARG, "CSR5 omega too large for bit fields");
    A.num_packets = (A.bit_y_offset + A.bit_scansum_offset + sigma + 31) / 32;
    A._p = (int32_t)((nnz + (int64_t)sigma * omega - 1) / ((int64_t)sigma * omega));
    const int32_t p = A._p;
    Geom g{sigma, omega, A.bit_y_offset, A.bit_scansum_offset, A.num_packets, p};
    uint32_t *tp_tmp = nullptr;
    sspmv_status st = dalloc(&A.row_offset, (size_t)m + 1, s);
    if (st == SSPMV_OK) st = dalloc(&A.col_index, (size_t)nnz, s);
    if (st == SSPMV_OK) st = dalloc((unsigned char **)&A.values, (size_t)nnz * sv, s);
    if (st == SSPMV_OK) st = dalloc(&A.tile_ptr, (size_t)p + 1, s);
    if (st == SSPMV_OK) st = dalloc(&tp_tmp, (size_t)p + 1, s);
    if (st == SSPMV_OK) st = dalloc(&A.tile_desc, (size_t)p * omega * A.num_packets, s);
    if (st == SSPMV_OK) st = dalloc(&A.tile_desc_offset_ptr, (size_t)p + 1, s);
    if (st == SSPMV_OK) {
        cudaMemcpyAsync(A.row_offset, csr->row_offset, ((size_t)m + 1) * 4, cudaMemcpyDeviceToDevice, cu(s));
        cudaMemsetAsync(tp_tmp, 0, ((size_t)p + 1) * 4, cu(s));
        cudaMemsetAsync(A.tile_ptr, 0, ((size_t)p + 1) * 4, cu(s));
        cudaMemsetAsync(A.tile_desc, 0, (size_t)std::max<int64_t>((int64_t)p * omega * A.num_packets, 1) * 4, cu(s));
        cudaMemsetAsync(A.tile_desc_offset_ptr, 0, ((size_t)p + 1) * 4, cu(s));
        if (p > 0) {
            c5_tile_ptr<<<grid_for(p, 256), 256, 0, cu(s)>>>(p, sigma * omega, (int32_t)m, (int32_t)nnz, csr->row_offset,
                                                             tp_tmp);
            c5_dirty<<<grid_for(p, 256), 256, 0, cu(s)>>>(p, csr->row_offset, tp_tmp, A.tile_ptr);
            c5_bits<<<grid_for(m, 256, (int64_t)num_sms() * 16), 256, 0, cu(s)>>>((int32_t)m, p, g, csr->row_offset,
                                                                                  A.tile_desc);
            c5_offsets_pack<<<grid_for(p, 128), 128, 0, cu(s)>>>(p, g, A.tile_ptr, A.tile_desc, A.tile_desc_offset_ptr);
            for (int i = 0; i < 4; i++) note_launch();
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) st = fail(SSPMV_CUDA_ERROR, "csr_to_csr5: %s", cudaGetErrorString(e));
            int32_t total = 0;
            if (st == SSPMV_OK) st = exclusive_scan_i32(A.tile_desc_offset_ptr, A.tile_desc_offset_ptr, p + 1, &total, s);
            A.num_offsets = total;
            uint32_t last = 0;
            if (st == SSPMV_OK) {
                e = cudaMemcpyAsync(&last, A.tile_ptr + p - 1, 4, cudaMemcpyDeviceToHost, cu(s));
                if (e == cudaSuccess) e = cudaStreamSynchronize(cu(s));
                if (e != cudaSuccess) st = fail(SSPMV_CUDA_ERROR, "csr_to_csr5: %s", cudaGetErrorString(e));
            }
            A.tail_partition_start = (int32_t)(last & 0x7FFFFFFFu);
        }
    }
    if (st == SSPMV_OK) st = dalloc(&A.tile_desc_offset, (size_t)A.num_offsets, s);
    if (st == SSPMV_OK && A.num_offsets > 0) {
        cudaMemsetAsync(A.tile_desc_offset, 0, (size_t)A.num_offsets * 4, cu(s));
        c5_desc_offsets<<<grid_for(p, 128), 128, 0, cu(s)>>>(p, g, csr->row_offset, A.tile_ptr, A.tile_desc,
                                                             A.tile_desc_offset_ptr, A.tile_desc_offset);
        note_launch();
    }
    if (st == SSPMV_OK && nnz > 0) {
        const unsigned gn = grid_for(nnz, 256, (int64_t)num_sms() * 16);
        c5_transpose<int32_t><<<gn, 256, 0, cu(s)>>>(nnz, p, sigma, omega, A.tile_ptr, csr->col_index, A.col_index);
        note_launch();
        st = dispatch_value(vt, [&](auto tag) -> sspmv_status {
            using V = decltype(tag);
            c5_transpose<V><<<gn, 256, 0, cu(s)>>>(nnz, p, sigma, omega, A.tile_ptr, (const V *)csr->values,
                                                   (V *)A.values);
            SSPMV_LAUNCH_CHECK();
            return SSPMV_OK;
        });
    }
    if (st == SSPMV_OK) {
        cudaError_t e = cudaStreamSynchronize(cu(s));
        if (e != cudaSuccess) st = fail(SSPMV_CUDA_ERROR, "csr_to_csr5: %s", cudaGetErrorString(e));
    }
    dfree(tp_tmp, s);
    if (st != SSPMV_OK) {
        dfree(A.row_offset, s);
        dfree(A.col_index, s);
        dfree(A.values, s);
        dfree(A.tile_ptr, s);
        dfree(A.tile_desc, s);
        dfree(A.tile_desc_offset_ptr, s);
        dfree(A.tile_desc_offset, s);
        return st;
    }
    *out = A;
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_spmm_csr5(double alpha, const sspmv_csr5 *A, int32_t k, const void *X, int64_t ldx,
                                        double beta, void *Y, int64_t ldy, sspmv_stream_t s) {
    if (!A) return fail(SSPMV_INVALID_ARG, "null matrix");
    SSPMV_TRY(check_spmm_args(&A->f, k, X, ldx, Y, ldy));
    if (A->f.num_rows == 0) return SSPMV_OK;
    Plan *pl = get_plan(&A->f);
    if (!pl) return fail(SSPMV_OUT_OF_MEMORY, "plan allocation failed");
    return dispatch_value(A->f.value_type, [&](auto tag) -> sspmv_status {
        using V = decltype(tag);
        return for_rhs_chunks<V>(k, (const V *)X, (V *)Y, [&](int32_t step, const V *xs, V *ys) {
            const V a = (V)alpha, b = (V)beta;
            switch (step) {
            case 8: return csr5_pass<V, 8>(A, pl, a, xs, ldx, b, ys, ldy, s);
            case 4: return csr5_pass<V, 4>(A, pl, a, xs, ldx, b, ys, ldy, s);
            case 2: return csr5_pass<V, 2>(A, pl, a, xs, ldx, b, ys, ldy, s);
            default: return csr5_pass<V, 1>(A, pl, a, xs, ldx, b, ys, ldy, s);
            }
        });
    });
}

extern "C" sspmv_status sspmv_LeSpMV_csr5(double alpha, const sspmv_csr5 *A, const void *x, double beta, void *y,
                                          sspmv_stream_t s) {
    return sspmv_spmm_csr5(alpha, A, 1, x, 1, beta, y, 1, s);
}

extern "C" sspmv_status sspmv_csr5_export(const sspmv_csr5 *A, uint32_t *tile_ptr, uint32_t *tile_desc,
                                          int32_t *tile_desc_offset_ptr, int32_t *tile_desc_offset, int32_t *col_index,
                                          void *values, sspmv_stream_t s) {
    if (!A) return fail(SSPMV_INVALID_ARG, "null matrix");
    auto cp = [&](void *dst, const void *src, size_t bytes) -> sspmv_status {
        if (dst && bytes) SSPMV_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, cu(s)));
        return SSPMV_OK;
    };
    const size_t p = (size_t)A->_p;
    SSPMV_TRY(cp(tile_ptr, A->tile_ptr, (p + 1) * 4));
    SSPMV_TRY(cp(tile_desc, A->tile_desc, p * A->omega * A->num_packets * 4));
    SSPMV_TRY(cp(tile_desc_offset_ptr, A->tile_desc_offset_ptr, (p + 1) * 4));
    SSPMV_TRY(cp(tile_desc_offset, A->tile_desc_offset, (size_t)A->num_offsets * 4));
    SSPMV_TRY(cp(col_index, A->col_index, (size_t)A->f.num_nnzs * 4));
    SSPMV_TRY(cp(values, A->values, (size_t)A->f.num_nnzs * vsize(A->f.value_type)));
    SSPMV_CUDA_TRY(cudaStreamSynchronize(cu(s)));
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_delete_csr5(sspmv_csr5 *A) {
    if (!A) return SSPMV_OK;
    delete_barrier();
    free_plan(&A->f, nullptr);
    if (A->f.owns) {
        dfree(A->row_offset, nullptr);
        dfree(A->col_index, nullptr);
        dfree(A->values, nullptr);
        dfree(A->tile_ptr, nullptr);
        dfree(A->tile_desc, nullptr);
        dfree(A->tile_desc_offset_ptr, nullptr);
        dfree(A->tile_desc_offset, nullptr);
    }
    A->row_offset = A->col_index = A->tile_desc_offset_ptr = A->tile_desc_offset = nullptr;
    A->tile_ptr = A->tile_desc = nullptr;
    A->values = nullptr;
    return SSPMV_OK;
}

extern "C" double sspmv_algorithmic_bytes_csr5(const sspmv_csr5 *A, int32_t k, int32_t beta_nonzero) {
    const double sv = (double)vsize(A->f.value_type);
    return (double)A->f.num_nnzs * (sv + 4.0) + (double)(A->f.num_rows + 1) * 4.0 + (double)(A->_p + 1) * 4.0 +
           (double)A->_p * A->omega * A->num_packets * 4.0 + (double)A->num_offsets * 4.0 +
           (double)k * (double)A->f.num_cols * sv + (double)k * (double)A->f.num_rows * sv * (beta_nonzero ? 2.0 : 1.0);
}
