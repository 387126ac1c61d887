/*
 * oracle.c -- CPU restatement of LeSpMV's structural conversion steps.
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  Value-typed steps live in
 * oracle_values.inc, included once per value type at the end of this file.
 *
 * Each routine cites the reference routine it restates (paths relative to the
 * LeSpMV project).  The restatements reproduce the reference's outputs,
 * including its quirks (tie order of the SELL sort, first-encounter DIA
 * diagonal order, CSR5 bit layout and the unset tile_ptr[_p]).
 */
#include "oracle.h"
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static int resolve_threads(int nthreads) {
    if (nthreads > 0) return nthreads;
    return oracle_max_threads();
}

/* include/sparse_conversion.h:197-203 */
int32_t oracle_ell_width(int32_t m, const int32_t *rowptr) {
    int32_t w = 0;
    for (int32_t i = 0; i < m; i++) {
        int32_t l = rowptr[i + 1] - rowptr[i];
        if (l > w) w = l;
    }
    return w;
}

static int32_t align_up(int32_t v, int32_t a) { return ((v + a - 1) / a) * a; }

/* include/sparse_conversion.h:272-296 */
int64_t oracle_sell_row_width(int32_t m, const int32_t *rowptr, int32_t C,
                              int32_t align, int32_t *row_width) {
    int32_t nchunks = (m + C - 1) / C;
    int64_t total = 0;
    for (int32_t c = 0; c < nchunks; c++) row_width[c] = 0;
    for (int32_t i = 0; i < m; i++) {
        int32_t l = rowptr[i + 1] - rowptr[i];
        if (l > row_width[i / C]) row_width[i / C] = l;
    }
    for (int32_t c = 0; c < nchunks; c++) {
        row_width[c] = align_up(row_width[c], align);
        total += (int64_t)row_width[c] * C;
    }
    return total;
}

typedef struct { int32_t nnz, row; } nnz_row_pair;

/* std::greater<std::pair<nnz,row>>: nnz descending, then row descending. */
static int cmp_pair_greater(const void *a, const void *b) {
    const nnz_row_pair *x = (const nnz_row_pair *)a, *y = (const nnz_row_pair *)b;
    if (x->nnz != y->nnz) return x->nnz > y->nnz ? -1 : 1;
    if (x->row != y->row) return x->row > y->row ? -1 : 1;
    return 0;
}

/* include/sparse_conversion.h:355-400 (SELL-c-sigma) and :501-523 (SELL-c-R) */
int oracle_sell_cs_reorder(int32_t m, const int32_t *rowptr, int32_t sigma,
                           int32_t C, int32_t *reorder) {
    if (sigma > 0 && (sigma % C) != 0) return -1;
    int32_t slice = sigma > 0 ? sigma : (m > 0 ? m : 1);
    nnz_row_pair *pairs = (nnz_row_pair *)malloc(sizeof(nnz_row_pair) * (size_t)(m > 0 ? m : 1));
    for (int32_t i = 0; i < m; i++) {
        pairs[i].nnz = rowptr[i + 1] - rowptr[i];
        pairs[i].row = i;
    }
    for (int64_t s = 0; s < m; s += slice) {
        int64_t e = s + slice < m ? s + slice : m;
        qsort(pairs + s, (size_t)(e - s), sizeof(nnz_row_pair), cmp_pair_greater);
    }
    for (int32_t i = 0; i < m; i++) reorder[i] = pairs[i].row;
    free(pairs);
    return 0;
}

/* include/sparse_conversion.h:405-433 */
int64_t oracle_sell_cs_chunk_len(int32_t m, const int32_t *rowptr,
                                 const int32_t *reorder, int32_t C,
                                 int32_t align, int32_t *chunk_len) {
    int32_t nchunks = (m + C - 1) / C;
    int64_t total = 0;
    for (int32_t c = 0; c < nchunks; c++) chunk_len[c] = 0;
    for (int32_t i = 0; i < m; i++) {
        int32_t r = reorder[i];
        int32_t l = rowptr[r + 1] - rowptr[r];
        if (l > chunk_len[i / C]) chunk_len[i / C] = l;
    }
    for (int32_t c = 0; c < nchunks; c++) {
        chunk_len[c] = align_up(chunk_len[c], align);
        total += (int64_t)chunk_len[c] * C;
    }
    return total;
}

/* include/sparse_conversion.h:626-649 */
int32_t oracle_dia_map(int32_t m, int32_t n, const int32_t *rowptr,
                       const int32_t *col, int32_t *diag_map) {
    int32_t nd = 0;
    for (int64_t t = 0; t < (int64_t)m + n; t++) diag_map[t] = -1;
    for (int32_t i = 0; i < m; i++) {
        for (int32_t jj = rowptr[i]; jj < rowptr[i + 1]; jj++) {
            int64_t idx = (int64_t)(m - i) + col[jj];
            if (diag_map[idx] == -1) diag_map[idx] = nd++;
        }
    }
    return nd;
}

static int cmp_i32(const void *a, const void *b) {
    int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

/* Distinct block columns of block row br, ascending (the reference marks a
 * dense nb-long flag vector and scans it, include/sparse_conversion.h:824-846). */
static int32_t bsr_block_cols(const int32_t *rowptr, const int32_t *col,
                              int32_t m, int32_t br, int32_t r, int32_t c,
                              unsigned char *flag, int32_t nb, int32_t *out) {
    int32_t s = rowptr[(int64_t)br * r];
    int64_t erow = (int64_t)br * r + r;
    if (erow > m) erow = m;
    int32_t e = rowptr[erow];
    int32_t cnt = 0;
    for (int32_t j = s; j < e; j++) flag[col[j] / c] = 1;
    /* collect in ascending order: scan touched columns via the flag vector */
    for (int32_t j = s; j < e; j++) {
        int32_t b = col[j] / c;
        if (flag[b] == 1) { flag[b] = 2; if (out) out[cnt] = b; cnt++; }
    }
    for (int32_t j = s; j < e; j++) flag[col[j] / c] = 0;
    (void)nb;
    if (out && cnt > 1) qsort(out, (size_t)cnt, sizeof(int32_t), cmp_i32);
    return cnt;
}

/* include/sparse_conversion.h:784-800 (r=c=1) and :817-848 */
int32_t oracle_bsr_row_ptr(int32_t m, int32_t n, const int32_t *rowptr,
                           const int32_t *col, int32_t r, int32_t c,
                           int32_t *row_ptr) {
    int32_t mb = (m + r - 1) / r, nb = (n + c - 1) / c;
    if (r == 1 && c == 1) {
        for (int32_t i = 0; i <= m; i++) row_ptr[i] = rowptr[i];
        return row_ptr[mb] - row_ptr[0];
    }
    unsigned char *flag = (unsigned char *)calloc((size_t)(nb > 0 ? nb : 1), 1);
    row_ptr[0] = 0;
    for (int32_t b = 0; b < mb; b++)
        row_ptr[b + 1] = bsr_block_cols(rowptr, col, m, b, r, c, flag, nb, NULL);
    for (int32_t b = 0; b < mb; b++) row_ptr[b + 1] += row_ptr[b];
    free(flag);
    return row_ptr[mb] - row_ptr[0];
}

/* include/sparse_conversion.h:861-888 (r=c=1: :805-813 copies col_index) */
void oracle_bsr_colindex(int32_t m, int32_t n, const int32_t *rowptr,
                         const int32_t *col, int32_t r, int32_t c,
                         const int32_t *row_ptr, int32_t *colindex) {
    int32_t mb = (m + r - 1) / r, nb = (n + c - 1) / c;
    if (r == 1 && c == 1) {
        for (int32_t j = 0; j < rowptr[m]; j++) colindex[j] = col[j];
        return;
    }
    unsigned char *flag = (unsigned char *)calloc((size_t)(nb > 0 ? nb : 1), 1);
    for (int32_t b = 0; b < mb; b++)
        bsr_block_cols(rowptr, col, m, b, r, c, flag, nb, colindex + row_ptr[b]);
    free(flag);
}

/* ---------------- CSR5 (include/sparse_conversion.h:939-1379) ---------------- */

/* :958-996 */
int oracle_csr5_geometry(int32_t nnz, int32_t sigma, int32_t omega,
                         oracle_csr5_geom *g) {
    memset(g, 0, sizeof(*g));
    g->sigma = sigma;
    g->omega = omega;
    int32_t base = 2;
    g->bit_y_offset = 1;
    while (base < sigma * omega) { base *= 2; g->bit_y_offset++; }
    base = 2;
    g->bit_scansum_offset = 1;
    while (base < omega) { base *= 2; g->bit_scansum_offset++; }
    if (g->bit_y_offset + g->bit_scansum_offset > 31) return -1;
    int32_t bit_all = g->bit_y_offset + g->bit_scansum_offset + sigma;
    g->num_packets = (int32_t)ceil((double)bit_all / 32.0);
    g->p = (int32_t)ceil((double)nnz / (double)(omega * sigma));
    return 0;
}

/* Row holding nonzero `boundary` (last row whose offset <= boundary),
 * the binary search at :1029-1044. */
static int32_t csr5_row_search(const int32_t *rowptr, int32_t m, int32_t boundary) {
    int32_t start = 0, stop = m, median;
    while (stop >= start) {
        median = (stop + start) / 2;
        if (boundary >= rowptr[median]) start = median + 1;
        else stop = median - 1;
    }
    return start - 1;
}

void oracle_csr5_descriptors(int32_t m, const int32_t *rowptr,
                             oracle_csr5_geom *g, uint32_t *tile_ptr,
                             uint32_t *tile_desc,
                             int32_t *tile_desc_offset_ptr) {
    const int32_t p = g->p, sigma = g->sigma, omega = g->omega, np = g->num_packets;
    const int32_t nnz = rowptr[m];
    const int32_t tile = sigma * omega;
    memset(tile_ptr, 0, sizeof(uint32_t) * (size_t)(p + 1));
    memset(tile_desc, 0, sizeof(uint32_t) * (size_t)p * omega * np);
    memset(tile_desc_offset_ptr, 0, sizeof(int32_t) * (size_t)(p + 1));

    /* step 1.1 (:1024-1045): tile_ptr[_p] is never written by the reference */
    for (int32_t t = 0; t < p; t++) {
        int64_t b = (int64_t)t * tile;
        if (b > nnz) b = nnz;
        tile_ptr[t] = (uint32_t)csr5_row_search(rowptr, m, (int32_t)b);
    }
    /* step 1.2 (:1048-1075): mark tiles that contain empty rows */
    for (int32_t t = 0; t < p; t++) {
        uint32_t start = tile_ptr[t] & 0x7FFFFFFFu;
        uint32_t stop = tile_ptr[t + 1] & 0x7FFFFFFFu;
        if (start == stop) continue;
        int dirty = 0;
        for (uint32_t r = start; r <= stop; r++) {
            if (rowptr[r] == rowptr[r + 1]) { dirty = 1; break; }
        }
        if (dirty) tile_ptr[t] = start | 0x80000000u;
    }
    g->tail_partition_start = p > 0 ? (int32_t)(tile_ptr[p - 1] & 0x7FFFFFFFu) : 0;

    const int32_t bit_all_offset = g->bit_y_offset + g->bit_scansum_offset;
    /* step 2.1 (:1086-1111): one bit per row start */
    for (int32_t t = 0; t < p - 1; t++) {
        int32_t rs = (int32_t)(tile_ptr[t] & 0x7FFFFFFFu);
        int32_t re = (int32_t)(tile_ptr[t + 1] & 0x7FFFFFFFu);
        for (int32_t rid = rs; rid <= re; rid++) {
            int32_t ptr = rowptr[rid];
            int32_t pid = ptr / tile;
            if (pid == t) {
                int32_t lx = (ptr / sigma) % omega;
                int32_t glid = ptr % sigma + bit_all_offset;
                int32_t ly = glid / 32, llid = glid % 32;
                tile_desc[(size_t)pid * omega * np + (size_t)ly * omega + lx] |= 1u << (31 - llid);
            }
        }
    }
    /* step 2.2 (:1113-1213): y_offset and scansum_offset per lane */
    int32_t *segn = (int32_t *)malloc(sizeof(int32_t) * (size_t)(omega + 1));
    int32_t *present = (int32_t *)malloc(sizeof(int32_t) * (size_t)(omega + 1));
    for (int32_t t = 0; t < p - 1; t++) {
        int with_empty = (int)((tile_ptr[t] >> 31) & 1u);
        int32_t rs = (int32_t)(tile_ptr[t] & 0x7FFFFFFFu);
        int32_t re = (int32_t)(tile_ptr[t + 1] & 0x7FFFFFFFu);
        if (rs == re) continue;
        for (int32_t l = 0; l <= omega; l++) { segn[l] = 0; present[l] = 0; }
        present[omega] = 1;
        uint32_t *td = tile_desc + (size_t)t * omega * np;
        for (int32_t lane = 0; lane < omega; lane++) {
            int32_t start, stop = 0, ly = 0;
            int32_t pres = (lane == 0);
            uint32_t bitflag = (td[lane] << bit_all_offset) | ((uint32_t)pres << 31);
            start = !((bitflag >> 31) & 1u);
            pres |= (int32_t)((bitflag >> 31) & 1u);
            for (int32_t i = 1; i < sigma; i++) {
                if ((!ly && i == 32 - bit_all_offset) ||
                    (ly && (i - (32 - bit_all_offset)) % 32 == 0)) {
                    ly++;
                    bitflag = td[(size_t)ly * omega + lane];
                }
                int32_t norm_i = !ly ? i : i - (32 - bit_all_offset);
                stop += (int32_t)((bitflag >> (31 - norm_i % 32)) & 1u);
                pres |= (int32_t)((bitflag >> (31 - norm_i % 32)) & 1u);
            }
            int32_t s = stop - start + pres;
            segn[lane] = s > 0 ? s : 0;
            present[lane] = pres;
        }
        /* exclusive scan over omega+1 entries */
        int32_t run = 0;
        for (int32_t l = 0; l <= omega; l++) { int32_t v = segn[l]; segn[l] = run; run += v; }
        if (with_empty) {
            tile_desc_offset_ptr[t] = segn[omega];
            tile_desc_offset_ptr[p] += segn[omega];
        }
        for (int32_t lane = 0; lane < omega; lane++) {
            int32_t y_offset = segn[lane], scansum = 0, next1 = lane + 1;
            if (present[lane]) {
                while (!present[next1] && next1 < omega) { scansum++; next1++; }
            }
            y_offset = lane ? y_offset - 1 : 0;
            uint32_t fp = td[lane];
            fp |= (uint32_t)y_offset << (32 - g->bit_y_offset);
            fp |= (uint32_t)scansum << (32 - bit_all_offset);
            td[lane] = fp;
        }
    }
    free(segn);
    free(present);
    /* :1217-1229 exclusive scan of tile_desc_offset_ptr when any tile is dirty */
    if (tile_desc_offset_ptr[p]) {
        int32_t run = 0;
        for (int32_t t = 0; t <= p; t++) {
            int32_t v = tile_desc_offset_ptr[t];
            tile_desc_offset_ptr[t] = run;
            run += v;
        }
    }
    g->num_offsets = tile_desc_offset_ptr[p];
}

/* Relative row of nonzero idx inside [rs, re], the search at :1290-1303. */
static int32_t csr5_rel_row(const int32_t *rowptr, int32_t rs, int32_t re, int32_t idx) {
    int32_t start = 0, stop = re - rs - 1, median;
    while (stop >= start) {
        median = (stop + start) / 2;
        if (idx >= rowptr[rs + 1 + median]) start = median + 1;
        else stop = median - 1;
    }
    return start - 1;
}

/* :1254-1358 */
void oracle_csr5_offsets(int32_t m, const int32_t *rowptr,
                         const oracle_csr5_geom *g, const uint32_t *tile_ptr,
                         const uint32_t *tile_desc,
                         const int32_t *tile_desc_offset_ptr,
                         int32_t *tile_desc_offset) {
    (void)m;
    const int32_t p = g->p, sigma = g->sigma, omega = g->omega, np = g->num_packets;
    const int32_t bit_all_offset = g->bit_y_offset + g->bit_scansum_offset;
    const int32_t bit_bitflag = 32 - bit_all_offset;
    if (!g->num_offsets) return;
    for (int32_t t = 0; t < p - 1; t++) {
        if (!((tile_ptr[t] >> 31) & 1u)) continue;
        int32_t rs = (int32_t)(tile_ptr[t] & 0x7FFFFFFFu);
        int32_t re = (int32_t)(tile_ptr[t + 1] & 0x7FFFFFFFu);
        int32_t optr = tile_desc_offset_ptr[t];
        const uint32_t *td = tile_desc + (size_t)t * omega * np;
        for (int32_t lane = 0; lane < omega; lane++) {
            int32_t ly = 0;
            uint32_t d = td[lane];
            int32_t y_offset = (int32_t)(d >> (32 - g->bit_y_offset));
            d <<= bit_all_offset;
            d = lane ? d : (d | 0x80000000u);
            int32_t bit = (int32_t)((d >> 31) & 1u);
            if (bit && lane) {
                int32_t idx = t * omega * sigma + lane * sigma;
                tile_desc_offset[optr + y_offset] = csr5_rel_row(rowptr, rs, re, idx);
                y_offset++;
            }
            for (int32_t i = 1; i < sigma; i++) {
                if ((!ly && i == bit_bitflag) || (ly && !(31 & (i - bit_bitflag)))) {
                    ly++;
                    d = td[(size_t)ly * omega + lane];
                }
                int32_t norm_i = 31 & (!ly ? i : i - bit_bitflag);
                bit = (int32_t)((d >> (31 - norm_i)) & 1u);
                if (bit) {
                    int32_t idx = t * omega * sigma + lane * sigma + i;
                    tile_desc_offset[optr + y_offset] = csr5_rel_row(rowptr, rs, re, idx);
                    y_offset++;
                }
            }
        }
    }
}

/* include/csr5_utils.h:11-87 (R2C): element (lane x, position y) of a tile,
 * stored at x*sigma+y in CSR order, moves to y*omega+x.  Tiles whose tile_ptr
 * words are equal ("fast track") and the last tile are left as they are. */
void oracle_csr5_transpose(int32_t nnz, const oracle_csr5_geom *g,
                           const uint32_t *tile_ptr, void *data,
                           int32_t elem_size) {
    (void)nnz;
    const int32_t sigma = g->sigma, omega = g->omega, tile = sigma * omega;
    unsigned char *buf = (unsigned char *)malloc((size_t)tile * elem_size);
    unsigned char *d = (unsigned char *)data;
    for (int32_t t = 0; t < g->p - 1; t++) {
        if (tile_ptr[t] == tile_ptr[t + 1]) continue;
        unsigned char *base = d + (size_t)t * tile * elem_size;
        for (int32_t x = 0; x < omega; x++)
            for (int32_t y = 0; y < sigma; y++)
                memcpy(buf + ((size_t)y * omega + x) * elem_size,
                       base + ((size_t)x * sigma + y) * elem_size, (size_t)elem_size);
        memcpy(base, buf, (size_t)tile * elem_size);
    }
    free(buf);
}

/* ---------------- value-typed steps ---------------- */
#define V double
#define S f64
#include "oracle_values.inc"
#undef V
#undef S
#define V float
#define S f32
#include "oracle_values.inc"
#undef V
#undef S
