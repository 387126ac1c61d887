/*
 * oracle_features.c -- CPU restatement of LeSpMV's matrix feature extractor
 * (class MTX, src/sparse_features.cpp:122-853, include/sparse_features.h).
 * TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Input is a general (non-symmetric-file) CSR matrix whose row-major order is
 * the order the reference would read its Matrix Market file in.  Features are
 * computed in double; the integer counts and arrays are exact.  The feature
 * order is the library's (SSPMV_FEATURE_* in include/sspmv.h): the 40 values
 * of the reference's .features file (FeaturesWrite, :1347-1400) followed by
 * the extra statistics the reference computes.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

static int cmp_i64(const void *a, const void *b) {
    int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
    return (x > y) - (x < y);
}

/* P_ratioAndGini (src/sparse_features.cpp:612-640) on a count vector. */
static void p_ratio_gini(const int64_t *vec, int64_t len, int64_t nnz, double *p_ratio, double *gini) {
    int64_t *o = (int64_t *)malloc(sizeof(int64_t) * (size_t)(len > 0 ? len : 1));
    memcpy(o, vec, sizeof(int64_t) * (size_t)len);
    qsort(o, (size_t)len, sizeof(int64_t), cmp_i64);
    int64_t quit = len, step = 0, count = 0;
    double p = 0, q = 0;
    do {
        --quit;
        ++count;
        step += o[quit];
        p = (double)count / (double)len;
        q = (double)step / (double)nnz;
    } while (p + q < 1.0 && quit > 0);
    *p_ratio = p;
    /* trapezoid over the cumulative sums (:88-100): cum_0/2 + sum (cum_i+cum_{i+1})/2 */
    double area = 0, cum = 0, prev = 0;
    for (int64_t i = 0; i < len; i++) {
        cum += (double)o[i];
        if (i == 0) area += cum / 2.0;
        else area += (prev + cum) / 2.0;
        prev = cum;
    }
    double total = (double)nnz * (double)len / 2.0;
    *gini = (total - area) / total;
    free(o);
}

/* Tile index of a row / column: the first t_mod blocks hold one more row
 * (:189-190, :243-244). */
static int64_t tile_of(int64_t i, int64_t num, int64_t mod) {
    int64_t thr = mod * (num + 1);
    return i < thr ? i / (num + 1) : mod + (num ? (i - thr) / num : 0);
}

typedef struct {
    int64_t r, c;
} pair64;

static int cmp_pair(const void *a, const void *b) {
    const pair64 *x = (const pair64 *)a, *y = (const pair64 *)b;
    if (x->r != y->r) return x->r < y->r ? -1 : 1;
    return (x->c > y->c) - (x->c < y->c);
}

void oracle_features(int32_t m, int32_t n, const int32_t *rowptr, const int32_t *col, const double *val, int32_t T,
                     double *F, int32_t *nnz_by_tiles, int32_t *uniq_rb, int32_t *uniq_cb) {
    const int64_t nnz = rowptr[m];
    const int64_t tn_rb = m / T, tm_rb = m % T, tn_cb = n / T, tm_cb = n % T;
    const int64_t TT = (int64_t)T * T;
    int64_t *row_cnt = (int64_t *)calloc((size_t)m + 1, sizeof(int64_t));
    int64_t *col_cnt = (int64_t *)calloc((size_t)n + 1, sizeof(int64_t));
    int64_t *diag = (int64_t *)calloc((size_t)m + n + 1, sizeof(int64_t));
    int64_t *tiles = (int64_t *)calloc((size_t)TT, sizeof(int64_t));
    int64_t *rb = (int64_t *)calloc((size_t)T, sizeof(int64_t));
    int64_t *cb = (int64_t *)calloc((size_t)T, sizeof(int64_t));
    int64_t *urb = (int64_t *)calloc((size_t)TT, sizeof(int64_t));
    int64_t *ucb = (int64_t *)calloc((size_t)TT, sizeof(int64_t));
    double *dom = (double *)calloc((size_t)m + 1, sizeof(double));
    double *maxr = (double *)calloc((size_t)m + 1, sizeof(double));
    double *minr = (double *)calloc((size_t)m + 1, sizeof(double));
    double *maxc = (double *)calloc((size_t)n + 1, sizeof(double));
    double *minc = (double *)calloc((size_t)n + 1, sizeof(double));
    int64_t lower = 0, upper = 0, ondiag = 0;
    double max_off = -1.79769313486231570e308, max_diag = -1.79769313486231570e308;
    /* MtxLoad, general real branch (:336-470) in file (= CSR) order */
    for (int64_t i = 0; i < m; i++) {
        for (int64_t jj = rowptr[i]; jj < rowptr[i + 1]; jj++) {
            const int64_t j = col[jj];
            const double v = val[jj], a = fabs(v);
            row_cnt[i]++;
            col_cnt[j]++;
            diag[j - i + m]++;
            const int64_t tr = tile_of(i, tn_rb, tm_rb), tc = tile_of(j, tn_cb, tm_cb);
            tiles[tr * T + tc]++;
            rb[tr]++;
            cb[tc]++;
            if (i == j) {
                ondiag++;
                if (a > max_diag) max_diag = a;
                dom[i] += a;
            } else {
                if (i > j) lower++;
                else upper++;
                if (a > max_off) max_off = a;
                dom[i] -= a;
            }
            const double lg = log10(a);
            if (maxr[i] < lg) maxr[i] = lg;
            if (a > 0.0 && minr[i] > lg) minr[i] = lg;
            if (maxc[j] < lg) maxc[j] = lg;
            if (a > 0.0 && minc[j] > lg) minc[j] = lg;
        }
    }
    /* uniq_RB / uniq_CB: distinct rows / columns met in each tile (Rows_flag,
     * Cols_flag, :214-232) */
    pair64 *keys = (pair64 *)malloc(sizeof(pair64) * (size_t)(nnz > 0 ? nnz : 1));
    int64_t k = 0;
    for (int64_t i = 0; i < m; i++)
        for (int64_t jj = rowptr[i]; jj < rowptr[i + 1]; jj++, k++) {
            keys[k].r = i;
            keys[k].c = tile_of(col[jj], tn_cb, tm_cb);
        }
    qsort(keys, (size_t)nnz, sizeof(pair64), cmp_pair);
    for (k = 0; k < nnz; k++)
        if (k == 0 || keys[k].r != keys[k - 1].r || keys[k].c != keys[k - 1].c)
            urb[tile_of(keys[k].r, tn_rb, tm_rb) * T + keys[k].c]++;
    k = 0;
    for (int64_t i = 0; i < m; i++)
        for (int64_t jj = rowptr[i]; jj < rowptr[i + 1]; jj++, k++) {
            keys[k].r = col[jj];
            keys[k].c = tile_of(i, tn_rb, tm_rb);
        }
    qsort(keys, (size_t)nnz, sizeof(pair64), cmp_pair);
    for (k = 0; k < nnz; k++)
        if (k == 0 || keys[k].r != keys[k - 1].r || keys[k].c != keys[k - 1].c)
            ucb[keys[k].c * T + tile_of(keys[k].r, tn_cb, tm_cb)]++;
    /* pattern / value symmetry (square only, :722-753): an off-diagonal entry
     * counts when its transpose is present (values compared exactly) */
    int64_t sym_p = 0, sym_v = 0;
    if (m == n) {
        k = 0;
        for (int64_t i = 0; i < m; i++)
            for (int64_t jj = rowptr[i]; jj < rowptr[i + 1]; jj++, k++) {
                keys[k].r = i;
                keys[k].c = col[jj];
            }
        qsort(keys, (size_t)nnz, sizeof(pair64), cmp_pair);
        for (int64_t i = 0; i < m; i++)
            for (int64_t jj = rowptr[i]; jj < rowptr[i + 1]; jj++) {
                const int64_t j = col[jj];
                if (i == j) continue;
                pair64 q = {j, i};
                const pair64 *hit = (const pair64 *)bsearch(&q, keys, (size_t)nnz, sizeof(pair64), cmp_pair);
                if (hit) {
                    sym_p++;
                    /* value of the transpose: first entry (j, i) in CSR order */
                    for (int64_t t = rowptr[j]; t < rowptr[j + 1]; t++)
                        if (col[t] == i) {
                            /* first value inserted for key (i,j) as well */
                            double vij = 0;
                            for (int64_t u = rowptr[i]; u < rowptr[i + 1]; u++)
                                if (col[u] == j) { vij = val[u]; break; }
                            if (val[t] == vij) sym_v++;
                            break;
                        }
                }
            }
    }
    free(keys);
    /* CalculateFeatures (:643-776) */
    const int64_t num_nnzs = nnz;
    int64_t nz_rows = 0, nz_cols = 0, dominance = 0, close = 0, ndiags = 0;
    int64_t min_r = 100000000, max_r = 0, min_c = 100000000, max_c = 0;
    const int64_t close_thr = (int64_t)(m + n - 1) / 20;
    for (int64_t t = 0; t < (int64_t)m + n; t++)
        if (diag[t]) {
            ndiags++;
            if (llabs(t - m) <= close_thr) close += diag[t];
        }
    const double ave_r = (double)num_nnzs / m, ave_c = (double)num_nnzs / n;
    double var_r = 0, var_c = 0, row_div = -1.0, col_div = -1.0;
    for (int64_t i = 0; i < m; i++) {
        if (row_cnt[i] < min_r) min_r = row_cnt[i];
        if (row_cnt[i] > max_r) max_r = row_cnt[i];
        if (row_cnt[i]) nz_rows++;
        if (minr[i]) {
            double t = maxr[i] - minr[i];
            if (t > row_div) row_div = t;
        }
        double d = (double)row_cnt[i] - ave_r;
        var_r += d * d;
        if (dom[i] > 0) dominance++;
    }
    for (int64_t j = 0; j < n; j++) {
        if (col_cnt[j] < min_c) min_c = col_cnt[j];
        if (col_cnt[j] > max_c) max_c = col_cnt[j];
        if (col_cnt[j]) nz_cols++;
        if (minc[j]) {
            double t = maxc[j] - minc[j];
            if (t > col_div) col_div = t;
        }
        double d = (double)col_cnt[j] - ave_c;
        var_c += d * d;
    }
    var_r /= m;
    var_c /= n;
    double pr_r, g_r, pr_c, g_c;
    p_ratio_gini(row_cnt, m, num_nnzs, &pr_r, &g_r);
    p_ratio_gini(col_cnt, n, num_nnzs, &pr_c, &g_c);
    /* CalculateTilesFeatures (:783-853); accumulators start at -1 (quirk) */
    double ave_t = (double)num_nnzs / ((double)T * T), ave_rb = (double)num_nnzs / T, ave_cb = ave_rb;
    double var_t = -1.0, var_rb = -1.0, var_cb = -1.0, nz_t = -1.0, nz_rb = -1.0, nz_cb = -1.0;
    int64_t min_t = 100000000, max_t = 0, min_rb = 100000000, max_rb = 0, min_cb = 100000000, max_cb = 0;
    for (int64_t i = 0; i < T; i++) {
        if (rb[i]) nz_rb += 1;
        if (cb[i]) nz_cb += 1;
        var_rb += (rb[i] - ave_rb) * (rb[i] - ave_rb);
        var_cb += (cb[i] - ave_cb) * (cb[i] - ave_cb);
        if (rb[i] < min_rb) min_rb = rb[i];
        if (rb[i] > max_rb) max_rb = rb[i];
        if (cb[i] < min_cb) min_cb = cb[i];
        if (cb[i] > max_cb) max_cb = cb[i];
    }
    nz_rb /= T;
    var_rb /= T;
    nz_cb /= T;
    var_cb /= T;
    for (int64_t i = 0; i < TT; i++) {
        if (tiles[i]) nz_t += 1;
        var_t += (tiles[i] - ave_t) * (tiles[i] - ave_t);
        if (tiles[i] < min_t) min_t = tiles[i];
        if (tiles[i] > max_t) max_t = tiles[i];
    }
    nz_t /= (double)TT;
    var_t /= (double)TT;
    double pr_t, g_t, pr_rb, g_rb, pr_cb, g_cb;
    p_ratio_gini(tiles, TT, num_nnzs, &pr_t, &g_t);
    p_ratio_gini(rb, T, num_nnzs, &pr_rb, &g_rb);
    p_ratio_gini(cb, T, num_nnzs, &pr_cb, &g_cb);
    int64_t sum_urb = 0, sum_ucb = 0;
    for (int64_t i = 0; i < TT; i++) {
        sum_urb += urb[i];
        sum_ucb += ucb[i];
    }
    /* CalculateTilesExtraFeatures (:942-968): mean over rows of the average
     * column step inside a row */
    double dist = 0;
    for (int64_t i = 0; i < m; i++) {
        const int64_t s = rowptr[i], e = rowptr[i + 1];
        if (e - s < 1) continue;
        int64_t d = 0;
        for (int64_t j = s; j + 1 < e; j++) d += col[j + 1] - col[j];
        dist += (double)d / (double)(e - s);
    }
    dist /= m;

    F[0] = m;
    F[1] = n;
    F[2] = (double)num_nnzs;
    F[3] = (double)num_nnzs / ((double)m * n);
    F[4] = (double)close / num_nnzs;
    F[5] = dist / n;
    F[6] = (double)nz_rows / m;
    F[7] = (double)max_r;
    F[8] = ave_r;
    F[9] = sqrt(var_r);
    F[10] = pr_r;
    F[11] = g_r;
    F[12] = (double)nz_cols / n;
    F[13] = (double)max_c;
    F[14] = ave_c;
    F[15] = sqrt(var_c);
    F[16] = pr_c;
    F[17] = g_c;
    F[18] = nz_t;
    F[19] = (double)max_t;
    F[20] = ave_t;
    F[21] = sqrt(var_t > 0 ? var_t : 0);
    F[22] = pr_t;
    F[23] = g_t;
    F[24] = nz_rb;
    F[25] = (double)max_rb;
    F[26] = ave_rb;
    F[27] = sqrt(var_rb > 0 ? var_rb : 0);
    F[28] = pr_rb;
    F[29] = g_rb;
    F[30] = nz_cb;
    F[31] = (double)max_cb;
    F[32] = ave_cb;
    F[33] = sqrt(var_cb > 0 ? var_cb : 0);
    F[34] = pr_cb;
    F[35] = g_cb;
    F[36] = (double)sum_urb / num_nnzs;
    F[37] = (double)sum_ucb / num_nnzs;
    F[38] = (double)sum_urb / m;
    F[39] = (double)sum_ucb / n;
    F[40] = (double)lower;
    F[41] = (double)upper;
    F[42] = (double)ondiag;
    F[43] = (double)ndiags;
    F[44] = (double)min_r;
    F[45] = (double)min_c;
    F[46] = (double)dominance / (m < n ? m : n);
    F[47] = max_off;
    F[48] = max_diag;
    F[49] = row_div;
    F[50] = col_div;
    F[51] = m == n ? (double)sym_p / (double)(num_nnzs - ondiag) : 0.0;
    F[52] = m == n ? (double)sym_v / (double)(num_nnzs - ondiag) : 0.0;
    F[53] = (double)min_t;
    F[54] = (double)min_rb;
    F[55] = (double)min_cb;
    F[56] = var_r;
    F[57] = var_c;
    F[58] = F[59] = F[60] = F[61] = -1.0; /* GrX: not computed (BSR_ANA disabled) */
    for (int64_t i = 0; i < TT; i++) {
        if (nnz_by_tiles) nnz_by_tiles[i] = (int32_t)tiles[i];
        if (uniq_rb) uniq_rb[i] = (int32_t)urb[i];
        if (uniq_cb) uniq_cb[i] = (int32_t)ucb[i];
    }
    free(row_cnt);
    free(col_cnt);
    free(diag);
    free(tiles);
    free(rb);
    free(cb);
    free(urb);
    free(ucb);
    free(dom);
    free(maxr);
    free(minr);
    free(maxc);
    free(minc);
}

/* BestDimForBSR (src/sparse_features.cpp:858-880). */
static int64_t best_dim_for_bsr(int64_t nums, int64_t target) {
    int64_t best = 0, best_diff = 10000;
    for (int64_t dim = 1; dim < nums; dim++) {
        int64_t mb = (nums + dim - 1) / dim;
        int64_t diff = mb > target ? mb - target : target - mb;
        if (diff < best_diff) {
            best_diff = diff;
            best = dim;
        }
        if (diff == 0) break;
    }
    return best > 0 ? best : 1;
}

/* AnalyzeTile_Group (src/sparse_features.cpp:884-934) on one dense R x Cd tile. */
static void analyze_tile_group(const double *t, int64_t R, int64_t Cd, int64_t X, long long *gr, long long *gc,
                               int flag_row, int flag_col) {
    if (flag_row) {
        for (int64_t bc = 0; bc < Cd; ++bc) {
            for (int64_t br = 0; br < R; br++) {
                if (t[br * Cd + bc] != 0) {
                    if (br + X <= R) {
                        int64_t step;
                        for (step = 1; step < X; step++)
                            if (t[(br + step) * Cd + bc] == 0) break;
                        if (step == X) ++*gr;
                        br += step;
                    } else {
                        break;
                    }
                }
            }
        }
    }
    if (flag_col) {
        for (int64_t br = 0; br < R; br++) {
            for (int64_t bc = 0; bc < Cd; ++bc) {
                if (t[br * Cd + bc] != 0) {
                    if (bc + X <= Cd) {
                        int64_t step;
                        for (step = 1; step < X; step++)
                            if (t[br * Cd + bc + step] == 0) break;
                        if (step == X) ++*gc;
                        bc += step;
                    } else {
                        break;
                    }
                }
            }
        }
    }
}

void oracle_grx(int32_t m, int32_t n, const int32_t *rowptr, const int32_t *col, const double *val, int32_t T,
                int32_t X, double *out) {
    const int64_t R = best_dim_for_bsr(m, T), Cd = best_dim_for_bsr(n, T);
    const int64_t mb = (m + R - 1) / R, nb = (n + Cd - 1) / Cd;
    const int flag_r = R >= X, flag_c = Cd >= X;
    const int64_t gpr = flag_r ? (R + X - 1) / X : 0, gpc = flag_c ? (Cd + X - 1) / X : 0;
    const int64_t nnz = rowptr[m];
    long long gr = 0, gc = 0;
    long long *pot_r = (long long *)calloc((size_t)(mb * gpr + 1), sizeof(long long));
    long long *pot_c = (long long *)calloc((size_t)(nb * gpc + 1), sizeof(long long));
    double *tile = (double *)calloc((size_t)(R * Cd), sizeof(double));
    char *seen = (char *)calloc((size_t)nb, 1);
    int64_t *touched = (int64_t *)malloc(sizeof(int64_t) * (size_t)nb);
    char *fr = (char *)malloc((size_t)(gpr + 1)), *fc = (char *)malloc((size_t)(gpc + 1));
    for (int64_t i = 0; i < mb; i++) {
        const int64_t r0 = i * R, r1 = r0 + R < m ? r0 + R : m;
        int64_t nt = 0;
        for (int64_t r = r0; r < r1; r++)
            for (int64_t q = rowptr[r]; q < rowptr[r + 1]; q++) {
                const int64_t j = col[q] / Cd;
                if (!seen[j]) {
                    seen[j] = 1;
                    touched[nt++] = j;
                }
            }
        for (int64_t u = 0; u < nt; u++) {
            const int64_t j = touched[u];
            seen[j] = 0;
            for (int64_t r = r0; r < r1; r++)
                for (int64_t q = rowptr[r]; q < rowptr[r + 1]; q++)
                    if (col[q] / Cd == j) tile[(r - r0) * Cd + (col[q] - j * Cd)] = val[q];
            /* potReuse flags: one count per tile for each row / column group holding a nonzero (:1030-1042) */
            memset(fr, 1, (size_t)(gpr + 1));
            memset(fc, 1, (size_t)(gpc + 1));
            for (int64_t br = 0; br < R; br++)
                for (int64_t bc = 0; bc < Cd; bc++)
                    if (tile[br * Cd + bc] != 0) {
                        if (flag_r && fr[br / X]) {
                            pot_r[i * gpr + br / X]++;
                            fr[br / X] = 0;
                        }
                        if (flag_c && fc[bc / X]) {
                            pot_c[j * gpc + bc / X]++;
                            fc[bc / X] = 0;
                        }
                    }
            analyze_tile_group(tile, R, Cd, X, &gr, &gc, flag_r, flag_c);
            for (int64_t r = r0; r < r1; r++)
                for (int64_t q = rowptr[r]; q < rowptr[r + 1]; q++)
                    if (col[q] / Cd == j) tile[(r - r0) * Cd + (col[q] - j * Cd)] = 0;
        }
    }
    long long sr = 0, sc = 0;
    for (int64_t k = 0; k < mb * gpr; k++) sr += pot_r[k];
    for (int64_t k = 0; k < nb * gpc; k++) sc += pot_c[k];
    out[0] = flag_r ? (double)gr / (double)nnz : -1.0;
    out[1] = flag_c ? (double)gc / (double)nnz : -1.0;
    out[2] = flag_r ? (double)sr / (double)(mb * gpr) : -1.0;
    out[3] = flag_c ? (double)sc / (double)(nb * gpc) : -1.0;
    free(pot_r);
    free(pot_c);
    free(tile);
    free(seen);
    free(touched);
    free(fr);
    free(fc);
}
