/*
 * ref_harness.cpp -- thin extern "C" wrapper around the reference's OWN
 * converters and SpMV kernels (LeSpMV, compiled from its sources by the
 * `ref` target of oracle/Makefile into oracle/_ref/libref.so).
 *
 * TEST INFRASTRUCTURE ONLY.  It is used in the development container to pin
 * the oracle restatement (oracle.c) and to write the golden fixtures under
 * tests/golden/.  It is never part of the product and is not built on
 * machines where the reference sources are absent.
 *
 * Outputs are malloc'd copies returned through ref_out; sliced formats are
 * flattened chunk by chunk (each chunk row-major as the reference stores it).
 * Free every returned array with ref_free().
 */
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>
#include <iostream>
// The feature extractor keeps its results in private members of class MTX;
// the harness reads them directly (same class layout, access opened).
#define private public
#include "LeSpMV.h"
#undef private

extern "C" {

typedef struct {
    int64_t ints[16];
    void *arrays[8];
    int64_t lens[8];
} ref_out;

void ref_free(void *p) { free(p); }
/* The reference sizes per-thread scratch by Le_get_thread_num() but runs its
 * loops under the OpenMP default team size (include/csr5_utils.h:23-32), so
 * both are set together. */
void ref_set_threads(int n) {
    Le_set_thread_num(n);
    omp_set_num_threads(n);
}

}  // extern "C"

template <typename T>
static T *dup(const T *src, int64_t n) {
    T *d = (T *)malloc(sizeof(T) * (size_t)(n > 0 ? n : 1));
    if (n > 0) memcpy(d, src, sizeof(T) * (size_t)n);
    return d;
}

template <typename V>
static CSR_Matrix<int, V> view_csr(int m, int n, const int *rp, const int *ci, const V *v) {
    CSR_Matrix<int, V> csr;
    csr.num_rows = m;
    csr.num_cols = n;
    csr.num_nnzs = rp[m];
    csr.row_offset = const_cast<int *>(rp);
    csr.col_index = const_cast<int *>(ci);
    csr.values = const_cast<V *>(v);
    csr.kernel_flag = 1;
    csr.partition = nullptr;
    return csr;
}

template <typename V>
static void do_coo_to_csr(int m, int n, int nnz, const int *ri, const int *ci, const V *v, ref_out *o) {
    COO_Matrix<int, V> coo;
    coo.num_rows = m; coo.num_cols = n; coo.num_nnzs = nnz;
    coo.row_index = const_cast<int *>(ri);
    coo.col_index = const_cast<int *>(ci);
    coo.values = const_cast<V *>(v);
    CSR_Matrix<int, V> csr = coo_to_csr(coo, false);
    o->arrays[0] = dup(csr.row_offset, (int64_t)m + 1); o->lens[0] = (int64_t)m + 1;
    o->arrays[1] = dup(csr.col_index, nnz); o->lens[1] = nnz;
    o->arrays[2] = dup(csr.values, nnz); o->lens[2] = nnz;
    delete_csr_matrix(csr);
}

template <typename V>
static void do_ell(int m, int n, const int *rp, const int *ci, const V *v, int ld, ref_out *o) {
    auto csr = view_csr(m, n, rp, ci, v);
    ELL_Matrix<int, V> ell = csr_to_ell(csr, ld == 1 ? ColMajor : RowMajor);
    int64_t tot = (int64_t)m * ell.max_row_width;
    o->ints[0] = ell.max_row_width;
    o->arrays[0] = dup(ell.col_index, tot); o->lens[0] = tot;
    o->arrays[1] = dup(ell.values, tot); o->lens[1] = tot;
    delete_ell_matrix(ell);
}

template <typename V>
static void do_sell(int m, int n, const int *rp, const int *ci, const V *v, int C, int align, ref_out *o) {
    auto csr = view_csr(m, n, rp, ci, v);
    S_ELL_Matrix<int, V> s = csr_to_sell(csr, nullptr, C, align);
    int64_t tot = 0;
    for (int c = 0; c < s.chunk_num; c++) tot += (int64_t)s.row_width[c] * C;
    int *cf = (int *)malloc(sizeof(int) * (size_t)(tot > 0 ? tot : 1));
    V *vf = (V *)malloc(sizeof(V) * (size_t)(tot > 0 ? tot : 1));
    int64_t b = 0;
    for (int c = 0; c < s.chunk_num; c++) {
        int64_t k = (int64_t)s.row_width[c] * C;
        memcpy(cf + b, s.col_index[c], sizeof(int) * (size_t)k);
        memcpy(vf + b, s.values[c], sizeof(V) * (size_t)k);
        b += k;
    }
    o->ints[0] = s.chunk_num; o->ints[1] = s.sliceWidth; o->ints[2] = s.alignment;
    o->arrays[0] = dup(s.row_width, s.chunk_num); o->lens[0] = s.chunk_num;
    o->arrays[1] = cf; o->lens[1] = tot;
    o->arrays[2] = vf; o->lens[2] = tot;
    delete_s_ell_matrix(s);
}

template <typename M, typename V>
static void flatten_cs(const M &s, int nchunks, int C, ref_out *o, int m) {
    int64_t tot = 0;
    for (int c = 0; c < nchunks; c++) tot += (int64_t)s.chunk_len[c] * C;
    int *cf = (int *)malloc(sizeof(int) * (size_t)(tot > 0 ? tot : 1));
    V *vf = (V *)malloc(sizeof(V) * (size_t)(tot > 0 ? tot : 1));
    int64_t b = 0;
    for (int c = 0; c < nchunks; c++) {
        int64_t k = (int64_t)s.chunk_len[c] * C;
        memcpy(cf + b, s.col_index[c], sizeof(int) * (size_t)k);
        memcpy(vf + b, s.values[c], sizeof(V) * (size_t)k);
        b += k;
    }
    o->arrays[0] = dup(s.reorder, m); o->lens[0] = m;
    o->arrays[1] = dup(s.chunk_len, nchunks); o->lens[1] = nchunks;
    o->arrays[2] = cf; o->lens[2] = tot;
    o->arrays[3] = vf; o->lens[3] = tot;
}

template <typename V>
static void do_sell_cs(int m, int n, const int *rp, const int *ci, const V *v, int sigma, int C, int align, ref_out *o) {
    auto csr = view_csr(m, n, rp, ci, v);
    SELL_C_Sigma_Matrix<int, V> s = csr_to_sell_c_sigma(csr, nullptr, sigma, C, align);
    o->ints[0] = s.sliceNum; o->ints[1] = s.chunkNum; o->ints[2] = s.validchunkNum;
    o->ints[3] = s.chunk_num_per_slice; o->ints[4] = s.alignment;
    flatten_cs<SELL_C_Sigma_Matrix<int, V>, V>(s, s.validchunkNum, C, o, m);
    delete_s_ell_c_sigma_matrix(s);
}

template <typename V>
static void do_sell_cr(int m, int n, const int *rp, const int *ci, const V *v, int C, int align, ref_out *o) {
    auto csr = view_csr(m, n, rp, ci, v);
    SELL_C_R_Matrix<int, V> s = csr_to_sell_c_R(csr, nullptr, C, align);
    o->ints[2] = s.validchunkNum; o->ints[4] = s.alignment;
    flatten_cs<SELL_C_R_Matrix<int, V>, V>(s, s.validchunkNum, C, o, m);
    delete_s_ell_c_R_matrix(s);
}

template <typename V>
static void do_dia(int m, int n, const int *rp, const int *ci, const V *v, int max_diags, int align, ref_out *o) {
    auto csr = view_csr(m, n, rp, ci, v);
    DIA_Matrix<int, V> d = csr_to_dia(csr, max_diags, nullptr, align);
    int64_t tot = (int64_t)d.complete_ndiags * d.stride;
    o->ints[0] = d.complete_ndiags; o->ints[1] = d.stride;
    o->arrays[0] = dup(d.diag_offsets, d.complete_ndiags); o->lens[0] = d.complete_ndiags;
    o->arrays[1] = dup(d.diag_data, tot); o->lens[1] = tot;
    delete_dia_matrix(d);
}

template <typename V>
static void do_bsr(int m, int n, const int *rp, const int *ci, const V *v, int r, int c, ref_out *o) {
    auto csr = view_csr(m, n, rp, ci, v);
    BSR_Matrix<int, V> b = csr_to_bsr(csr, r, c);
    int64_t tot = (int64_t)b.nnzb * r * c;
    o->ints[0] = b.mb; o->ints[1] = b.nb; o->ints[2] = b.nnzb; o->ints[3] = b.blockNNZ;
    o->arrays[0] = dup(b.row_ptr, (int64_t)b.mb + 1); o->lens[0] = (int64_t)b.mb + 1;
    o->arrays[1] = dup(b.block_colindex, b.nnzb); o->lens[1] = b.nnzb;
    o->arrays[2] = dup(b.block_data, tot); o->lens[2] = tot;
    delete_bsr_matrix(b);
}

template <typename V>
static void do_csr5(int m, int n, const int *rp, const int *ci, const V *v, ref_out *o) {
    auto csr = view_csr(m, n, rp, ci, v);
    CSR5_Matrix<int, uint32_t, V> c5 = csr_to_csr5<int, uint32_t, V>(csr, nullptr);
    int nnz = rp[m];
    o->ints[0] = c5.sigma; o->ints[1] = c5.omega; o->ints[2] = c5.bit_y_offset;
    o->ints[3] = c5.bit_scansum_offset; o->ints[4] = c5.num_packets; o->ints[5] = c5._p;
    o->ints[6] = c5.num_offsets; o->ints[7] = c5.tail_partition_start;
    int64_t ntd = (int64_t)c5._p * c5.omega * c5.num_packets;
    o->arrays[0] = dup(c5.tile_ptr, (int64_t)c5._p + 1); o->lens[0] = (int64_t)c5._p + 1;
    o->arrays[1] = dup(c5.tile_desc, ntd); o->lens[1] = ntd;
    o->arrays[2] = dup(c5.tile_desc_offset_ptr, (int64_t)c5._p + 1); o->lens[2] = (int64_t)c5._p + 1;
    o->arrays[3] = dup(c5.tile_desc_offset, c5.num_offsets); o->lens[3] = c5.num_offsets;
    o->arrays[4] = dup(c5.col_index, nnz); o->lens[4] = nnz;
    o->arrays[5] = dup(c5.values, nnz); o->lens[5] = nnz;
    if (c5.num_offsets == 0) c5.tile_desc_offset = nullptr;
    delete_csr5_matrix(c5);
}

/* Convert with the reference converter (its default parameters unless given)
 * and run LeSpMV_<fmt> with the given kernel_flag.  y is in/out. */
template <typename V>
static int do_spmv(const char *fmt, int flag, int p0, int p1, int p2, int m, int n,
                   const int *rp, const int *ci, const V *v, V alpha, const V *x, V beta, V *y) {
    auto csr = view_csr(m, n, rp, ci, v);
    const int align = SIMD_WIDTH / 8 / sizeof(V);
    if (!strcmp(fmt, "csr")) {
        csr.kernel_flag = flag;
        LeSpMV_csr(alpha, csr, x, beta, y);
        delete_array(csr.partition);
    } else if (!strcmp(fmt, "coo")) {
        COO_Matrix<int, V> a = csr_to_coo(csr);
        a.kernel_flag = flag; a.partition = nullptr;
        LeSpMV_coo(alpha, a, x, beta, y);
        delete_coo_matrix(a);
    } else if (!strcmp(fmt, "ell")) {
        ELL_Matrix<int, V> a = csr_to_ell(csr, p0 == 1 ? ColMajor : RowMajor);
        a.kernel_flag = flag; a.partition = nullptr;
        LeSpMV_ell(alpha, a, x, beta, y);
        delete_ell_matrix(a);
    } else if (!strcmp(fmt, "sell")) {
        S_ELL_Matrix<int, V> a = csr_to_sell(csr, nullptr, p0 > 0 ? p0 : CHUNK_SIZE, p1 > 0 ? p1 : align);
        a.kernel_flag = flag; a.partition = nullptr;
        LeSpMV_sell(alpha, a, x, beta, y);
        delete_s_ell_matrix(a);
    } else if (!strcmp(fmt, "sell_c_sigma")) {
        SELL_C_Sigma_Matrix<int, V> a = csr_to_sell_c_sigma(csr, nullptr, p0 > 0 ? p0 : SELL_SIGMA,
                                                             p1 > 0 ? p1 : CHUNK_SIZE, p2 > 0 ? p2 : align);
        a.kernel_flag = flag; a.partition = nullptr;
        LeSpMV_sell_c_sigma(alpha, a, x, beta, y);
        delete_s_ell_c_sigma_matrix(a);
    } else if (!strcmp(fmt, "sell_c_R")) {
        SELL_C_R_Matrix<int, V> a = csr_to_sell_c_R(csr, nullptr, p0 > 0 ? p0 : CHUNK_SIZE, p1 > 0 ? p1 : align);
        a.kernel_flag = flag; a.partition = nullptr;
        LeSpMV_sell_c_R(alpha, a, x, beta, y);
        delete_s_ell_c_R_matrix(a);
    } else if (!strcmp(fmt, "dia")) {
        DIA_Matrix<int, V> a = csr_to_dia(csr, (int)MAX_DIAG_NUM, nullptr, align);
        a.kernel_flag = flag; a.partition = nullptr;
        LeSpMV_dia(alpha, a, x, beta, y);
        delete_dia_matrix(a);
    } else if (!strcmp(fmt, "bsr")) {
        BSR_Matrix<int, V> a = csr_to_bsr(csr, p0 > 0 ? p0 : BSR_BlockDimRow, p1 > 0 ? p1 : align);
        a.kernel_flag = flag; a.partition = nullptr;
        LeSpMV_bsr(alpha, a, x, beta, y);
        delete_bsr_matrix(a);
    } else {
        return -1;
    }
    return 0;
}

template <typename V>
static int do_read(const char *path, ref_out *o) {
    CSR_Matrix<int, V> csr = read_csr_matrix<int, V>(path);
    o->ints[0] = csr.num_rows; o->ints[1] = csr.num_cols; o->ints[2] = csr.num_nnzs;
    o->arrays[0] = dup(csr.row_offset, (int64_t)csr.num_rows + 1); o->lens[0] = (int64_t)csr.num_rows + 1;
    o->arrays[1] = dup(csr.col_index, csr.num_nnzs); o->lens[1] = csr.num_nnzs;
    o->arrays[2] = dup(csr.values, csr.num_nnzs); o->lens[2] = csr.num_nnzs;
    delete_csr_matrix(csr);
    return 0;
}

/* MTX feature extraction of a Matrix Market file (MtxLoad + CalculateFeatures
 * + CalculateTilesExtraFeatures, src/sparse_features.cpp), in the library's
 * feature order (62 values); arrays: nnz_by_Tiles_, uniq_RB, uniq_CB. */
template <typename V>
static int do_features(const char *path, double *F, ref_out *o) {
    MTX<int, V> x;
    if (!x.MtxLoad(path)) return -1;
    x.CalculateFeatures();
    x.CalculateTilesExtraFeatures(path);
    double v[62] = {
        (double)x.num_rows, (double)x.num_cols, (double)x.num_nnzs, (double)x.nnz_ratio_,
        (double)x.diag_close_ratio_, (double)x.distance_per_row_ / x.num_cols, (double)x.nz_row_ratio_,
        (double)x.max_nnz_each_row_, (double)x.ave_nnz_each_row_, (double)x.standard_dev_row_,
        (double)x.P_ratio_row_, (double)x.Gini_row_, (double)x.nz_col_ratio_, (double)x.max_nnz_each_col_,
        (double)x.ave_nnz_each_col_, (double)x.standard_dev_col_, (double)x.P_ratio_col_, (double)x.Gini_col_,
        (double)x.t_nz_ratio_tiles_, (double)x.t_max_nnz_all_tiles_, (double)x.t_ave_nnz_all_tiles,
        (double)x.t_standard_dev_all_tiles, (double)x.t_P_ratio_all_tiles_, (double)x.t_Gini_all_tiles_,
        (double)x.t_nz_ratio_RB_, (double)x.t_max_nnz_each_RB_, (double)x.t_ave_nnz_RB, (double)x.t_standard_dev_RB,
        (double)x.t_P_ratio_RB_, (double)x.t_Gini_RB_, (double)x.t_nz_ratio_CB_, (double)x.t_max_nnz_each_CB_,
        (double)x.t_ave_nnz_CB, (double)x.t_standard_dev_CB, (double)x.t_P_ratio_CB_, (double)x.t_Gini_CB_,
        (double)x.uniqR, (double)x.uniqC, (double)x.potReuseR, (double)x.potReuseC,
        (double)x.nnz_lower_, (double)x.nnz_upper_, (double)x.nnz_diagonal_, (double)x.complete_ndiags,
        (double)x.min_nnz_each_row_, (double)x.min_nnz_each_col_, (double)x.diagonal_dominant_ratio_,
        (double)x.max_value_offdiag_, (double)x.max_value_diagonal_, (double)x.row_variability_,
        (double)x.col_variability_, (double)x.pattern_symm_, (double)x.value_symm_,
        (double)x.t_min_nnz_all_tiles_, (double)x.t_min_nnz_each_RB_, (double)x.t_min_nnz_each_CB_,
        (double)x.var_nnz_each_row_, (double)x.var_nnz_each_col_, (double)x.GrX_uniqR, (double)x.GrX_uniqC,
        (double)x.GrX_potReuseR, (double)x.GrX_potReuseC};
    memcpy(F, v, sizeof(v));
    o->ints[0] = x.t_num_blocks;
    o->arrays[0] = dup(x.nnz_by_Tiles_.data(), (int64_t)x.nnz_by_Tiles_.size());
    o->lens[0] = (int64_t)x.nnz_by_Tiles_.size();
    o->arrays[1] = dup(x.uniq_RB.data(), (int64_t)x.uniq_RB.size());
    o->lens[1] = (int64_t)x.uniq_RB.size();
    o->arrays[2] = dup(x.uniq_CB.data(), (int64_t)x.uniq_CB.size());
    o->lens[2] = (int64_t)x.uniq_CB.size();
    return 0;
}

extern "C" int ref_features_f64(const char *path, double *F, ref_out *o) { return do_features<double>(path, F, o); }
extern "C" int ref_features_f32(const char *path, double *F, ref_out *o) { return do_features<float>(path, F, o); }

#define REF_EXPORT(V, S)                                                                      \
    extern "C" void ref_coo_to_csr_##S(int m, int n, int nnz, const int *ri, const int *ci,       \
                                       const V *v, ref_out *o) { do_coo_to_csr<V>(m, n, nnz, ri, ci, v, o); } \
    extern "C" void ref_csr_to_ell_##S(int m, int n, const int *rp, const int *ci, const V *v,    \
                                       int ld, ref_out *o) { do_ell<V>(m, n, rp, ci, v, ld, o); } \
    extern "C" void ref_csr_to_sell_##S(int m, int n, const int *rp, const int *ci, const V *v,   \
                                        int C, int al, ref_out *o) { do_sell<V>(m, n, rp, ci, v, C, al, o); } \
    extern "C" void ref_csr_to_sell_c_sigma_##S(int m, int n, const int *rp, const int *ci,       \
                                                const V *v, int sg, int C, int al, ref_out *o) {  \
        do_sell_cs<V>(m, n, rp, ci, v, sg, C, al, o); }                                           \
    extern "C" void ref_csr_to_sell_c_R_##S(int m, int n, const int *rp, const int *ci,           \
                                            const V *v, int C, int al, ref_out *o) {              \
        do_sell_cr<V>(m, n, rp, ci, v, C, al, o); }                                               \
    extern "C" void ref_csr_to_dia_##S(int m, int n, const int *rp, const int *ci, const V *v,    \
                                       int md, int al, ref_out *o) { do_dia<V>(m, n, rp, ci, v, md, al, o); } \
    extern "C" void ref_csr_to_bsr_##S(int m, int n, const int *rp, const int *ci, const V *v,    \
                                       int r, int c, ref_out *o) { do_bsr<V>(m, n, rp, ci, v, r, c, o); } \
    extern "C" void ref_csr_to_csr5_##S(int m, int n, const int *rp, const int *ci, const V *v,   \
                                        ref_out *o) { do_csr5<V>(m, n, rp, ci, v, o); }           \
    extern "C" int ref_spmv_##S(const char *fmt, int flag, int p0, int p1, int p2, int m, int n,  \
                                const int *rp, const int *ci, const V *v, V alpha, const V *x,    \
                                V beta, V *y) {                                                    \
        return do_spmv<V>(fmt, flag, p0, p1, p2, m, n, rp, ci, v, alpha, x, beta, y); }            \
    extern "C" int ref_read_csr_##S(const char *path, ref_out *o) { return do_read<V>(path, o); }

REF_EXPORT(double, f64)
REF_EXPORT(float, f32)
