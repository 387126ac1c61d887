// sliced.cu -- ELL, S-ELL, SELL-c-sigma and SELL-c-R on sm_103a: GPU
// converters from CSR, SpMV / SpMM kernels, export to the reference layout.
//
// All four share one device layout: a slab of chunks, chunk c holding C rows
// in slot-major order (slot k of the chunk's row r at chunk_ptr[c] + k*C + r,
// padding col -1 / value 0 after each row's last nonzero).  ELL is the case
// of one chunk of C = num_rows rows (the reference's column-major ELL).
// A thread owns one (stored) row: the C threads of a chunk read C consecutive
// slots per step, and a warp covers 32/C chunks.  A row stops at its first
// padding slot, so padding costs at most one partially used sector per row
// instead of being streamed.  SELL variants write y through `reorder`.
//
// Converters (bit-exact logical content vs the reference):
//   ELL          include/sparse_conversion.h:187-248
//   S-ELL        include/sparse_conversion.h:258-334
//   SELL-c-sigma include/sparse_conversion.h:337-479 (sort: nnz desc, row desc)
//   SELL-c-R     include/sparse_conversion.h:483-598
// The per-slice sort is a stable LSD radix sort of keys
// slice*(maxlen+1) + (maxlen - len) over rows fed in descending row order.
#include <algorithm>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "plan.cuh"
#include "primitives.cuh"
#include "serve.cuh"
#include "spmv_common.cuh"

namespace sspmv {
sspmv_status check_dims(int32_t vt, int64_t m, int64_t n, int64_t nnz);
void init_features(sspmv_features *f, int32_t vt, int64_t m, int64_t n, int64_t nnz, int32_t owns);
}  // namespace sspmv

using namespace sspmv;

namespace {

constexpr int kBlock = 256;

// ------------------------------------------------------------------ SpMV --
// A thread per stored row reads its slots (C consecutive rows read together)
// up to its first padding slot, so a warp runs as long as its longest row.
// Where a few long rows would keep most lanes of their warps idle, the
// thread pass stops at a cap (chosen once per matrix by choose_cap): the rest
// of each longer row (its "overflow") is copied once into compact arrays.
// Short tails form a CSR matrix multiplied by the CSR stream kernel (every
// lane busy whatever the row lengths); long tails are cut into pieces of one
// row, a warp each; a fix-up adds each overflow row's thread partial and the
// rest.  The compact copy also skips the padding of the short rows that
// share a long row's chunk (slot-major storage puts them in the same sectors).
constexpr int kSlots = 4;  // slots of a row whose loads are in flight together

template <typename V, int K, bool PLAIN = false>
__global__ void __launch_bounds__(kBlock) sliced_spmv_kernel(
    int m, int C, const int64_t *__restrict__ chunk_ptr, const int32_t *__restrict__ reorder,
    const int32_t *__restrict__ col, const V *__restrict__ val, const V *__restrict__ x, int64_t ldx, int xvec,
    V alpha, V beta, V *__restrict__ y, int64_t ldy, int64_t cap, const int32_t *__restrict__ ovf_id,
    V *__restrict__ ovf_part) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = div_nonneg(i, C);
        const int r = (int)(i - c * C);
        const int64_t base = ld_stream(chunk_ptr + c);
        const int64_t wfull = div_nonneg(ld_stream(chunk_ptr + c + 1) - base, C);
        const int64_t w = min(wfull, cap);
        const int32_t *cp = col + base + r;
        const V *vp = val + base + r;
        V s[K];
#pragma unroll
        for (int q = 0; q < K; q++) s[q] = V(0);
        int64_t k = 0;
        for (; k + kSlots <= w; k += kSlots) {
            int cc[kSlots];
            V aa[kSlots];
#pragma unroll
            for (int u = 0; u < kSlots; u++) {
                cc[u] = ld_stream(cp + (k + u) * C);
                aa[u] = ld_stream(vp + (k + u) * C);
            }
#pragma unroll
            for (int u = 0; u < kSlots; u++)
                if (cc[u] >= 0) {
                    V xr[K];
                    ld_xrow<V, K>(x, cc[u], ldx, xvec, xr);
#pragma unroll
                    for (int q = 0; q < K; q++) s[q] += aa[u] * xr[q];
                }
            if (cc[kSlots - 1] < 0) break;  // padding is a suffix of the row
        }
        if (k + kSlots > w) {
            for (; k < w; k++) {
                const int cc = ld_stream(cp + k * C);
                if (cc < 0) break;
                const V aa = ld_stream(vp + k * C);
                V xr[K];
                ld_xrow<V, K>(x, cc, ldx, xvec, xr);
#pragma unroll
                for (int q = 0; q < K; q++) s[q] += aa * xr[q];
            }
        }
        if (wfull > w && ld_stream(cp + w * C) >= 0) {  // the row goes on past the cap: overflow
            V *op = ovf_part + (int64_t)ovf_id[i] * kMaxK;
#pragma unroll
            for (int q = 0; q < K; q++) op[q] = s[q];
            continue;
        }
        const int64_t row = reorder ? (int64_t)ld_stream(reorder + i) : i;
        V *yp = y + row * ldy;
#pragma unroll
        for (int q = 0; q < K; q++) yp[q] = row_out(PLAIN, alpha, s[q], beta, yp + q);
    }
}

// Long tails (kPieceMin nonzeros or more; 64 measured best against 256, 1024
// and 4096) are cut into pieces of at most kPieceElems nonzeros of one row, a
// warp per piece, lanes on consecutive elements; piece = {overflow row, first
// element, end element} of the compact arrays.
constexpr int64_t kPieceMin = 64;
constexpr int64_t kPieceElems = 2048;

template <typename V, int K>
__global__ void __launch_bounds__(kBlock) sliced_piece_kernel(int64_t npieces, const int4 *__restrict__ pieces,
                                                              const int32_t *__restrict__ ocol,
                                                              const V *__restrict__ oval, const V *__restrict__ x,
                                                              int64_t ldx, int xvec, V *__restrict__ partial) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (warp >= npieces) return;
    const int4 pc = pieces[warp];
    V s[K];
#pragma unroll
    for (int q = 0; q < K; q++) s[q] = V(0);
    int64_t e = (int64_t)pc.y + lane;
    for (; e + 96 < pc.z; e += 128) {
        int cc[4];
        V aa[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            cc[u] = ld_stream(ocol + e + 32 * u);
            aa[u] = ld_stream(oval + e + 32 * u);
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            V xr[K];
            ld_xrow<V, K>(x, cc[u], ldx, xvec, xr);
#pragma unroll
            for (int q = 0; q < K; q++) s[q] += aa[u] * xr[q];
        }
    }
    for (; e < pc.z; e += 32) {
        const int cc = ld_stream(ocol + e);
        const V aa = ld_stream(oval + e);
        V xr[K];
        ld_xrow<V, K>(x, cc, ldx, xvec, xr);
#pragma unroll
        for (int q = 0; q < K; q++) s[q] += aa * xr[q];
    }
#pragma unroll
    for (int q = 0; q < K; q++) s[q] = warp_sum(s[q]);
    if (lane == 0) {
#pragma unroll
        for (int q = 0; q < K; q++) partial[warp * kMaxK + q] = s[q];
    }
}

// One thread per overflow row o: its thread partial plus the rest of the row
// -- the overflow CSR result y_ovf[o] (alpha = 1, beta = 0) for the first
// nshort rows (short tails), the row's pieces in order for the others.
template <typename V, int K>
__global__ void sliced_overflow_fixup(int64_t nov, int64_t nshort, const int32_t *__restrict__ ovf_rows,
                                      const int32_t *__restrict__ reorder, const V *__restrict__ ovf_part,
                                      const V *__restrict__ y_ovf, const int32_t *__restrict__ piece_begin,
                                      const V *__restrict__ partial, V alpha, V beta, V *__restrict__ y,
                                      int64_t ldy) {
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= nov) return;
    V sum[K];
#pragma unroll
    for (int q = 0; q < K; q++) sum[q] = ovf_part[o * kMaxK + q];
    if (o < nshort) {
#pragma unroll
        for (int q = 0; q < K; q++) sum[q] += y_ovf[o * kMaxK + q];
    } else {
        for (int32_t pc = piece_begin[o - nshort]; pc < piece_begin[o - nshort + 1]; pc++)
#pragma unroll
            for (int q = 0; q < K; q++) sum[q] += partial[(int64_t)pc * kMaxK + q];
    }
    const int64_t i = ovf_rows[o];
    const int64_t row = reorder ? (int64_t)reorder[i] : i;
    V *yp = y + row * ldy;
#pragma unroll
    for (int q = 0; q < K; q++) yp[q] = axpby(alpha, sum[q], beta, yp + q);
}

// Plan building: stored length of every stored row (padding is a suffix:
// binary search for the first slot with col < 0).
__global__ void stored_row_lengths(int64_t m, int C, const int64_t *__restrict__ chunk_ptr,
                                   const int32_t *__restrict__ col, int32_t *__restrict__ len) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = div_nonneg(i, C);
        const int r = (int)(i - c * C);
        const int64_t base = chunk_ptr[c];
        const int64_t w = div_nonneg(chunk_ptr[c + 1] - base, C);
        int64_t lo = 0, hi = w;  // first padding slot in [0, w]
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if (col[base + mid * C + r] >= 0) lo = mid + 1;
            else hi = mid;
        }
        len[i] = (int32_t)lo;
    }
}

// Overflow ids of the stored rows: ovf_id[rows[o]] = o.
__global__ void set_overflow_ids(int64_t nov, const int32_t *__restrict__ rows, int32_t *__restrict__ ovf_id) {
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o < nov) ovf_id[rows[o]] = (int32_t)o;
}

// Copies slots cap.. of each overflow row into the compact CSR arrays (one
// warp per row).
template <typename V>
__global__ void copy_overflow(int64_t nov, int C, int64_t cap, const int32_t *__restrict__ ovf_rows,
                              const int32_t *__restrict__ ovf_ptr, const int64_t *__restrict__ chunk_ptr,
                              const int32_t *__restrict__ col, const V *__restrict__ val, int32_t *__restrict__ ocol,
                              V *__restrict__ oval) {
    const int lane = threadIdx.x & 31;
    const int64_t o = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (o >= nov) return;
    const int64_t i = ovf_rows[o];
    const int64_t c = div_nonneg(i, C);
    const int r = (int)(i - c * C);
    const int64_t base = chunk_ptr[c] + cap * C + r;
    const int64_t n = (int64_t)ovf_ptr[o + 1] - ovf_ptr[o], dst = ovf_ptr[o];
    for (int64_t e = lane; e < n; e += 32) {
        ocol[dst + e] = col[base + e * C];
        oval[dst + e] = val[base + e * C];
    }
}

struct SlicedView {
    int64_t m;
    int32_t C;
    const int64_t *chunk_ptr;
    const int32_t *reorder;
    const int32_t *col;
    const void *val;
    int64_t nchunks;
    int64_t n;  // columns
};

// Cost model of the cap, in picoseconds of GB300 time (fitted to measured
// kernel times: the thread pass of S-ELL C=4 on a 4M-row power-law matrix,
// the CSR stream kernel per nonzero on a 4M-row uniform matrix): the thread
// pass costs kWarpSlotPs per warp and slot it runs (a warp runs as many slots
// as its longest row, up to the cap), and no less than its longest thread:
// kIterPs per 4 slots, each step a dependent chain of an HBM load and an x
// gather (a 38k-slot row alone takes ~15 ms); the overflow costs kOvfNnzPs
// per nonzero, kOvfRowPs per row (partial, CSR row, fix-up) and kOvfLaunchPs
// for its extra launches.
constexpr double kWarpSlotPs = 73.0;
constexpr double kIterPs = 1.5e6;
constexpr double kOvfNnzPs = 4.8;
constexpr double kOvfRowPs = 20.0;
constexpr double kOvfLaunchPs = 6.0e6;
constexpr int64_t kCaps[] = {8, 12, 16, 24, 32, 48, 64, 96, 128, 256, 512};
constexpr int64_t kNoCap = INT64_MAX;

// The cap of least modelled time (kNoCap: no overflow), from the stored row
// lengths (stored order: thread i runs stored row i, a warp 32 of them).
int64_t choose_cap(const std::vector<int32_t> &len) {
    const int64_t m = (int64_t)len.size();
    constexpr int32_t H = 1024;  // exact histogram below H; longer rows listed
    std::vector<int64_t> hist(H, 0);
    std::vector<int32_t> longer, wmax((size_t)((m + 31) / 32), 0);
    for (int64_t i = 0; i < m; i++) {
        const int32_t l = len[(size_t)i];
        int32_t &w = wmax[(size_t)(i >> 5)];
        w = std::max(w, l);
        if (l < H) hist[(size_t)l]++;
        else longer.push_back(l);
    }
    double slots = 0;
    int32_t longest = 0;
    for (int32_t w : wmax) {
        slots += w;
        longest = std::max(longest, w);
    }
    auto thread_pass = [&](double warp_slots, int64_t slots_of_longest) {
        return std::max(kWarpSlotPs * warp_slots, kIterPs * (double)((slots_of_longest + 3) / 4));
    };
    double best_cost = thread_pass(slots, longest);
    int64_t best = kNoCap;
    for (int64_t cap : kCaps) {
        double thread = 0, ovn = 0, ovr = 0;
        for (int32_t w : wmax) thread += (double)std::min<int64_t>(w, cap);
        for (int64_t l = cap + 1; l < H; l++) {
            ovn += (double)hist[(size_t)l] * (double)(l - cap);
            ovr += (double)hist[(size_t)l];
        }
        for (int32_t l : longer)
            if (l > cap) {
                ovn += (double)(l - cap);
                ovr += 1;
            }
        const double cost = thread_pass(thread, std::min<int64_t>(longest, cap)) + kOvfNnzPs * ovn +
                            kOvfRowPs * ovr + (ovr > 0 ? kOvfLaunchPs : 0.0);
        if (cost < best_cost) {
            best_cost = cost;
            best = cap;
        }
    }
    return best;
}

void free_overflow(Plan *p, sspmv_stream_t s) {
    if (p->sub) {
        free_plan(&p->sub->f, s);
        delete p->sub;
        p->sub = nullptr;
    }
    for (int e : {0, 1, 2, 3, 4, 5, 6, 7, 8, 9}) {
        dfree(p->extra[e], s);
        p->extra[e] = nullptr;
    }
    p->extra_i[1] = p->extra_i[4] = p->extra_i[5] = 0;
}

// Overflow plan of a sliced matrix, built on its first SpMV (and again after
// sspmv_set_kernel changes the cap).  Overflow rows are ordered short tails
// first, then long tails (kPieceMin nonzeros or more), their tails copied in
// that order into the compact arrays.  extra[0] compact row offsets (nov+1;
// its first nshort+1 entries are the short-tail CSR's row_offset), extra[1]
// overflow rows (stored positions), extra[2] short-tail CSR result (nshort x
// kMaxK), extra[3] pieces (int4), extra[4] thread partials of the overflow
// rows, extra[5] / extra[6] compact columns / values, extra[7] piece partials,
// extra[8] overflow id per stored row (-1: none), extra[9] first piece of each
// long row (+1 entry); p->sub the short-tail CSR matrix (its stream plan built
// here); extra_i[1] overflow rows, [2] the cap, [3] the kernel parameter the
// plan was built for, [4] short-tail rows, [5] pieces, [7] built.
sspmv_status ensure_overflow_plan(const sspmv_features *f, const SlicedView &v, Plan *p, sspmv_stream_t s) {
    if (p->extra_i[7] && p->extra_i[3] == p->param) return SSPMV_OK;
    std::lock_guard<PlanMutex> g(plan_mutex());
    if (p->extra_i[7] && p->extra_i[3] == p->param) return SSPMV_OK;
    p->extra_i[7] = 0;
    free_overflow(p, s);  // a plan for another cap, or one whose building failed
    std::vector<int32_t> len((size_t)v.m);
    {
        int32_t *dlen = nullptr;
        SSPMV_TRY(dalloc(&dlen, (size_t)v.m, s));
        stored_row_lengths<<<grid_for(v.m, 256, (int64_t)num_sms() * 32), 256, 0, cu(s)>>>(v.m, v.C, v.chunk_ptr,
                                                                                           v.col, dlen);
        SSPMV_LAUNCH_CHECK();
        SSPMV_CUDA_TRY(cudaMemcpyAsync(len.data(), dlen, len.size() * 4, cudaMemcpyDeviceToHost, cu(s)));
        SSPMV_CUDA_TRY(cudaStreamSynchronize(cu(s)));
        dfree(dlen, s);
    }
    const int64_t cap = p->param > 0 ? (int64_t)p->param : choose_cap(len);
    std::vector<int32_t> rows, long_rows;
    int64_t total = 0;
    for (int64_t i = 0; i < v.m; i++) {
        const int64_t l = len[(size_t)i];
        if (l <= cap) continue;
        total += l - cap;
        (l - cap >= kPieceMin ? long_rows : rows).push_back((int32_t)i);
    }
    if (total > 0x7fffffff) return fail(SSPMV_NOT_SUPPORTED, "overflow of the long rows exceeds the int32 range");
    const int64_t nshort = (int64_t)rows.size();
    rows.insert(rows.end(), long_rows.begin(), long_rows.end());
    const int64_t nov = (int64_t)rows.size();
    std::vector<int32_t> optr{0}, pbegin;
    std::vector<int4> pieces;
    for (int64_t o = 0; o < nov; o++) {
        const int32_t o0 = optr.back(), n = len[(size_t)rows[(size_t)o]] - (int32_t)cap;
        if (o >= nshort) {
            pbegin.push_back((int32_t)pieces.size());
            for (int64_t e = 0; e < n; e += kPieceElems)
                pieces.push_back(make_int4((int)o, (int)(o0 + e), (int)(o0 + std::min<int64_t>(n, e + kPieceElems)), 0));
        }
        optr.push_back(o0 + n);
    }
    pbegin.push_back((int32_t)pieces.size());
    const int64_t novf = optr.back(), npieces = (int64_t)pieces.size();
    if (nov > 0) {
        const size_t sv = vsize(f->value_type);
        int32_t *dptr = nullptr, *drows = nullptr, *dov = nullptr, *ocol = nullptr, *dpb = nullptr;
        int4 *dpieces = nullptr;
        unsigned char *yov = nullptr, *opart = nullptr, *oval = nullptr, *ppart = nullptr;
        // each buffer belongs to the plan as soon as it exists (free_overflow)
        SSPMV_TRY(dalloc(&dptr, optr.size(), s));
        p->extra[0] = dptr;
        SSPMV_TRY(dalloc(&drows, rows.size(), s));
        p->extra[1] = drows;
        SSPMV_TRY(dalloc(&yov, (size_t)std::max<int64_t>(nshort, 1) * kMaxK * sv, s));
        p->extra[2] = yov;
        SSPMV_TRY(dalloc(&dpieces, pieces.size(), s));
        p->extra[3] = dpieces;
        SSPMV_TRY(dalloc(&opart, (size_t)nov * kMaxK * sv, s));
        p->extra[4] = opart;
        SSPMV_TRY(dalloc(&ocol, (size_t)novf, s));
        p->extra[5] = ocol;
        SSPMV_TRY(dalloc(&oval, (size_t)novf * sv, s));
        p->extra[6] = oval;
        SSPMV_TRY(dalloc(&ppart, (size_t)std::max<int64_t>(npieces, 1) * kMaxK * sv, s));
        p->extra[7] = ppart;
        SSPMV_TRY(dalloc(&dov, (size_t)v.m, s));
        p->extra[8] = dov;
        SSPMV_TRY(dalloc(&dpb, pbegin.size(), s));
        p->extra[9] = dpb;
        SSPMV_CUDA_TRY(cudaMemcpyAsync(dptr, optr.data(), optr.size() * 4, cudaMemcpyHostToDevice, cu(s)));
        SSPMV_CUDA_TRY(cudaMemcpyAsync(drows, rows.data(), rows.size() * 4, cudaMemcpyHostToDevice, cu(s)));
        SSPMV_CUDA_TRY(cudaMemcpyAsync(dpb, pbegin.data(), pbegin.size() * 4, cudaMemcpyHostToDevice, cu(s)));
        if (npieces > 0)
            SSPMV_CUDA_TRY(cudaMemcpyAsync(dpieces, pieces.data(), pieces.size() * sizeof(int4),
                                           cudaMemcpyHostToDevice, cu(s)));
        SSPMV_CUDA_TRY(cudaMemsetAsync(dov, 0xff, (size_t)v.m * 4, cu(s)));
        set_overflow_ids<<<grid_for(nov, 256), 256, 0, cu(s)>>>(nov, drows, dov);
        SSPMV_LAUNCH_CHECK();
        SSPMV_TRY(dispatch_value(f->value_type, [&](auto tag) -> sspmv_status {
            using V = decltype(tag);
            copy_overflow<V><<<grid_for(nov * 32, 256), 256, 0, cu(s)>>>(nov, v.C, cap, drows, dptr, v.chunk_ptr,
                                                                         v.col, (const V *)v.val, ocol, (V *)oval);
            SSPMV_LAUNCH_CHECK();
            return SSPMV_OK;
        }));
        if (nshort > 0) {
            p->sub = new (std::nothrow) sspmv_csr();
            if (!p->sub) return fail(SSPMV_OUT_OF_MEMORY, "overflow matrix allocation failed");
            SSPMV_TRY(sspmv_csr_wrap(p->sub, f->value_type, nshort, v.n, optr[(size_t)nshort], dptr, ocol, oval));
            const int32_t *rs = nullptr;
            int64_t nch = 0;
            int32_t gap = 0;
            SSPMV_TRY(csr_stream_plan(p->sub, &rs, &nch, &gap, s));  // built now, not inside a later SpMV
        }
        SSPMV_CUDA_TRY(cudaStreamSynchronize(cu(s)));
    }
    p->extra_i[1] = nov;
    p->extra_i[2] = nov > 0 ? cap : kNoCap;
    p->extra_i[3] = p->param;
    p->extra_i[4] = nshort;
    p->extra_i[5] = npieces;
    p->extra_i[7] = 1;
    return SSPMV_OK;
}

template <typename V, int K>
sspmv_status launch_sliced(const SlicedView &v, Plan *p, V alpha, const V *x, int64_t ldx, V beta, V *y,
                           int64_t ldy, sspmv_stream_t s) {
    const int64_t nov = p ? p->extra_i[1] : 0;
    const unsigned grid = grid_for(v.m, kBlock, (int64_t)num_sms() * 16);
    const int xvec = xrow_vec(x, ldx, sizeof(V), K);
    auto go = [&](auto kernel) {
        kernel<<<grid, kBlock, 0, cu(s)>>>(
            (int)v.m, v.C, v.chunk_ptr, v.reorder, v.col, (const V *)v.val, x, ldx, xvec, alpha, beta, y, ldy,
            nov > 0 ? p->extra_i[2] : kNoCap, nov > 0 ? (const int32_t *)p->extra[8] : nullptr,
            nov > 0 ? (V *)p->extra[4] : nullptr);
    };
    if (K == 1 && alpha == V(1) && beta == V(0)) go(sliced_spmv_kernel<V, K, K == 1>);  // y = sum
    else go(sliced_spmv_kernel<V, K>);
    SSPMV_LAUNCH_CHECK();
    if (nov > 0) {
        const int64_t nshort = p->extra_i[4], npieces = p->extra_i[5];
        if (nshort > 0) SSPMV_TRY(sspmv_spmm_csr(1.0, p->sub, K, x, ldx, 0.0, p->extra[2], kMaxK, s));
        if (npieces > 0) {
            sliced_piece_kernel<V, K><<<grid_for(npieces * 32, kBlock), kBlock, 0, cu(s)>>>(
                npieces, (const int4 *)p->extra[3], (const int32_t *)p->extra[5], (const V *)p->extra[6], x, ldx,
                xvec, (V *)p->extra[7]);
            SSPMV_LAUNCH_CHECK();
        }
        sliced_overflow_fixup<V, K><<<grid_for(nov, 256), 256, 0, cu(s)>>>(
            nov, nshort, (const int32_t *)p->extra[1], v.reorder, (const V *)p->extra[4], (const V *)p->extra[2],
            (const int32_t *)p->extra[9], (const V *)p->extra[7], alpha, beta, y, ldy);
        SSPMV_LAUNCH_CHECK();
    }
    return SSPMV_OK;
}

sspmv_status spmm_sliced(const sspmv_features *f, const SlicedView &v, double alpha, int32_t k, const void *X,
                         int64_t ldx, double beta, void *Y, int64_t ldy, sspmv_stream_t s) {
    SSPMV_TRY(check_spmm_args(f, k, X, ldx, Y, ldy));
    if (v.m == 0) return SSPMV_OK;
    Plan *p = nullptr;
    if (v.nchunks > 0) {  // ELL (nchunks == 0 here) keeps every row in the thread pass
        p = get_plan(f);
        if (!p) return fail(SSPMV_OUT_OF_MEMORY, "plan allocation failed");
        SSPMV_TRY(ensure_overflow_plan(f, v, p, s));
    }
    return dispatch_value(f->value_type, [&](auto tag) -> sspmv_status {
        using V = decltype(tag);
        return for_rhs_chunks<V>(k, (const V *)X, (V *)Y, [&](int32_t step, const V *xs, V *ys) {
            const V a = (V)alpha, b = (V)beta;
            switch (step) {
            case 8: return launch_sliced<V, 8>(v, p, a, xs, ldx, b, ys, ldy, s);
            case 4: return launch_sliced<V, 4>(v, p, a, xs, ldx, b, ys, ldy, s);
            case 2: return launch_sliced<V, 2>(v, p, a, xs, ldx, b, ys, ldy, s);
            default: return launch_sliced<V, 1>(v, p, a, xs, ldx, b, ys, ldy, s);
            }
        });
    });
}

// ------------------------------------------------------------ converters --
// keys for the slice sort: position p holds row m-1-p (descending input order)
__global__ void sell_sort_keys(int64_t m, int64_t sigma, int32_t maxlen, const int32_t *__restrict__ rp,
                               uint64_t *__restrict__ keys, uint32_t *__restrict__ vals) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < m; p += (int64_t)gridDim.x * blockDim.x) {
        const int64_t row = m - 1 - p;
        const int32_t len = rp[row + 1] - rp[row];
        keys[p] = (uint64_t)(row / sigma) * (uint64_t)(maxlen + 1) + (uint64_t)(maxlen - len);
        vals[p] = (uint32_t)row;
    }
}

__global__ void copy_u32_to_i32(int64_t n, const uint32_t *__restrict__ in, int32_t *__restrict__ out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (int32_t)in[i];
}

// chunk width = max row length in the chunk, rounded up to `align`.  Pass 1
// (thread per stored row position) folds row lengths into width[] with
// atomicMax -- one atomic per block when the block's rows lie in one chunk
// (ELL is a single chunk of all rows), one per row otherwise; width[] starts
// at zero.  Pass 2 rounds and sizes each chunk.
__global__ void chunk_row_max(int64_t m, int32_t C, const int32_t *__restrict__ rp,
                              const int32_t *__restrict__ reorder, int32_t *__restrict__ width) {
    __shared__ int s_max[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < m; base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = base + threadIdx.x;
        int len = 0;
        if (i < m) {
            const int64_t r = reorder ? reorder[i] : i;
            len = rp[r + 1] - rp[r];
        }
        const int64_t last = min(base + (int64_t)blockDim.x, m) - 1;
        if (base / C == last / C) {  // block-uniform branch
            int v = len;
            for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
            if (lane == 0) s_max[warp] = v;
            __syncthreads();
            if (threadIdx.x == 0) {
                int b = 0;
                for (int w = 0; w < nwarps; w++) b = max(b, s_max[w]);
                if (b > 0) atomicMax(width + base / C, b);
            }
            __syncthreads();
        } else if (len > 0) {
            atomicMax(width + i / C, len);
        }
    }
}

__global__ void chunk_widths(int64_t nchunks, int32_t C, int32_t align, int32_t *__restrict__ width,
                             int64_t *__restrict__ slots) {
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < nchunks;
         c += (int64_t)gridDim.x * blockDim.x) {
        const int32_t w = ((width[c] + align - 1) / align) * align;
        width[c] = w;
        slots[c] = (int64_t)w * C;
    }
}

// Copies the CSR rows into the slab: a thread per stored row, except rows of
// kFillLong nonzeros or more, which the CTA holding them copies together
// after its short rows (one thread walking a 38k-nonzero row alone took
// milliseconds).
constexpr int64_t kFillLong = 256;

template <typename V>
__global__ void __launch_bounds__(256) sliced_fill(int64_t m, int32_t C, const int64_t *__restrict__ chunk_ptr,
                                                   const int32_t *__restrict__ reorder,
                                                   const int32_t *__restrict__ rp, const int32_t *__restrict__ ci,
                                                   const V *__restrict__ cv, int32_t *__restrict__ col,
                                                   V *__restrict__ val) {
    __shared__ int64_t s_long[256];
    __shared__ int s_count;
    for (int64_t b0 = (int64_t)blockIdx.x * blockDim.x; b0 < m; b0 += (int64_t)gridDim.x * blockDim.x) {
        if (threadIdx.x == 0) s_count = 0;
        __syncthreads();
        const int64_t i = b0 + threadIdx.x;
        if (i < m) {
            const int64_t r = reorder ? reorder[i] : i;
            const int64_t s0 = rp[r], len = rp[r + 1] - s0;
            if (len >= kFillLong) {
                s_long[atomicAdd(&s_count, 1)] = i;
            } else {
                const int64_t ic = div_nonneg(i, C);
                const int64_t base = chunk_ptr[ic] + (i - ic * C);
                for (int64_t k = 0; k < len; k++) {
                    col[base + k * C] = ci[s0 + k];
                    val[base + k * C] = cv[s0 + k];
                }
            }
        }
        __syncthreads();
        for (int t = 0; t < s_count; t++) {  // CTA-uniform
            const int64_t li = s_long[t];
            const int64_t r = reorder ? reorder[li] : li;
            const int64_t s0 = rp[r], len = rp[r + 1] - s0;
            const int64_t lc = div_nonneg(li, C);
            const int64_t base = chunk_ptr[lc] + (li - lc * C);
            for (int64_t k = threadIdx.x; k < len; k += blockDim.x) {
                col[base + k * C] = ci[s0 + k];
                val[base + k * C] = cv[s0 + k];
            }
        }
        __syncthreads();  // s_long / s_count are reused by the next round
    }
}

struct SlicedBuild {
    int32_t *reorder = nullptr;
    int32_t *width = nullptr;
    int64_t *chunk_ptr = nullptr;
    int64_t total = 0;
    int32_t *col = nullptr;
    void *val = nullptr;
    int64_t nchunks = 0;
    void release(sspmv_stream_t s) {
        dfree(reorder, s);
        dfree(width, s);
        dfree(chunk_ptr, s);
        dfree(col, s);
        dfree(val, s);
        *this = SlicedBuild();
    }
};

// sigma: 0 = no reordering (S-ELL / ELL), otherwise the slice height
// (>= num_rows for SELL-c-R).
sspmv_status build_sliced(const sspmv_csr *A, int32_t C, int32_t align, int64_t sigma, SlicedBuild &b,
                          sspmv_stream_t s) {
    const int64_t m = A->f.num_rows;
    const int32_t vt = A->f.value_type;
    b.nchunks = (m + C - 1) / C;
    int32_t maxlen = 0;
    SSPMV_TRY(max_row_length(A->row_offset, m, &maxlen, s));
    const unsigned g = grid_for(m, 256, (int64_t)num_sms() * 16);
    sspmv_status st = SSPMV_OK;
    if (sigma > 0) {
        uint64_t *keys = nullptr;
        uint32_t *vals = nullptr;
        st = dalloc(&b.reorder, (size_t)m, s);
        if (st == SSPMV_OK) st = dalloc(&keys, (size_t)m, s);
        if (st == SSPMV_OK) st = dalloc(&vals, (size_t)m, s);
        if (st == SSPMV_OK && m > 0) {
            sell_sort_keys<<<g, 256, 0, cu(s)>>>(m, sigma, maxlen, A->row_offset, keys, vals);
            note_launch();
            const uint64_t nslices = (uint64_t)((m + sigma - 1) / sigma);
            const uint64_t maxkey = (nslices - 1) * (uint64_t)(maxlen + 1) + (uint64_t)maxlen;
            st = radix_sort_pairs(keys, vals, m, bits_for(maxkey), s);
            if (st == SSPMV_OK) {
                copy_u32_to_i32<<<g, 256, 0, cu(s)>>>(m, vals, b.reorder);
                note_launch();
            }
        }
        dfree(keys, s);
        dfree(vals, s);
        if (st != SSPMV_OK) { b.release(s); return st; }
    }
    st = dalloc(&b.width, (size_t)b.nchunks, s);
    if (st == SSPMV_OK) st = dalloc(&b.chunk_ptr, (size_t)b.nchunks + 1, s);
    if (st == SSPMV_OK && b.nchunks > 0) {
        cudaError_t e = cudaMemsetAsync(b.width, 0, (size_t)b.nchunks * 4, cu(s));
        if (e != cudaSuccess) st = fail(SSPMV_CUDA_ERROR, "width memset: %s", cudaGetErrorString(e));
        if (st == SSPMV_OK && m > 0) {
            chunk_row_max<<<grid_for(m, 256, (int64_t)num_sms() * 16), 256, 0, cu(s)>>>(m, C, A->row_offset,
                                                                                      b.reorder, b.width);
            note_launch();
        }
        if (st == SSPMV_OK) {
            chunk_widths<<<grid_for(b.nchunks, 256, (int64_t)num_sms() * 16), 256, 0, cu(s)>>>(b.nchunks, C, align,
                                                                                             b.width, b.chunk_ptr);
            note_launch();
            st = exclusive_scan_i64(b.chunk_ptr, b.chunk_ptr, b.nchunks, &b.total, s);
        }
    }
    if (st == SSPMV_OK) {
        cudaError_t e = cudaMemcpyAsync(b.chunk_ptr + b.nchunks, &b.total, 8, cudaMemcpyHostToDevice, cu(s));
        if (e != cudaSuccess) st = fail(SSPMV_CUDA_ERROR, "chunk_ptr: %s", cudaGetErrorString(e));
    }
    if (st == SSPMV_OK) st = dalloc(&b.col, (size_t)b.total, s);
    if (st == SSPMV_OK) st = dalloc((unsigned char **)&b.val, (size_t)b.total * vsize(vt), s);
    if (st == SSPMV_OK && b.total > 0) {
        cudaError_t e = cudaMemsetAsync(b.col, 0xff, (size_t)b.total * 4, cu(s));
        if (e == cudaSuccess) e = cudaMemsetAsync(b.val, 0, (size_t)b.total * vsize(vt), cu(s));
        if (e != cudaSuccess) st = fail(SSPMV_CUDA_ERROR, "memset: %s", cudaGetErrorString(e));
    }
    if (st == SSPMV_OK && m > 0) {
        st = dispatch_value(vt, [&](auto tag) -> sspmv_status {
            using V = decltype(tag);
            sliced_fill<V><<<g, 256, 0, cu(s)>>>(m, C, b.chunk_ptr, b.reorder, A->row_offset, A->col_index,
                                                 (const V *)A->values, b.col, (V *)b.val);
            SSPMV_LAUNCH_CHECK();
            return SSPMV_OK;
        });
    }
    if (st == SSPMV_OK) {
        cudaError_t e = cudaStreamSynchronize(cu(s));
        if (e != cudaSuccess) st = fail(SSPMV_CUDA_ERROR, "convert: %s", cudaGetErrorString(e));
    }
    if (st != SSPMV_OK) b.release(s);
    return st;
}

sspmv_status check_csr(const sspmv_csr *A) {
    if (!A) return fail(SSPMV_INVALID_ARG, "null csr");
    return check_dims(A->f.value_type, A->f.num_rows, A->f.num_cols, A->f.num_nnzs);
}

// Host copy of a slot-major slab, reordered to the reference's row-major chunks.
sspmv_status export_slab(const int64_t *d_chunk_ptr, int64_t nchunks, int32_t C, int64_t total, const int32_t *d_col,
                         const void *d_val, size_t sv, int32_t *col_out, void *val_out, sspmv_stream_t s) {
    std::vector<int64_t> cp((size_t)nchunks + 1);
    std::vector<int32_t> col((size_t)std::max<int64_t>(total, 1));
    std::vector<unsigned char> val((size_t)std::max<int64_t>(total, 1) * sv);
    SSPMV_CUDA_TRY(cudaMemcpyAsync(cp.data(), d_chunk_ptr, (size_t)(nchunks + 1) * 8, cudaMemcpyDeviceToHost, cu(s)));
    if (total > 0) {
        SSPMV_CUDA_TRY(cudaMemcpyAsync(col.data(), d_col, (size_t)total * 4, cudaMemcpyDeviceToHost, cu(s)));
        SSPMV_CUDA_TRY(cudaMemcpyAsync(val.data(), d_val, (size_t)total * sv, cudaMemcpyDeviceToHost, cu(s)));
    }
    SSPMV_CUDA_TRY(cudaStreamSynchronize(cu(s)));
    for (int64_t c = 0; c < nchunks; c++) {
        const int64_t base = cp[(size_t)c], w = (cp[(size_t)c + 1] - base) / C;
        for (int32_t r = 0; r < C; r++)
            for (int64_t k = 0; k < w; k++) {
                const int64_t src = base + k * C + r, dst = base + (int64_t)r * w + k;
                if (col_out) col_out[dst] = col[(size_t)src];
                if (val_out) std::memcpy((unsigned char *)val_out + dst * sv, val.data() + src * sv, sv);
            }
    }
    return SSPMV_OK;
}

sspmv_status d2h(void *dst, const void *src, size_t bytes, sspmv_stream_t s) {
    if (!dst || bytes == 0) return SSPMV_OK;
    SSPMV_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, cu(s)));
    SSPMV_CUDA_TRY(cudaStreamSynchronize(cu(s)));
    return SSPMV_OK;
}

double sliced_bytes(const sspmv_features *f, int64_t nchunks, bool reorder, int32_t k, int32_t beta_nonzero) {
    const double sv = (double)vsize(f->value_type);
    return (double)f->num_nnzs * (sv + 4.0) + (double)(nchunks + 1) * 8.0 +
           (reorder ? (double)f->num_rows * 4.0 : 0.0) + (double)k * (double)f->num_cols * sv +
           (double)k * (double)f->num_rows * sv * (beta_nonzero ? 2.0 : 1.0);
}

}  // namespace

// =================================================================== ELL ===
// coo_to_ell (include/sparse_conversion.h:94-142): row counts, then each row's
// entries in COO order.  The same slab as csr_to_ell on the COO's stable
// row sort (coo_to_csr keeps each row's entries in COO order), so that is how
// it is built.  Like the reference it ignores ld (it always sets RowMajor).
extern "C" sspmv_status sspmv_coo_to_ell(const sspmv_coo *coo, int32_t ld, sspmv_ell *out, sspmv_stream_t s) {
    if (!coo || !out) return fail(SSPMV_INVALID_ARG, "null argument");
    (void)ld;
    sspmv_csr csr;
    SSPMV_TRY(sspmv_coo_to_csr(coo, &csr, s));
    const sspmv_status st = sspmv_csr_to_ell(&csr, SSPMV_ROW_MAJOR, out, s);
    sspmv_delete_csr(&csr);
    return st;
}

extern "C" sspmv_status sspmv_csr_to_ell(const sspmv_csr *csr, int32_t ld, sspmv_ell *out, sspmv_stream_t s) {
    SSPMV_TRY(check_csr(csr));
    if (!out) return fail(SSPMV_INVALID_ARG, "null output");
    if (ld != SSPMV_ROW_MAJOR && ld != SSPMV_COL_MAJOR) return fail(SSPMV_INVALID_ARG, "ld must be 0 or 1");
    const int64_t m = csr->f.num_rows;
    int32_t width = 0;
    SSPMV_TRY(max_row_length(csr->row_offset, m, &width, s));
    if ((double)m * (double)width > 4.0e9)
        return fail(SSPMV_INFEASIBLE, "ELL needs %lld x %d slots", (long long)m, width);
    // ELL == one chunk of C = m rows, alignment 1.
    SlicedBuild b;
    SSPMV_TRY(build_sliced(csr, (int32_t)std::max<int64_t>(m, 1), 1, 0, b, s));
    sspmv_ell A;
    init_features(&A.f, csr->f.value_type, m, csr->f.num_cols, csr->f.num_nnzs, 1);
    A.ld = ld;
    A.max_row_width = width;
    A.min_row_width = 0;
    A.col_index = b.col;
    A.values = b.val;
    Plan *p = get_plan(&A.f);
    p->extra[0] = b.chunk_ptr;  // {0, m*width}
    dfree(b.width, s);
    *out = A;
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_spmm_ell(double alpha, const sspmv_ell *A, int32_t k, const void *X, int64_t ldx,
                                       double beta, void *Y, int64_t ldy, sspmv_stream_t s) {
    if (!A) return fail(SSPMV_INVALID_ARG, "null matrix");
    Plan *p = get_plan(&A->f);
    SlicedView v{A->f.num_rows, (int32_t)std::max<int64_t>(A->f.num_rows, 1), (const int64_t *)p->extra[0], nullptr,
                 A->col_index, A->values, 0, A->f.num_cols};
    return spmm_sliced(&A->f, v, alpha, k, X, ldx, beta, Y, ldy, s);
}

extern "C" sspmv_status sspmv_LeSpMV_ell(double alpha, const sspmv_ell *A, const void *x, double beta, void *y,
                                         sspmv_stream_t s) {
    return sspmv_spmm_ell(alpha, A, 1, x, 1, beta, y, 1, s);
}

extern "C" sspmv_status sspmv_ell_export(const sspmv_ell *A, int32_t *col_index, void *values, sspmv_stream_t s) {
    if (!A) return fail(SSPMV_INVALID_ARG, "null matrix");
    const int64_t m = A->f.num_rows, w = A->max_row_width, tot = m * w;
    const size_t sv = vsize(A->f.value_type);
    if (A->ld == SSPMV_COL_MAJOR) {
        SSPMV_TRY(d2h(col_index, A->col_index, (size_t)tot * 4, s));
        SSPMV_TRY(d2h(values, A->values, (size_t)tot * sv, s));
        return SSPMV_OK;
    }
    std::vector<int32_t> col((size_t)std::max<int64_t>(tot, 1));
    std::vector<unsigned char> val((size_t)std::max<int64_t>(tot, 1) * sv);
    SSPMV_TRY(d2h(col.data(), A->col_index, (size_t)tot * 4, s));
    SSPMV_TRY(d2h(val.data(), A->values, (size_t)tot * sv, s));
    for (int64_t i = 0; i < m; i++)
        for (int64_t k = 0; k < w; k++) {
            if (col_index) col_index[i * w + k] = col[(size_t)(k * m + i)];
            if (values) std::memcpy((unsigned char *)values + (i * w + k) * sv, val.data() + (k * m + i) * sv, sv);
        }
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_delete_ell(sspmv_ell *A) {
    if (!A) return SSPMV_OK;
    delete_barrier();
    free_plan(&A->f, nullptr);
    if (A->f.owns) {
        dfree(A->col_index, nullptr);
        dfree(A->values, nullptr);
    }
    A->col_index = nullptr;
    A->values = nullptr;
    return SSPMV_OK;
}

extern "C" double sspmv_algorithmic_bytes_ell(const sspmv_ell *A, int32_t k, int32_t beta_nonzero) {
    return sliced_bytes(&A->f, 0, false, k, beta_nonzero) - 8.0;
}

// ================================================================= S-ELL ===
extern "C" sspmv_status sspmv_csr_to_sell(const sspmv_csr *csr, int32_t C, int32_t align, sspmv_s_ell *out,
                                          sspmv_stream_t s) {
    SSPMV_TRY(check_csr(csr));
    if (!out) return fail(SSPMV_INVALID_ARG, "null output");
    if (C == 0) C = 4;
    if (align == 0) align = default_alignment(csr->f.value_type);
    if (C < 1 || align < 1) return fail(SSPMV_INVALID_ARG, "chunkwidth and alignment must be >= 1");
    SlicedBuild b;
    SSPMV_TRY(build_sliced(csr, C, align, 0, b, s));
    sspmv_s_ell A;
    init_features(&A.f, csr->f.value_type, csr->f.num_rows, csr->f.num_cols, csr->f.num_nnzs, 1);
    A.sliceWidth = C;
    A.chunk_num = (int32_t)b.nchunks;
    A.alignment = align;
    A.row_width = b.width;
    A.chunk_ptr = b.chunk_ptr;
    A.total_slots = b.total;
    A.col_index = b.col;
    A.values = b.val;
    *out = A;
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_spmm_sell(double alpha, const sspmv_s_ell *A, int32_t k, const void *X, int64_t ldx,
                                        double beta, void *Y, int64_t ldy, sspmv_stream_t s) {
    if (!A) return fail(SSPMV_INVALID_ARG, "null matrix");
    SlicedView v{A->f.num_rows, A->sliceWidth,   A->chunk_ptr,   nullptr,
                 A->col_index,  A->values,     A->chunk_num,   A->f.num_cols};
    return spmm_sliced(&A->f, v, alpha, k, X, ldx, beta, Y, ldy, s);
}

extern "C" sspmv_status sspmv_LeSpMV_sell(double alpha, const sspmv_s_ell *A, const void *x, double beta, void *y,
                                          sspmv_stream_t s) {
    return sspmv_spmm_sell(alpha, A, 1, x, 1, beta, y, 1, s);
}

extern "C" sspmv_status sspmv_sell_export(const sspmv_s_ell *A, int32_t *row_width, int32_t *col_index,
                                          void *values, sspmv_stream_t s) {
    if (!A) return fail(SSPMV_INVALID_ARG, "null matrix");
    SSPMV_TRY(d2h(row_width, A->row_width, (size_t)A->chunk_num * 4, s));
    return export_slab(A->chunk_ptr, A->chunk_num, A->sliceWidth, A->total_slots, A->col_index, A->values,
                       vsize(A->f.value_type), col_index, values, s);
}

extern "C" sspmv_status sspmv_delete_sell(sspmv_s_ell *A) {
    if (!A) return SSPMV_OK;
    delete_barrier();
    free_plan(&A->f, nullptr);
    if (A->f.owns) {
        dfree(A->row_width, nullptr);
        dfree(A->chunk_ptr, nullptr);
        dfree(A->col_index, nullptr);
        dfree(A->values, nullptr);
    }
    A->row_width = nullptr;
    A->chunk_ptr = nullptr;
    A->col_index = nullptr;
    A->values = nullptr;
    return SSPMV_OK;
}

extern "C" double sspmv_algorithmic_bytes_sell(const sspmv_s_ell *A, int32_t k, int32_t beta_nonzero) {
    return sliced_bytes(&A->f, A->chunk_num, false, k, beta_nonzero);
}

// ========================================================== SELL-c-sigma ===
extern "C" sspmv_status sspmv_csr_to_sell_c_sigma(const sspmv_csr *csr, int32_t sigma, int32_t C, int32_t align,
                                                  sspmv_sell_c_sigma *out, sspmv_stream_t s) {
    SSPMV_TRY(check_csr(csr));
    if (!out) return fail(SSPMV_INVALID_ARG, "null output");
    if (sigma == 0) sigma = 16384;
    if (C == 0) C = 4;
    if (align == 0) align = default_alignment(csr->f.value_type);
    if (C < 1 || align < 1 || sigma < 1) return fail(SSPMV_INVALID_ARG, "sigma, C and alignment must be >= 1");
    if (sigma % C) return fail(SSPMV_INVALID_ARG, "sigma (%d) must be a multiple of C (%d)", sigma, C);
    SlicedBuild b;
    SSPMV_TRY(build_sliced(csr, C, align, sigma, b, s));
    const int64_t m = csr->f.num_rows;
    sspmv_sell_c_sigma A;
    init_features(&A.f, csr->f.value_type, m, csr->f.num_cols, csr->f.num_nnzs, 1);
    A.sliceWidth_Sigma = sigma;
    A.chunkWidth_C = C;
    A.sliceNum = (int32_t)((m + sigma - 1) / sigma);
    A.chunk_num_per_slice = sigma / C;
    A.chunkNum = A.sliceNum * A.chunk_num_per_slice;
    A.validchunkNum = (int32_t)b.nchunks;
    A.alignment = align;
    A.reorder = b.reorder;
    A.chunk_len = b.width;
    A.chunk_ptr = b.chunk_ptr;
    A.total_slots = b.total;
    A.col_index = b.col;
    A.values = b.val;
    *out = A;
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_spmm_sell_c_sigma(double alpha, const sspmv_sell_c_sigma *A, int32_t k, const void *X,
                                                int64_t ldx, double beta, void *Y, int64_t ldy, sspmv_stream_t s) {
    if (!A) return fail(SSPMV_INVALID_ARG, "null matrix");
    SlicedView v{A->f.num_rows, A->chunkWidth_C,   A->chunk_ptr,   A->reorder,
                 A->col_index,  A->values,         A->validchunkNum, A->f.num_cols};
    return spmm_sliced(&A->f, v, alpha, k, X, ldx, beta, Y, ldy, s);
}

extern "C" sspmv_status sspmv_LeSpMV_sell_c_sigma(double alpha, const sspmv_sell_c_sigma *A, const void *x,
                                                  double beta, void *y, sspmv_stream_t s) {
    return sspmv_spmm_sell_c_sigma(alpha, A, 1, x, 1, beta, y, 1, s);
}

extern "C" sspmv_status sspmv_sell_c_sigma_export(const sspmv_sell_c_sigma *A, int32_t *reorder, int32_t *chunk_len,
                                                  int32_t *col_index, void *values, sspmv_stream_t s) {
    if (!A) return fail(SSPMV_INVALID_ARG, "null matrix");
    SSPMV_TRY(d2h(reorder, A->reorder, (size_t)A->f.num_rows * 4, s));
    SSPMV_TRY(d2h(chunk_len, A->chunk_len, (size_t)A->validchunkNum * 4, s));
    return export_slab(A->chunk_ptr, A->validchunkNum, A->chunkWidth_C, A->total_slots, A->col_index, A->values,
                       vsize(A->f.value_type), col_index, values, s);
}

extern "C" sspmv_status sspmv_delete_sell_c_sigma(sspmv_sell_c_sigma *A) {
    if (!A) return SSPMV_OK;
    delete_barrier();
    free_plan(&A->f, nullptr);
    if (A->f.owns) {
        dfree(A->reorder, nullptr);
        dfree(A->chunk_len, nullptr);
        dfree(A->chunk_ptr, nullptr);
        dfree(A->col_index, nullptr);
        dfree(A->values, nullptr);
    }
    A->reorder = A->chunk_len = A->col_index = nullptr;
    A->chunk_ptr = nullptr;
    A->values = nullptr;
    return SSPMV_OK;
}

extern "C" double sspmv_algorithmic_bytes_sell_c_sigma(const sspmv_sell_c_sigma *A, int32_t k, int32_t beta_nonzero) {
    return sliced_bytes(&A->f, A->validchunkNum, true, k, beta_nonzero);
}

// ============================================================== SELL-c-R ===
extern "C" sspmv_status sspmv_csr_to_sell_c_R(const sspmv_csr *csr, int32_t C, int32_t align, sspmv_sell_c_R *out,
                                              sspmv_stream_t s) {
    SSPMV_TRY(check_csr(csr));
    if (!out) return fail(SSPMV_INVALID_ARG, "null output");
    if (C == 0) C = 4;
    if (align == 0) align = default_alignment(csr->f.value_type);
    if (C < 1 || align < 1) return fail(SSPMV_INVALID_ARG, "C and alignment must be >= 1");
    const int64_t m = csr->f.num_rows;
    SlicedBuild b;
    SSPMV_TRY(build_sliced(csr, C, align, std::max<int64_t>(m, 1), b, s));
    sspmv_sell_c_R A;
    init_features(&A.f, csr->f.value_type, m, csr->f.num_cols, csr->f.num_nnzs, 1);
    A.chunkWidth_C = C;
    A.validchunkNum = (int32_t)b.nchunks;
    A.alignment = align;
    A.reorder = b.reorder;
    A.chunk_len = b.width;
    A.chunk_ptr = b.chunk_ptr;
    A.total_slots = b.total;
    A.col_index = b.col;
    A.values = b.val;
    *out = A;
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_spmm_sell_c_R(double alpha, const sspmv_sell_c_R *A, int32_t k, const void *X,
                                            int64_t ldx, double beta, void *Y, int64_t ldy, sspmv_stream_t s) {
    if (!A) return fail(SSPMV_INVALID_ARG, "null matrix");
    SlicedView v{A->f.num_rows, A->chunkWidth_C,   A->chunk_ptr,   A->reorder,
                 A->col_index,  A->values,         A->validchunkNum, A->f.num_cols};
    return spmm_sliced(&A->f, v, alpha, k, X, ldx, beta, Y, ldy, s);
}

extern "C" sspmv_status sspmv_LeSpMV_sell_c_R(double alpha, const sspmv_sell_c_R *A, const void *x, double beta,
                                              void *y, sspmv_stream_t s) {
    return sspmv_spmm_sell_c_R(alpha, A, 1, x, 1, beta, y, 1, s);
}

extern "C" sspmv_status sspmv_sell_c_R_export(const sspmv_sell_c_R *A, int32_t *reorder, int32_t *chunk_len,
                                              int32_t *col_index, void *values, sspmv_stream_t s) {
    if (!A) return fail(SSPMV_INVALID_ARG, "null matrix");
    SSPMV_TRY(d2h(reorder, A->reorder, (size_t)A->f.num_rows * 4, s));
    SSPMV_TRY(d2h(chunk_len, A->chunk_len, (size_t)A->validchunkNum * 4, s));
    return export_slab(A->chunk_ptr, A->validchunkNum, A->chunkWidth_C, A->total_slots, A->col_index, A->values,
                       vsize(A->f.value_type), col_index, values, s);
}

extern "C" sspmv_status sspmv_delete_sell_c_R(sspmv_sell_c_R *A) {
    if (!A) return SSPMV_OK;
    delete_barrier();
    free_plan(&A->f, nullptr);
    if (A->f.owns) {
        dfree(A->reorder, nullptr);
        dfree(A->chunk_len, nullptr);
        dfree(A->chunk_ptr, nullptr);
        dfree(A->col_index, nullptr);
        dfree(A->values, nullptr);
    }
    A->reorder = A->chunk_len = A->col_index = nullptr;
    A->chunk_ptr = nullptr;
    A->values = nullptr;
    return SSPMV_OK;
}

extern "C" double sspmv_algorithmic_bytes_sell_c_R(const sspmv_sell_c_R *A, int32_t k, int32_t beta_nonzero) {
    return sliced_bytes(&A->f, A->validchunkNum, true, k, beta_nonzero);
}
