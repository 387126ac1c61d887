// benchmark_spmv.cpp -- the reference's benchmark_spmv_<fmt> programs
// (test/benchmark_spmv_<fmt>.cpp) over the C ABI, on the GPU.
//
// One executable; the format comes from the program name (installed as
// benchmark_spmv_csr, benchmark_spmv_coo, ..., benchmark_spmv_csr5) or from
// --format=<fmt>.  Same command line as the reference:
//     benchmark_spmv_<fmt> my_matrix.mtx [--matID=N] [--precision=32|64]
//                          [--Index=0] [--sche=0..3] [--threads=T] [--ld=0|1]
// --sche and --threads select CPU OpenMP schedules there; they are accepted
// and recorded but do not change the GPU kernels.  --Index=1 (64-bit
// indices) is not supported by this library (int32 indices).
// Extra GPU options: --chunkwidth, --slicewidth, --alignment (sliced
// formats), --blockr / --blockc (BSR), --sigma / --omega (CSR5),
// --kernel=<flag> (kernel_flag), --perf=<file> (default
// ./performance/mat_perf.txt, as the reference's MAT_PERFORMANCE),
// --bytes=reference|algorithmic (the byte count behind the printed GB/s:
// the reference's bytes_per_spmv by default).
//
// As the reference does, it reads the matrix (Matrix Market), converts CSR
// to the format (timed: "format_convert", ms), compares the format's SpMV
// against CSR (maximum relative error, the reference's thresholds), times
// SpMV with alpha = 1, beta = 0 (warm-up, then 1000 iterations, or fewer so
// that a slow SpMV runs about 20 s, at least 20; CUDA events), prints the
// reference's benchmarking line and appends its mat_perf.txt line.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "sspmv.h"

namespace {

const char *get_arg(int argc, char **argv, const char *key) {
    const char *val = nullptr;
    const size_t n = strlen(key);
    for (int i = 1; i < argc; i++)
        if (strncmp(argv[i], "--", 2) == 0 && strncmp(argv[i] + 2, key, n) == 0) val = argv[i];
    return val;
}

const char *get_argval(int argc, char **argv, const char *key) {
    const char *val = nullptr;
    const size_t n = strlen(key);
    for (int i = 1; i < argc; i++) {
        const char *t = argv[i];
        if (strncmp(t, "--", 2) != 0) continue;
        t += 2;
        if (strncmp(t, key, n) != 0) continue;
        t += n;
        if (*t != '=') continue;
        val = t + 1;
    }
    return val;
}

int argint(int argc, char **argv, const char *key, int def) {
    const char *v = get_argval(argc, argv, key);
    return v ? atoi(v) : def;
}

std::string stem(const std::string &path) {
    size_t a = path.find_last_of("/\\");
    a = a == std::string::npos ? 0 : a + 1;
    size_t b = path.find_last_of('.');
    if (b == std::string::npos || b < a) b = path.size();
    return path.substr(a, b - a);
}

const char *kFormats[] = {"csr", "coo", "ell", "sell", "sell_c_sigma", "sell_c_R", "dia", "bsr", "csr5"};

void usage(const char *prog) {
    printf("Usage:\n");
    printf("\t%s with following parameters:\n", prog);
    printf("\t my_matrix.mtx\n");
    printf("\t --matID     = m_num, giving the matrix ID number in dataset (default 0).\n");
    printf("\t --Index     = 0 (int:default); 1 (long long) is not supported on this build\n");
    printf("\t --precision = 32(or 64)\n");
    printf("\t --sche      = schedule strategy of the CPU build (accepted, recorded, no effect on the GPU)\n");
    printf("\t --threads   = CPU threads of the CPU build (accepted, no effect on the GPU)\n");
    printf("\t --ld        = ELL layout recorded in the format (0 row-major, 1 column-major)\n");
    printf("\t --format    = csr|coo|ell|sell|sell_c_sigma|sell_c_R|dia|bsr|csr5 (default: from the program name)\n");
    printf("\t --bytes     = reference (default: the reference's bytes_per_spmv) | algorithmic (no padding, x and y once)\n");
    printf("\t --chunkwidth, --slicewidth, --alignment, --blockr, --blockc, --sigma, --omega, --kernel, --perf\n");
    printf("Note: my_matrix.mtx must be real-valued sparse matrix in the MatrixMarket file format.\n");
}

// Device buffer freed at scope exit.
struct DevBuf {
    void *p = nullptr;
    explicit DevBuf(size_t n) {
        if (cudaMalloc(&p, n ? n : 1) != cudaSuccess) p = nullptr;
    }
    ~DevBuf() {
        if (p) cudaFree(p);
    }
};

#define CHECK(call)                                                                                  \
    do {                                                                                             \
        sspmv_status s_ = (call);                                                                    \
        if (s_ != SSPMV_OK) {                                                                        \
            fprintf(stderr, "%s: %s: %s\n", #call, sspmv_status_string(s_), sspmv_last_error());    \
            return 1;                                                                                \
        }                                                                                            \
    } while (0)

// Any converted matrix with its SpMV entry point and deleter.
struct FormatMatrix {
    std::string fmt;
    sspmv_csr csr;
    sspmv_coo coo;
    sspmv_ell ell;
    sspmv_s_ell sell;
    sspmv_sell_c_sigma scs;
    sspmv_sell_c_R scr;
    sspmv_dia dia;
    sspmv_bsr bsr;
    sspmv_csr5 csr5;
    sspmv_features *features() {
        if (fmt == "coo") return &coo.f;
        if (fmt == "ell") return &ell.f;
        if (fmt == "sell") return &sell.f;
        if (fmt == "sell_c_sigma") return &scs.f;
        if (fmt == "sell_c_R") return &scr.f;
        if (fmt == "dia") return &dia.f;
        if (fmt == "bsr") return &bsr.f;
        if (fmt == "csr5") return &csr5.f;
        return &csr.f;
    }
    sspmv_status spmv(double a, const void *x, double b, void *y) {
        if (fmt == "coo") return sspmv_LeSpMV_coo(a, &coo, x, b, y, nullptr);
        if (fmt == "ell") return sspmv_LeSpMV_ell(a, &ell, x, b, y, nullptr);
        if (fmt == "sell") return sspmv_LeSpMV_sell(a, &sell, x, b, y, nullptr);
        if (fmt == "sell_c_sigma") return sspmv_LeSpMV_sell_c_sigma(a, &scs, x, b, y, nullptr);
        if (fmt == "sell_c_R") return sspmv_LeSpMV_sell_c_R(a, &scr, x, b, y, nullptr);
        if (fmt == "dia") return sspmv_LeSpMV_dia(a, &dia, x, b, y, nullptr);
        if (fmt == "bsr") return sspmv_LeSpMV_bsr(a, &bsr, x, b, y, nullptr);
        if (fmt == "csr5") return sspmv_LeSpMV_csr5(a, &csr5, x, b, y, nullptr);
        return sspmv_LeSpMV_csr(a, &csr, x, b, y, nullptr);
    }
    // The reference's bytes_per_spmv (include/spmv_benchmark.h:26-150).
    double reference_bytes() {
        if (fmt == "coo") return sspmv_reference_bytes_coo(&coo);
        if (fmt == "ell") return sspmv_reference_bytes_ell(&ell);
        if (fmt == "sell") return sspmv_reference_bytes_sell(&sell);
        if (fmt == "sell_c_sigma") return sspmv_reference_bytes_sell_c_sigma(&scs);
        if (fmt == "sell_c_R") return sspmv_reference_bytes_sell_c_R(&scr);
        if (fmt == "dia") return sspmv_reference_bytes_dia(&dia);
        if (fmt == "bsr") return sspmv_reference_bytes_bsr(&bsr);
        if (fmt == "csr5") return sspmv_reference_bytes_csr5(&csr5);
        return sspmv_reference_bytes_csr(&csr);
    }
    // Structural bytes without padding, x and y once (sspmv_algorithmic_bytes_<fmt>).
    double algorithmic_bytes() {
        if (fmt == "coo") return sspmv_algorithmic_bytes_coo(&coo, 1, 0);
        if (fmt == "ell") return sspmv_algorithmic_bytes_ell(&ell, 1, 0);
        if (fmt == "sell") return sspmv_algorithmic_bytes_sell(&sell, 1, 0);
        if (fmt == "sell_c_sigma") return sspmv_algorithmic_bytes_sell_c_sigma(&scs, 1, 0);
        if (fmt == "sell_c_R") return sspmv_algorithmic_bytes_sell_c_R(&scr, 1, 0);
        if (fmt == "dia") return sspmv_algorithmic_bytes_dia(&dia, 1, 0);
        if (fmt == "bsr") return sspmv_algorithmic_bytes_bsr(&bsr, 1, 0);
        if (fmt == "csr5") return sspmv_algorithmic_bytes_csr5(&csr5, 1, 0);
        return sspmv_algorithmic_bytes_csr(&csr, 1, 0);
    }
    void release() {
        if (fmt == "coo") sspmv_delete_coo(&coo);
        else if (fmt == "ell") sspmv_delete_ell(&ell);
        else if (fmt == "sell") sspmv_delete_sell(&sell);
        else if (fmt == "sell_c_sigma") sspmv_delete_sell_c_sigma(&scs);
        else if (fmt == "sell_c_R") sspmv_delete_sell_c_R(&scr);
        else if (fmt == "dia") sspmv_delete_dia(&dia);
        else if (fmt == "bsr") sspmv_delete_bsr(&bsr);
        else if (fmt == "csr5") sspmv_delete_csr5(&csr5);
    }
};

// The reference's maximum_relative_error (include/sparse_operation.h:76-94):
// max over entries with a != b of |a - b| / (|a| + |b| + sqrt(eps)), in V.
template <typename V>
V max_relative_error(const std::vector<V> &a, const std::vector<V> &b, size_t count) {
    V mx = 0;
    const V eps = std::sqrt(std::numeric_limits<V>::epsilon());
    for (size_t i = 0; i < count; i++) {
        const V d = std::abs(a[i] - b[i]);
        if (d != 0) mx = std::max(mx, d / (std::abs(a[i]) + std::abs(b[i]) + eps));
    }
    return mx;
}

template <typename V>
int run(int argc, char **argv, const std::string &fmt, const char *path, int32_t vt) {
    int64_t m = 0, n = 0, nnz = 0;
    CHECK(sspmv_read_mtx(path, vt, &m, &n, &nnz, nullptr, nullptr, nullptr));
    std::vector<int32_t> rp(m + 1), ci(std::max<int64_t>(nnz, 1));
    std::vector<V> cv(std::max<int64_t>(nnz, 1));
    CHECK(sspmv_read_mtx(path, vt, &m, &n, &nnz, rp.data(), ci.data(), cv.data()));
    printf("Using %lld-by-%lld matrix with %lld nonzero values\n", (long long)m, (long long)n, (long long)nnz);
    fflush(stdout);

    const int matID = argint(argc, argv, "matID", 0);
    const int sche = argint(argc, argv, "sche", 0);
    if (sche < 0 || sche > 3) {
        printf("sche must be [0,1,2,3]. '--help see more details'\n");
        return 1;
    }
    FormatMatrix F;
    F.fmt = fmt;
    CHECK(sspmv_csr_create(&F.csr, vt, m, n, nnz, rp.data(), ci.data(), cv.data(), 1, nullptr));

    const int C = argint(argc, argv, "chunkwidth", 0), align = argint(argc, argv, "alignment", 0);
    const int sigma = argint(argc, argv, "slicewidth", 0);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaDeviceSynchronize();
    cudaEventRecord(e0);
    sspmv_status st = SSPMV_OK;
    if (fmt == "coo") st = sspmv_csr_to_coo(&F.csr, &F.coo, nullptr);
    else if (fmt == "ell") st = sspmv_csr_to_ell(&F.csr, argint(argc, argv, "ld", 0), &F.ell, nullptr);
    else if (fmt == "sell") st = sspmv_csr_to_sell(&F.csr, C, align, &F.sell, nullptr);
    else if (fmt == "sell_c_sigma") st = sspmv_csr_to_sell_c_sigma(&F.csr, sigma, C, align, &F.scs, nullptr);
    else if (fmt == "sell_c_R") st = sspmv_csr_to_sell_c_R(&F.csr, C, align, &F.scr, nullptr);
    else if (fmt == "dia") st = sspmv_csr_to_dia(&F.csr, 0, align, &F.dia, nullptr);
    else if (fmt == "bsr")
        st = sspmv_csr_to_bsr(&F.csr, argint(argc, argv, "blockr", 0), argint(argc, argv, "blockc", 0), &F.bsr, nullptr);
    else if (fmt == "csr5")
        st = sspmv_csr_to_csr5(&F.csr, argint(argc, argv, "sigma", 0), argint(argc, argv, "omega", 0), &F.csr5, nullptr);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float convert_ms = 0;
    cudaEventElapsedTime(&convert_ms, e0, e1);
    if (st != SSPMV_OK) {
        fprintf(stderr, "csr_to_%s: %s: %s\n", fmt.c_str(), sspmv_status_string(st), sspmv_last_error());
        sspmv_delete_csr(&F.csr);
        return 1;
    }
    if (const char *k = get_argval(argc, argv, "kernel")) CHECK(sspmv_set_kernel(F.features(), atoi(k), 0));

    // correctness against CSR: x_i = rand-like U[0,1), y = 0 (alpha = 1, beta = 0)
    std::vector<V> x(std::max<int64_t>(n, 1)), y_ref(std::max<int64_t>(m, 1)), y(std::max<int64_t>(m, 1));
    if (vt == SSPMV_F64) sspmv_synth_vector_f64(n, 13, (double *)x.data());
    else sspmv_synth_vector_f32(n, 13, (float *)x.data());
    for (auto &v : x) v = (v + V(1)) / V(2);
    DevBuf dx(x.size() * sizeof(V) + 256), dy(y.size() * sizeof(V)), dyr(y.size() * sizeof(V));
    if (!dx.p || !dy.p || !dyr.p) {
        fprintf(stderr, "device allocation failed\n");
        return 1;
    }
    cudaMemset(dx.p, 0, x.size() * sizeof(V) + 256);
    cudaMemcpy(dx.p, x.data(), n * sizeof(V), cudaMemcpyHostToDevice);
    cudaMemset(dy.p, 0, m * sizeof(V));
    cudaMemset(dyr.p, 0, m * sizeof(V));
    CHECK(sspmv_LeSpMV_csr(1.0, &F.csr, dx.p, 0.0, dyr.p, nullptr));
    CHECK(F.spmv(1.0, dx.p, 0.0, dy.p));
    cudaMemcpy(y_ref.data(), dyr.p, m * sizeof(V), cudaMemcpyDeviceToHost);
    cudaMemcpy(y.data(), dy.p, m * sizeof(V), cudaMemcpyDeviceToHost);
    const double err = (double)max_relative_error(y_ref, y, (size_t)m);
    printf("\ttesting %-26s[gpu]: [max error %9f]", (fmt + "_gpu").c_str(), err);
    const double eps = std::numeric_limits<V>::epsilon();
    if (err > 5 * std::sqrt(eps) && err < 0.01) printf(" POSSIBLE small Round-Error");
    else if (err >= 0.005) printf(" POSSIBLE FAILURE");
    printf("\n");

    // timing: warm-up estimate, then the reference's iteration rule
    cudaEventRecord(e0);
    CHECK(F.spmv(1.0, dx.p, 0.0, dy.p));
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float est = 0;
    cudaEventElapsedTime(&est, e0, e1);
    const int max_iter = argint(argc, argv, "iters", 1000), min_iter = std::min(20, max_iter);
    int iters = max_iter;
    if (est >= 20) iters = std::min(max_iter, std::max(min_iter, (int)(20.0 * 1000 / est)));
    printf("\tPerforming %d iterations\n", iters);
    cudaEventRecord(e0);
    for (int i = 0; i < iters; i++) CHECK(F.spmv(1.0, dx.p, 0.0, dy.p));
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float total = 0;
    cudaEventElapsedTime(&total, e0, e1);
    const cudaError_t ce = cudaGetLastError();
    if (ce != cudaSuccess) {
        fprintf(stderr, "CUDA error: %s\n", cudaGetErrorString(ce));
        return 1;
    }
    const double msec = total / iters, sec = msec / 1000.0;
    const double gflops = sec == 0 ? 0 : 2.0 * (double)nnz / sec / 1e9;
    const char *bytes_model = get_argval(argc, argv, "bytes");
    const bool algorithmic = bytes_model && strcmp(bytes_model, "algorithmic") == 0;
    const double nbytes = algorithmic ? F.algorithmic_bytes() : F.reference_bytes();
    const double gbytes = sec == 0 || nbytes < 0 ? 0 : nbytes / sec / 1e9;
    printf("\tbenchmarking %-20s [%s]: %8.4f ms ( %5.4f GFLOP/s %5.4f GB/s)\n", (fmt + "_gpu").c_str(), "gpu", msec,
           gflops, gbytes);

    const char *perf = get_argval(argc, argv, "perf");
    const std::string perf_path = perf ? perf : "./performance/mat_perf.txt";
    FILE *fp = fopen(perf_path.c_str(), "a");
    if (!fp) {
        printf("Unable to open perf-saved file: %s\n", perf_path.c_str());
    } else {
        const std::string name = stem(path);
        const int chunk = F.fmt == "sell" ? F.sell.sliceWidth : F.fmt == "sell_c_sigma" ? F.scs.chunkWidth_C
                          : F.fmt == "sell_c_R" ? F.scr.chunkWidth_C : 4;
        const double cv_ms = convert_ms;
        if (fmt == "csr") fprintf(fp, "%d %s CSR %d %d %8.4f %5.4f \n", matID, name.c_str(), 2, sche, msec, gflops);
        else if (fmt == "coo")
            fprintf(fp, "%d %s COO %d %d %8.4f %5.4f %5.4f \n", matID, name.c_str(), 1, sche, msec, gflops, cv_ms);
        else if (fmt == "bsr")
            fprintf(fp, "%d %s BSR %d %d %8.4f %5.4f %5.4f \n", matID, name.c_str(), 2, sche, msec, gflops, cv_ms);
        else if (fmt == "csr5") fprintf(fp, "%d %s CSR5 %8.4f %5.4f \n", matID, name.c_str(), msec, gflops);
        else if (fmt == "dia")
            fprintf(fp, "%d %s DIA %d %d %8.4f %5.4f %5.4f \n", matID, name.c_str(), 1, sche, msec, gflops, cv_ms);
        else if (fmt == "ell")
            fprintf(fp, "%d %s ELL %d %d %8.4f %5.4f %5.4f \n", matID, name.c_str(), 2, sche, msec, gflops, cv_ms);
        else if (fmt == "sell")
            fprintf(fp, "%d %s S-ELL %d %d %d %8.4f %5.4f %5.4f \n", matID, name.c_str(), 2, sche, chunk, msec, gflops,
                    cv_ms);
        else if (fmt == "sell_c_R")
            fprintf(fp, "%d %s S-ELL-R %d %d %d %8.4f %5.4f \n", matID, name.c_str(), 2, sche, chunk, msec, gflops);
        else if (fmt == "sell_c_sigma")
            fprintf(fp, "%d %s S-ELL-sigma %d %d %d %d %8.4f %5.4f %5.4f \n", matID, name.c_str(), 2, sche, chunk,
                    F.scs.sliceWidth_Sigma, msec, gflops, cv_ms);
        fclose(fp);
    }
    F.release();
    sspmv_delete_csr(&F.csr);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return 0;
}

}  // namespace

int main(int argc, char **argv) {
    std::string prog = argv[0];
    const size_t slash = prog.find_last_of('/');
    if (slash != std::string::npos) prog = prog.substr(slash + 1);
    if (get_arg(argc, argv, "help")) {
        usage(prog.c_str());
        return EXIT_SUCCESS;
    }
    std::string fmt;
    if (const char *f = get_argval(argc, argv, "format")) fmt = f;
    else if (prog.rfind("benchmark_spmv_", 0) == 0) fmt = prog.substr(strlen("benchmark_spmv_"));
    bool known = false;
    for (const char *k : kFormats) known |= fmt == k;
    if (!known) {
        fprintf(stderr, "unknown format '%s' (program name benchmark_spmv_<fmt> or --format=<fmt>)\n", fmt.c_str());
        usage(prog.c_str());
        return EXIT_FAILURE;
    }
    const int precision = argint(argc, argv, "precision", 32);
    const int index = argint(argc, argv, "Index", 0);
    const int threads = argint(argc, argv, "threads", 0);
    printf("\nUsing %d-bit floating point precision, %d-bit Index, threads = %d\n\n", precision, (index + 1) * 32,
           threads);
    if (index != 0 || (precision != 32 && precision != 64)) {
        if (index != 0) fprintf(stderr, "--Index=%d: 64-bit indices are not supported (int32 indices only)\n", index);
        usage(prog.c_str());
        return EXIT_FAILURE;
    }
    const char *path = nullptr;
    for (int i = 1; i < argc; i++)
        if (argv[i][0] != '-') {
            path = argv[i];
            break;
        }
    if (!path) {
        printf("You need to input a matrix file!\n");
        return EXIT_FAILURE;
    }
    const int rc = precision == 64 ? run<double>(argc, argv, fmt, path, SSPMV_F64)
                                   : run<float>(argc, argv, fmt, path, SSPMV_F32);
    return rc == 0 ? EXIT_SUCCESS : EXIT_FAILURE;
}
