// nn.cu -- FP32 kernels of the format selector's multilayer perceptron:
// dense layers (forward with bias and ReLU, backward), softmax cross-entropy,
// masked squared error and the Adam update.
//
// The reference's selector is a Keras network trained offline
// (SmartAdpter/models/SpMV_Adapter.py); here the network is small (about 140
// inputs, two hidden layers of 256, 9 + 9 outputs) and is trained and run on
// the GPU with these kernels, the host (PyTorch tensors for memory) only
// sequencing the calls.  Layer shapes are tiny -- a batch of at most a few
// thousand matrices -- so one tiled SIMT GEMM with transpose flags covers all
// products; tensor cores would not pay at this size.
#include "common.cuh"

namespace sspmv {
namespace {

constexpr int kTile = 32;  // C tile: 32 x 32, 16 x 16 threads, 2 x 2 outputs each

// C[M x N] = alpha * op(A)[M x K] * op(B)[K x N] + beta * C (+ bias[col], ReLU),
// row-major with leading dimensions; op(A)[i][k] = transA ? A[k*lda + i] : A[i*lda + k].
__global__ void __launch_bounds__(256) gemm_kernel(int M, int N, int K, const float *__restrict__ A, int lda,
                                                   int transA, const float *__restrict__ B, int ldb, int transB,
                                                   float alpha, float beta, float *__restrict__ C, int ldc,
                                                   const float *__restrict__ bias, int relu) {
    __shared__ float As[kTile][kTile + 1];
    __shared__ float Bs[kTile][kTile + 1];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int row0 = blockIdx.y * kTile, col0 = blockIdx.x * kTile;
    float acc[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
    for (int k0 = 0; k0 < K; k0 += kTile) {
        for (int e = threadIdx.x; e < kTile * kTile; e += 256) {
            const int r = e / kTile, c = e % kTile;
            const int gi = row0 + r, gk = k0 + c;
            As[r][c] = (gi < M && gk < K) ? (transA ? A[(int64_t)gk * lda + gi] : A[(int64_t)gi * lda + gk]) : 0.f;
            const int bk = k0 + r, bj = col0 + c;
            Bs[r][c] = (bk < K && bj < N) ? (transB ? B[(int64_t)bj * ldb + bk] : B[(int64_t)bk * ldb + bj]) : 0.f;
        }
        __syncthreads();
#pragma unroll 8
        for (int kk = 0; kk < kTile; kk++) {
            const float a0 = As[ty][kk], a1 = As[ty + 16][kk];
            const float b0 = Bs[kk][tx], b1 = Bs[kk][tx + 16];
            acc[0][0] += a0 * b0;
            acc[0][1] += a0 * b1;
            acc[1][0] += a1 * b0;
            acc[1][1] += a1 * b1;
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 2; j++) {
            const int gi = row0 + ty + 16 * i, gj = col0 + tx + 16 * j;
            if (gi < M && gj < N) {
                float v = alpha * acc[i][j];
                if (beta != 0.f) v += beta * C[(int64_t)gi * ldc + gj];
                if (bias) v += bias[gj];
                if (relu) v = fmaxf(v, 0.f);
                C[(int64_t)gi * ldc + gj] = v;
            }
        }
}

sspmv_status gemm(int M, int N, int K, const float *A, int lda, int transA, const float *B, int ldb, int transB,
                  float alpha, float beta, float *C, int ldc, const float *bias, int relu, sspmv_stream_t s) {
    if (M <= 0 || N <= 0) return SSPMV_OK;
    dim3 grid((N + kTile - 1) / kTile, (M + kTile - 1) / kTile);
    gemm_kernel<<<grid, 256, 0, cu(s)>>>(M, N, K, A, lda, transA, B, ldb, transB, alpha, beta, C, ldc, bias, relu);
    SSPMV_LAUNCH_CHECK();
    return SSPMV_OK;
}

// dy *= (y > 0) for a ReLU output y.
__global__ void relu_mask(int64_t n, const float *__restrict__ y, float *__restrict__ dy) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (!(y[i] > 0.f)) dy[i] = 0.f;
}

// db[j] = sum_b dy[b][j]
__global__ void column_sum(int B, int N, const float *__restrict__ dy, int ld, float *__restrict__ db) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N) return;
    float s = 0.f;
    for (int b = 0; b < B; b++) s += dy[(int64_t)b * ld + j];
    db[j] = s;
}

// One thread per row: softmax over C logits, loss -log p[label], dlogits =
// (p - onehot) / B.  Rows with label < 0 contribute nothing.
__global__ void softmax_xent_kernel(int B, int C, const float *__restrict__ logits, int ld,
                                    const int32_t *__restrict__ labels, float *__restrict__ dlogits, int ldd,
                                    float *__restrict__ loss_rows) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const float *z = logits + (int64_t)b * ld;
    float *dz = dlogits + (int64_t)b * ldd;
    const int lab = labels[b];
    float mx = -INFINITY;
    for (int c = 0; c < C; c++) mx = fmaxf(mx, z[c]);
    float sum = 0.f;
    for (int c = 0; c < C; c++) sum += expf(z[c] - mx);
    const float lse = mx + logf(sum);
    for (int c = 0; c < C; c++) {
        const float p = expf(z[c] - lse);
        dz[c] = lab < 0 ? 0.f : (p - (c == lab ? 1.f : 0.f)) / (float)B;
    }
    loss_rows[b] = lab < 0 ? 0.f : lse - z[lab];
}

// Masked squared error: d = w * 2 (pred - target) mask / count, loss rows.
__global__ void masked_mse_kernel(int B, int C, const float *__restrict__ pred, int ld, const float *__restrict__ target,
                                  const float *__restrict__ mask, float weight, float inv_count,
                                  float *__restrict__ dpred, int ldd, float *__restrict__ loss_rows) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    float l = 0.f;
    for (int c = 0; c < C; c++) {
        const float mk = mask[(int64_t)b * C + c];
        const float d = pred[(int64_t)b * ld + c] - target[(int64_t)b * C + c];
        dpred[(int64_t)b * ldd + c] = mk != 0.f ? weight * 2.f * d * inv_count : 0.f;
        l += mk != 0.f ? d * d : 0.f;
    }
    loss_rows[b] = l * inv_count;
}

__global__ void adam_kernel(int64_t n, float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                            float *__restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2,
                            float wd) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float gi = g[i] + wd * w[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

}  // namespace
}  // namespace sspmv

using namespace sspmv;

extern "C" sspmv_status sspmv_nn_linear_forward(int32_t B, int32_t in, int32_t out, const float *x, int32_t ldx,
                                                const float *W, const float *b, int32_t relu, float *y, int32_t ldy,
                                                sspmv_stream_t s) {
    if (B < 0 || in <= 0 || out <= 0 || !x || !W || !y || ldx < in || ldy < out)
        return fail(SSPMV_INVALID_ARG, "nn_linear_forward: bad arguments");
    // y = x W^T + b, W is out x in (row-major)
    return gemm(B, out, in, x, ldx, 0, W, in, 1, 1.f, 0.f, y, ldy, b, relu, s);
}

extern "C" sspmv_status sspmv_nn_linear_backward(int32_t B, int32_t in, int32_t out, const float *x, int32_t ldx,
                                                 const float *W, const float *y, int32_t relu, float *dy, int32_t ldy,
                                                 float *dx, int32_t lddx, float *dW, float *db, sspmv_stream_t s) {
    if (B <= 0 || in <= 0 || out <= 0 || !x || !W || !dy || !dW || !db || ldx < in || ldy < out)
        return fail(SSPMV_INVALID_ARG, "nn_linear_backward: bad arguments");
    if (relu) {
        if (!y) return fail(SSPMV_INVALID_ARG, "nn_linear_backward: relu needs the layer output");
        if (ldy != out) return fail(SSPMV_INVALID_ARG, "nn_linear_backward: relu needs ldy == out");
        relu_mask<<<grid_for((int64_t)B * out, 256, 1024), 256, 0, cu(s)>>>((int64_t)B * out, y, dy);
        SSPMV_LAUNCH_CHECK();
    }
    // dW[out x in] = dy^T x ; db = column sums of dy ; dx[B x in] = dy W
    SSPMV_TRY(gemm(out, in, B, dy, ldy, 1, x, ldx, 0, 1.f, 0.f, dW, in, nullptr, 0, s));
    column_sum<<<grid_for(out, 128), 128, 0, cu(s)>>>(B, out, dy, ldy, db);
    SSPMV_LAUNCH_CHECK();
    if (dx) SSPMV_TRY(gemm(B, in, out, dy, ldy, 0, W, in, 0, 1.f, 0.f, dx, lddx, nullptr, 0, s));
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_nn_softmax_xent(int32_t B, int32_t C, const float *logits, int32_t ld,
                                              const int32_t *labels, float *dlogits, int32_t ldd, float *loss_rows,
                                              sspmv_stream_t s) {
    if (B <= 0 || C <= 0 || !logits || !labels || !dlogits || !loss_rows || ld < C || ldd < C)
        return fail(SSPMV_INVALID_ARG, "nn_softmax_xent: bad arguments");
    softmax_xent_kernel<<<grid_for(B, 128), 128, 0, cu(s)>>>(B, C, logits, ld, labels, dlogits, ldd, loss_rows);
    SSPMV_LAUNCH_CHECK();
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_nn_masked_mse(int32_t B, int32_t C, const float *pred, int32_t ld, const float *target,
                                            const float *mask, float weight, float count, float *dpred, int32_t ldd,
                                            float *loss_rows, sspmv_stream_t s) {
    if (B <= 0 || C <= 0 || !pred || !target || !mask || !dpred || !loss_rows || ld < C || ldd < C || count <= 0)
        return fail(SSPMV_INVALID_ARG, "nn_masked_mse: bad arguments");
    masked_mse_kernel<<<grid_for(B, 128), 128, 0, cu(s)>>>(B, C, pred, ld, target, mask, weight, 1.f / count, dpred,
                                                           ldd, loss_rows);
    SSPMV_LAUNCH_CHECK();
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_nn_adam(int64_t n, float *w, const float *g, float *m, float *v, float lr, float beta1,
                                      float beta2, float eps, int32_t step, float weight_decay, sspmv_stream_t s) {
    if (n < 0 || step < 1 || (n > 0 && (!w || !g || !m || !v))) return fail(SSPMV_INVALID_ARG, "nn_adam: bad arguments");
    if (n == 0) return SSPMV_OK;
    const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
    adam_kernel<<<grid_for(n, 256, 2048), 256, 0, cu(s)>>>(n, w, g, m, v, lr, beta1, beta2, eps, c1, c2, weight_decay);
    SSPMV_LAUNCH_CHECK();
    return SSPMV_OK;
}
