// Small learned preconditioner network: a bias-free 3-layer MLP with ReLU,
//     y = W3^T relu(W2^T relu(W1^T x)),
// BF16 weights and activations into BF16 tensor-core products with FP32 accumulation, FP32
// master weights, gradients and Adam moments. It acts per angular block: one row of X per
// block. The reference has no learned component; the solve it accelerates is the block
// preconditioner of CayleyPropagator (pyprop/propagator/CayleyPropagator.py:56-63,91-96).
//
// Products are tiled 64 x 64 x 32 per CTA (4 warps, 2 x 2 16x16 fragments each). Operands are
// staged through shared memory with an optional transpose on load, so the same kernel forms
// X W (forward), dY W^T (backward data) and X^T dY (weight gradients). The batch (the number
// of angular blocks, tens to a few thousand rows) and the widths (hundreds to a few thousand)
// make these products weight-bandwidth bound at inference and small at training.
#include "pg_internal.cuh"

#include <cuda_bf16.h>
#include <mma.h>

#include <random>

using namespace nvcuda;
typedef __nv_bfloat16 bf16;

static const int GT_M = 64, GT_N = 64, GT_K = 32;
static const int GT_LDA = GT_K + 8, GT_LDB = GT_N + 8, GT_LDC = GT_N + 4;

// Epilogues: 0 store FP32; 1 ReLU, store BF16 (and FP32 when given); 2 multiply by the ReLU
// mask (mask > 0), store BF16 (and FP32 when given).
enum { EPI_F32 = 0, EPI_RELU = 1, EPI_MASK = 2 };

// C[M][N] = op(A)[M][K] op(B)[K][N]; A(i,k) = ta ? A[k*lda+i] : A[i*lda+k],
// B(k,j) = tb ? B[j*ldb+k] : B[k*ldb+j]. With Cacc (FP32 [M][N], zeroed before) the K range is
// split over gridDim.z: each slice adds its partial product with atomics and the epilogue runs
// in mlp_epilogue_kernel (products with few output tiles and a long K, such as the first
// layer's 38400-wide input, would otherwise occupy a handful of SMs).
template <int EPI>
__global__ void __launch_bounds__(128) mlp_gemm_kernel(int M, int N, int K, const bf16 *__restrict__ A, int lda, int ta,
                                                       const bf16 *__restrict__ B, int ldb, int tb, float *C, int ldc,
                                                       bf16 *Cb, int ldcb, const bf16 *__restrict__ mask, int ldm,
                                                       float *Cacc)
{
    __shared__ __align__(32) bf16 As[GT_M * GT_LDA];
    __shared__ __align__(32) bf16 Bs[GT_K * GT_LDB];
    __shared__ __align__(32) float Cs[GT_M * GT_LDC];
    const int warp = threadIdx.x >> 5;
    const int m0 = blockIdx.y * GT_M, n0 = blockIdx.x * GT_N;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    wmma::fragment<wmma::accumulator, 16, 16, 16, float> acc[2][2];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b) wmma::fill_fragment(acc[a][b], 0.0f);
    const bf16 zero = __float2bfloat16(0.0f);
    const int kper = ((K + (int)gridDim.z - 1) / (int)gridDim.z + GT_K - 1) / GT_K * GT_K;
    const int kbeg = (int)blockIdx.z * kper, kend = min(K, kbeg + kper);
    for (int k0 = kbeg; k0 < kend; k0 += GT_K) {
        for (int e = threadIdx.x; e < GT_M * GT_K; e += 128) {
            const int i = e / GT_K, k = e % GT_K;
            const int gi = m0 + i, gk = k0 + k;
            bf16 v = zero;
            if (gi < M && gk < kend) v = ta ? A[(size_t)gk * lda + gi] : A[(size_t)gi * lda + gk];
            As[i * GT_LDA + k] = v;
        }
        for (int e = threadIdx.x; e < GT_K * GT_N; e += 128) {
            const int k = e / GT_N, j = e % GT_N;
            const int gk = k0 + k, gj = n0 + j;
            bf16 v = zero;
            if (gk < kend && gj < N) v = tb ? B[(size_t)gj * ldb + gk] : B[(size_t)gk * ldb + gj];
            Bs[k * GT_LDB + j] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GT_K; kk += 16) {
            wmma::fragment<wmma::matrix_a, 16, 16, 16, bf16, wmma::row_major> fa[2];
            wmma::fragment<wmma::matrix_b, 16, 16, 16, bf16, wmma::row_major> fb[2];
#pragma unroll
            for (int a = 0; a < 2; ++a) wmma::load_matrix_sync(fa[a], As + (wm + 16 * a) * GT_LDA + kk, GT_LDA);
#pragma unroll
            for (int b = 0; b < 2; ++b) wmma::load_matrix_sync(fb[b], Bs + kk * GT_LDB + wn + 16 * b, GT_LDB);
#pragma unroll
            for (int a = 0; a < 2; ++a)
#pragma unroll
                for (int b = 0; b < 2; ++b) wmma::mma_sync(acc[a][b], fa[a], fb[b], acc[a][b]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b)
            wmma::store_matrix_sync(Cs + (wm + 16 * a) * GT_LDC + wn + 16 * b, acc[a][b], GT_LDC, wmma::mem_row_major);
    __syncthreads();
    for (int e = threadIdx.x; e < GT_M * GT_N; e += 128) {
        const int i = e / GT_N, j = e % GT_N;
        const int gi = m0 + i, gj = n0 + j;
        if (gi >= M || gj >= N) continue;
        float v = Cs[i * GT_LDC + j];
        if (Cacc) {
            atomicAdd(Cacc + (size_t)gi * N + gj, v);
            continue;
        }
        if (EPI == EPI_RELU) v = fmaxf(v, 0.0f);
        if (EPI == EPI_MASK && !(__bfloat162float(mask[(size_t)gi * ldm + gj]) > 0.0f)) v = 0.0f;
        if (C) C[(size_t)gi * ldc + gj] = v;
        if (EPI != EPI_F32) Cb[(size_t)gi * ldcb + gj] = __float2bfloat16(v);
    }
}

// the epilogue of a K-split product on its summed FP32 result
template <int EPI>
__global__ void mlp_epilogue_kernel(int M, int N, const float *__restrict__ Cacc, float *C, int ldc, bf16 *Cb, int ldcb,
                                    const bf16 *__restrict__ mask, int ldm)
{
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)M * N;
         e += (long long)gridDim.x * blockDim.x) {
        const int gi = (int)(e / N), gj = (int)(e - (long long)gi * N);
        float v = Cacc[e];
        if (EPI == EPI_RELU) v = fmaxf(v, 0.0f);
        if (EPI == EPI_MASK && !(__bfloat162float(mask[(size_t)gi * ldm + gj]) > 0.0f)) v = 0.0f;
        if (C) C[(size_t)gi * ldc + gj] = v;
        if (EPI != EPI_F32) Cb[(size_t)gi * ldcb + gj] = __float2bfloat16(v);
    }
}

// dY = 2 (Y - T) / batch as BF16, loss += sum (Y - T)^2 / batch (FP64 atomic)
__global__ void mlp_loss_kernel(const float *__restrict__ Y, const float *__restrict__ T, long long n, float inv_batch,
                                bf16 *__restrict__ dY, double *loss)
{
    double part = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float d = Y[i] - T[i];
        dY[i] = __float2bfloat16(2.0f * d * inv_batch);
        part += (double)d * d * inv_batch;
    }
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((threadIdx.x & 31) == 0 && part != 0.0) atomicAdd(loss, part);
}

// Adam on the FP32 master weights; the BF16 copy used by the products follows.
__global__ void mlp_adam_kernel(float *__restrict__ w, bf16 *__restrict__ wb, const float *__restrict__ g,
                                float *__restrict__ m1, float *__restrict__ m2, long long n, float lr, float b1, float b2,
                                float eps, float c1, float c2)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float a = b1 * m1[i] + (1.0f - b1) * gi;
        const float b = b2 * m2[i] + (1.0f - b2) * gi * gi;
        m1[i] = a;
        m2[i] = b;
        const float upd = lr * (a / c1) / (sqrtf(b / c2) + eps);
        const float nw = w[i] - upd;
        w[i] = nw;
        wb[i] = __float2bfloat16(nw);
    }
}

__global__ void f32_to_bf16_kernel(const float *__restrict__ x, bf16 *__restrict__ y, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        y[i] = __float2bfloat16(x[i]);
}

// Block features: row a = [y_{a-1}, y_a, y_{a+1}] (real/imaginary interleaved, zero outside
// 0..nblk-1 and in the padding up to d_in), scaled by `scale` (device FP64, optional: 1/||y||).
__global__ void mlp_block_features_kernel(const cxf *__restrict__ y, int nblk, int N, int d_in,
                                          const double *__restrict__ inv_scale, bf16 *__restrict__ X)
{
    const float s = inv_scale ? (float)*inv_scale : 1.0f;
    const long long total = (long long)nblk * d_in;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int a = (int)(e / d_in), c = (int)(e % d_in);
        float v = 0.0f;
        if (c < 6 * N) {
            const int nb = a - 1 + c / (2 * N);
            const int i = (c % (2 * N)) >> 1;
            if (nb >= 0 && nb < nblk) {
                const cxf z = y[(size_t)nb * N + i];
                v = (c & 1) ? z.y : z.x;
            }
        }
        X[e] = __float2bfloat16(v * s);
    }
}

// z = y + s * (out_re + i out_im) / inv_scale, out [nblk][2N] FP32 (the network's correction)
__global__ void mlp_apply_correction_kernel(const cxf *__restrict__ y, const float *__restrict__ out, int nblk, int N,
                                            int d_out, const cxd *__restrict__ s, const double *__restrict__ inv_scale,
                                            const int *__restrict__ enabled, cxf *__restrict__ z)
{
    const long long n = (long long)nblk * N;
    const bool on = !enabled || *enabled;
    const double is = inv_scale ? *inv_scale : 1.0;
    const float k = is > 0.0 ? (float)(1.0 / is) : 0.0f;
    const cxf sc = mk<float>((float)s->x * k, (float)s->y * k);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int a = (int)(e / N), i = (int)(e % N);
        cxf v = y[e];
        if (on) {
            const cxf o = mk<float>(out[(size_t)a * d_out + 2 * i], out[(size_t)a * d_out + 2 * i + 1]);
            v.x += sc.x * o.x - sc.y * o.y;
            v.y += sc.x * o.y + sc.y * o.x;
        }
        z[e] = v;
    }
}

// ------------------------------------------------------------------------------------
// host object
// ------------------------------------------------------------------------------------
struct pg_mlp {
    pg_ctx *ctx = nullptr;
    int d_in = 0, h = 0, d_out = 0;
    int rows[3] = {0, 0, 0}, cols[3] = {0, 0, 0};
    float *W[3] = {nullptr, nullptr, nullptr}, *G[3] = {nullptr, nullptr, nullptr};
    float *M1[3] = {nullptr, nullptr, nullptr}, *M2[3] = {nullptr, nullptr, nullptr};
    bf16 *Wb[3] = {nullptr, nullptr, nullptr};
    int adam_t = 0;
    int cap = 0;  // batch capacity of the activation buffers
    bf16 *h1 = nullptr, *h2 = nullptr, *dY = nullptr, *dh1 = nullptr, *dh2 = nullptr;
    float *y = nullptr;
    float *acc = nullptr;  // [cap][h] FP32 sums of K-split products
    double *d_loss = nullptr, *h_loss = nullptr;
    long long n(int l) const { return (long long)rows[l] * cols[l]; }
};

static int grid_for(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 1184)); }

template <int EPI>
static int gemm(pg_mlp *m, int M, int N, int K, const bf16 *A, int lda, int ta, const bf16 *B, int ldb, int tb, float *C,
                int ldc, bf16 *Cb, int ldcb, const bf16 *mask, int ldm)
{
    if (M <= 0 || N <= 0) return PG_OK;
    dim3 grid((N + GT_N - 1) / GT_N, (M + GT_M - 1) / GT_M);
    const int sms = std::max(1, m->ctx->num_sms);
    const long long tiles = (long long)grid.x * grid.y;
    int split = 1;
    if (tiles < sms && K >= 16 * GT_K && (long long)M * N <= (long long)m->cap * m->h && m->acc)
        split = (int)std::min<long long>((2LL * sms + tiles - 1) / tiles, K / (8 * GT_K));
    if (split > 1) {
        grid.z = split;
        PG_CUDA_TRY(cudaMemsetAsync(m->acc, 0, sizeof(float) * (size_t)M * N, m->ctx->stream));
        mlp_gemm_kernel<EPI><<<grid, 128, 0, m->ctx->stream>>>(M, N, K, A, lda, ta, B, ldb, tb, C, ldc, Cb, ldcb, mask,
                                                               ldm, m->acc);
        m->ctx->launches++;
        PG_TRY(pg_check_launch(m->ctx));
        mlp_epilogue_kernel<EPI><<<grid_for((long long)M * N), 256, 0, m->ctx->stream>>>(M, N, m->acc, C, ldc, Cb, ldcb,
                                                                                        mask, ldm);
        m->ctx->launches++;
        return pg_check_launch(m->ctx);
    }
    mlp_gemm_kernel<EPI><<<grid, 128, 0, m->ctx->stream>>>(M, N, K, A, lda, ta, B, ldb, tb, C, ldc, Cb, ldcb, mask, ldm,
                                                           nullptr);
    m->ctx->launches++;
    return pg_check_launch(m->ctx);
}

static int ensure_cap(pg_mlp *m, int batch)
{
    if (batch <= m->cap) return PG_OK;
    cudaFree(m->h1); cudaFree(m->h2); cudaFree(m->dY); cudaFree(m->dh1); cudaFree(m->dh2); cudaFree(m->y);
    cudaFree(m->acc);
    m->h1 = m->h2 = m->dY = m->dh1 = m->dh2 = nullptr;
    m->y = m->acc = nullptr;
    const size_t b = (size_t)batch;
    PG_CUDA_TRY(cudaMalloc(&m->h1, b * m->h * sizeof(bf16)));
    PG_CUDA_TRY(cudaMalloc(&m->h2, b * m->h * sizeof(bf16)));
    PG_CUDA_TRY(cudaMalloc(&m->dh1, b * m->h * sizeof(bf16)));
    PG_CUDA_TRY(cudaMalloc(&m->dh2, b * m->h * sizeof(bf16)));
    PG_CUDA_TRY(cudaMalloc(&m->dY, b * m->d_out * sizeof(bf16)));
    PG_CUDA_TRY(cudaMalloc(&m->y, b * m->d_out * sizeof(float)));
    PG_CUDA_TRY(cudaMalloc(&m->acc, b * m->h * sizeof(float)));
    m->cap = batch;
    return PG_OK;
}

// Y = MLP(X) for `batch` rows (X BF16 [batch][d_in], Y FP32 [batch][d_out]); keeps h1, h2.
int pg_mlp_forward_dev(pg_mlp *m, const void *X, int batch, float *Y)
{
    PG_TRY(ensure_cap(m, batch));
    PG_TRY(gemm<EPI_RELU>(m, batch, m->h, m->d_in, (const bf16 *)X, m->d_in, 0, m->Wb[0], m->h, 0, nullptr, 0, m->h1,
                          m->h, nullptr, 0));
    PG_TRY(gemm<EPI_RELU>(m, batch, m->h, m->h, m->h1, m->h, 0, m->Wb[1], m->h, 0, nullptr, 0, m->h2, m->h, nullptr,
                          0));
    return gemm<EPI_F32>(m, batch, m->d_out, m->h, m->h2, m->h, 0, m->Wb[2], m->d_out, 0, Y, m->d_out, nullptr, 0,
                         nullptr, 0);
}

// forward, mean squared error against T (FP32 [batch][d_out]) into d_loss, backward into G
static int forward_backward(pg_mlp *m, const void *X, const float *T, int batch)
{
    PG_TRY(pg_mlp_forward_dev(m, X, batch, m->y));
    cudaStream_t s = m->ctx->stream;
    const long long ny = (long long)batch * m->d_out;
    PG_CUDA_TRY(cudaMemsetAsync(m->d_loss, 0, sizeof(double), s));
    mlp_loss_kernel<<<grid_for(ny), 256, 0, s>>>(m->y, T, ny, 1.0f / (float)batch, m->dY, m->d_loss);
    m->ctx->launches++;
    PG_TRY(pg_check_launch(m->ctx));
    const int h = m->h, dout = m->d_out, din = m->d_in;
    // dW3 = h2^T dY ; dh2 = (dY W3^T) * [h2 > 0]
    PG_TRY(gemm<EPI_F32>(m, h, dout, batch, m->h2, h, 1, m->dY, dout, 0, m->G[2], dout, nullptr, 0, nullptr, 0));
    PG_TRY(gemm<EPI_MASK>(m, batch, h, dout, m->dY, dout, 0, m->Wb[2], dout, 1, nullptr, 0, m->dh2, h, m->h2, h));
    // dW2 = h1^T dh2 ; dh1 = (dh2 W2^T) * [h1 > 0]
    PG_TRY(gemm<EPI_F32>(m, h, h, batch, m->h1, h, 1, m->dh2, h, 0, m->G[1], h, nullptr, 0, nullptr, 0));
    PG_TRY(gemm<EPI_MASK>(m, batch, h, h, m->dh2, h, 0, m->Wb[1], h, 1, nullptr, 0, m->dh1, h, m->h1, h));
    // dW1 = X^T dh1
    return gemm<EPI_F32>(m, din, h, batch, (const bf16 *)X, din, 1, m->dh1, h, 0, m->G[0], h, nullptr, 0, nullptr, 0);
}

extern "C" int pg_mlp_create(pg_ctx *ctx, int d_in, int hidden, int d_out, unsigned long long seed, pg_mlp **out)
{
    if (!ctx || !out || d_in <= 0 || hidden <= 0 || d_out <= 0) return PG_ERR_ARG;
    if (d_in % 8 != 0 || hidden % 8 != 0 || d_out % 8 != 0) return PG_ERR_SHAPE;
    pg_mlp *m = new pg_mlp();
    m->ctx = ctx;
    m->d_in = d_in;
    m->h = hidden;
    m->d_out = d_out;
    const int r[3] = {d_in, hidden, hidden}, c[3] = {hidden, hidden, d_out};
    std::mt19937_64 gen(seed);
    for (int l = 0; l < 3; ++l) {
        m->rows[l] = r[l];
        m->cols[l] = c[l];
        const long long n = m->n(l);
        // He-normal for the ReLU layers; the last layer starts near zero so an untrained
        // network leaves the block preconditioner unchanged
        std::normal_distribution<float> nd(0.0f, l < 2 ? std::sqrt(2.0f / (float)r[l]) : 1e-3f / std::sqrt((float)r[l]));
        std::vector<float> w((size_t)n);
        for (auto &v : w) v = nd(gen);
        PG_CUDA_TRY(cudaMalloc(&m->W[l], n * sizeof(float)));
        PG_CUDA_TRY(cudaMalloc(&m->G[l], n * sizeof(float)));
        PG_CUDA_TRY(cudaMalloc(&m->M1[l], n * sizeof(float)));
        PG_CUDA_TRY(cudaMalloc(&m->M2[l], n * sizeof(float)));
        PG_CUDA_TRY(cudaMalloc(&m->Wb[l], n * sizeof(bf16)));
        PG_CUDA_TRY(cudaMemcpy(m->W[l], w.data(), n * sizeof(float), cudaMemcpyHostToDevice));
        PG_CUDA_TRY(cudaMemset(m->M1[l], 0, n * sizeof(float)));
        PG_CUDA_TRY(cudaMemset(m->M2[l], 0, n * sizeof(float)));
        f32_to_bf16_kernel<<<grid_for(n), 256, 0, ctx->stream>>>(m->W[l], m->Wb[l], n);
        PG_TRY(pg_check_launch(ctx));
    }
    PG_CUDA_TRY(cudaMalloc(&m->d_loss, sizeof(double)));
    PG_CUDA_TRY(cudaMallocHost(&m->h_loss, sizeof(double)));
    PG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    *out = m;
    return PG_OK;
}

extern "C" int pg_mlp_destroy(pg_mlp *m)
{
    if (!m) return PG_ERR_ARG;
    cudaStreamSynchronize(m->ctx->stream);
    for (int l = 0; l < 3; ++l) {
        cudaFree(m->W[l]); cudaFree(m->G[l]); cudaFree(m->M1[l]); cudaFree(m->M2[l]); cudaFree(m->Wb[l]);
    }
    cudaFree(m->h1); cudaFree(m->h2); cudaFree(m->dY); cudaFree(m->dh1); cudaFree(m->dh2); cudaFree(m->y);
    cudaFree(m->acc);
    cudaFree(m->d_loss);
    if (m->h_loss) cudaFreeHost(m->h_loss);
    delete m;
    return PG_OK;
}

extern "C" long long pg_mlp_parameter_count(const pg_mlp *m)
{
    return m ? m->n(0) + m->n(1) + m->n(2) : -1;
}

// host FP32 [W1 (d_in x h) | W2 (h x h) | W3 (h x d_out)], row-major (fan-in rows)
extern "C" int pg_mlp_get_weights(pg_mlp *m, float *host)
{
    if (!m || !host) return PG_ERR_ARG;
    PG_CUDA_TRY(cudaStreamSynchronize(m->ctx->stream));
    for (int l = 0; l < 3; ++l) {
        PG_CUDA_TRY(cudaMemcpy(host, m->W[l], m->n(l) * sizeof(float), cudaMemcpyDeviceToHost));
        host += m->n(l);
    }
    return PG_OK;
}

// sets the master weights (and their BF16 copy) and resets the optimizer state
extern "C" int pg_mlp_set_weights(pg_mlp *m, const float *host)
{
    if (!m || !host) return PG_ERR_ARG;
    PG_CUDA_TRY(cudaStreamSynchronize(m->ctx->stream));
    for (int l = 0; l < 3; ++l) {
        const long long n = m->n(l);
        PG_CUDA_TRY(cudaMemcpy(m->W[l], host, n * sizeof(float), cudaMemcpyHostToDevice));
        PG_CUDA_TRY(cudaMemset(m->M1[l], 0, n * sizeof(float)));
        PG_CUDA_TRY(cudaMemset(m->M2[l], 0, n * sizeof(float)));
        f32_to_bf16_kernel<<<grid_for(n), 256, 0, m->ctx->stream>>>(m->W[l], m->Wb[l], n);
        PG_TRY(pg_check_launch(m->ctx));
        host += n;
    }
    m->adam_t = 0;
    PG_CUDA_TRY(cudaStreamSynchronize(m->ctx->stream));
    return PG_OK;
}

extern "C" int pg_mlp_forward(pg_mlp *m, const void *X_bf16, int batch, float *Y)
{
    if (!m || !X_bf16 || !Y || batch < 0) return PG_ERR_ARG;
    return pg_mlp_forward_dev(m, X_bf16, batch, Y);
}

// loss = mean over rows of ||MLP(x) - t||^2 and its gradient (host FP32, layout of the weights)
extern "C" int pg_mlp_gradients(pg_mlp *m, const void *X_bf16, const float *T, int batch, double *loss,
                                float *grads_host)
{
    if (!m || !X_bf16 || !T || batch <= 0) return PG_ERR_ARG;
    PG_TRY(forward_backward(m, X_bf16, T, batch));
    PG_CUDA_TRY(cudaMemcpyAsync(m->h_loss, m->d_loss, sizeof(double), cudaMemcpyDeviceToHost, m->ctx->stream));
    PG_CUDA_TRY(cudaStreamSynchronize(m->ctx->stream));
    if (loss) *loss = *m->h_loss;
    if (grads_host)
        for (int l = 0; l < 3; ++l) {
            PG_CUDA_TRY(cudaMemcpy(grads_host, m->G[l], m->n(l) * sizeof(float), cudaMemcpyDeviceToHost));
            grads_host += m->n(l);
        }
    return PG_OK;
}

// one Adam step on a batch; loss (optional) waits for the step
extern "C" int pg_mlp_train_step(pg_mlp *m, const void *X_bf16, const float *T, int batch, float lr, double *loss)
{
    if (!m || !X_bf16 || !T || batch <= 0 || !(lr >= 0.0f)) return PG_ERR_ARG;
    PG_TRY(forward_backward(m, X_bf16, T, batch));
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    m->adam_t += 1;
    const float c1 = 1.0f - std::pow(b1, (float)m->adam_t), c2 = 1.0f - std::pow(b2, (float)m->adam_t);
    for (int l = 0; l < 3; ++l) {
        const long long n = m->n(l);
        mlp_adam_kernel<<<grid_for(n), 256, 0, m->ctx->stream>>>(m->W[l], m->Wb[l], m->G[l], m->M1[l], m->M2[l], n, lr,
                                                                 b1, b2, eps, c1, c2);
        m->ctx->launches++;
        PG_TRY(pg_check_launch(m->ctx));
    }
    if (loss) {
        PG_CUDA_TRY(cudaMemcpyAsync(m->h_loss, m->d_loss, sizeof(double), cudaMemcpyDeviceToHost, m->ctx->stream));
        PG_CUDA_TRY(cudaStreamSynchronize(m->ctx->stream));
        *loss = *m->h_loss;
    }
    return PG_OK;
}

int pg_mlp_block_features_dev(pg_ctx *ctx, const void *y, int nblk, int N, int d_in, const double *inv_scale, void *X)
{
    if (d_in < 6 * N) return PG_ERR_SHAPE;
    const long long total = (long long)nblk * d_in;
    mlp_block_features_kernel<<<grid_for(total), 256, 0, ctx->stream>>>((const cxf *)y, nblk, N, d_in, inv_scale,
                                                                        (bf16 *)X);
    ctx->launches++;
    return pg_check_launch(ctx);
}

int pg_mlp_apply_correction_dev(pg_ctx *ctx, const void *y, const float *out, int nblk, int N, int d_out,
                                const cxd *s, const double *inv_scale, const int *enabled, void *z)
{
    if (d_out < 2 * N) return PG_ERR_SHAPE;
    const long long n = (long long)nblk * N;
    mlp_apply_correction_kernel<<<grid_for(n), 256, 0, ctx->stream>>>((const cxf *)y, out, nblk, N, d_out, s,
                                                                      inv_scale, enabled, (cxf *)z);
    ctx->launches++;
    return pg_check_launch(ctx);
}

// Features of the block preconditioner's output y (complex64 [nblk][N]) for the network:
// row a = [y_{a-1}, y_a, y_{a+1}] re/im interleaved, zero-padded to d_in (BF16).
extern "C" int pg_mlp_block_features(pg_ctx *ctx, const void *y, int nblk, int N, int d_in, void *X_bf16)
{
    if (!ctx || !y || !X_bf16 || nblk <= 0 || N <= 0) return PG_ERR_ARG;
    return pg_mlp_block_features_dev(ctx, y, nblk, N, d_in, nullptr, X_bf16);
}

// internal: the network's context and widths; activation buffers for `batch` rows (so that
// a later forward pass inside stream capture does not allocate)
int pg_mlp_describe(pg_mlp *m, pg_ctx **ctx, int *d_in, int *d_out)
{
    if (!m) return PG_ERR_ARG;
    *ctx = m->ctx;
    *d_in = m->d_in;
    *d_out = m->d_out;
    return PG_OK;
}

int pg_mlp_reserve(pg_mlp *m, int batch) { return ensure_cap(m, batch); }
