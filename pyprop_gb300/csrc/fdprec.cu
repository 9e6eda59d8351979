// Fast-diagonalization solve of the separable part of a two-electron channel block.
//
// For a coupled channel a = (l1, l2, L, M) the block of the Cayley matrix that is separable in
// the two radial coordinates is
//     M_a = cS S x S + cH (h_l1 x S + S x h_l2),
// h_l = -1/2 d^2/dr^2 + l(l+1)/(2 r^2) - z/r the one-electron radial Hamiltonian and S the
// B-spline overlap. With the generalized eigenvectors h_l V_l = S V_l Lambda_l (V^T S V = 1),
//     M_a^-1 = (V_l1 x V_l2) D_a (V_l1 x V_l2)^T,   D_a[i][j] = 1 / (cS + cH (lambda_l1,i + lambda_l2,j)),
// exact for this part (the reference's two-electron block preconditioners factor the whole
// channel block including the electron-electron repulsion with sparse LU / ILU,
// examples/tensor/helium_stabilization/preconditioner.py:77-244; the repulsion is what remains
// for GMRES and for the learned correction). On a channel's N x N radial block X:
//     Y = V1 (D o (V1^T X V2)) V2^T,
// four dense N x N x N products. One CTA per channel keeps V1, V2 and X in shared memory and
// runs the four products in place (each thread: a 4 x 4 tile of outputs in registers, all
// reads done before the barrier that precedes the write-back).
#include "pg_internal.cuh"

#include <algorithm>

namespace {

// four consecutive entries of a shared-memory row (16-byte aligned: the row offset and the
// column are multiples of 4) as 16-byte vector loads: fewer instructions and bank conflicts
__device__ __forceinline__ void fd_ld4(const float *p, float (&v)[4])
{
    const float4 q = *reinterpret_cast<const float4 *>(p);
    v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
}
__device__ __forceinline__ void fd_ld4(const double *p, double (&v)[4])
{
    const double2 a = *reinterpret_cast<const double2 *>(p), b = *reinterpret_cast<const double2 *>(p + 2);
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}
__device__ __forceinline__ void fd_ld4(const cx<float> *p, cx<float> (&v)[4])
{
    const float4 a = *reinterpret_cast<const float4 *>(p), b = *reinterpret_cast<const float4 *>(p + 2);
    v[0] = mk<float>(a.x, a.y); v[1] = mk<float>(a.z, a.w); v[2] = mk<float>(b.x, b.y); v[3] = mk<float>(b.z, b.w);
}
__device__ __forceinline__ void fd_ld4(const cx<double> *p, cx<double> (&v)[4])
{
#pragma unroll
    for (int w = 0; w < 4; ++w) {
        const double2 q = *reinterpret_cast<const double2 *>(p + w);
        v[w] = mk<double>(q.x, q.y);
    }
}

template <typename R>
__global__ void __launch_bounds__(1024) fd_solve_kernel(int N, int NP, const R *__restrict__ V,
                                                        const cx<R> *__restrict__ D, const int *__restrict__ lidx,
                                                        cx<R> *__restrict__ x)
{
    extern __shared__ __align__(16) unsigned char fd_smem[];
    const int a = blockIdx.x;
    const int l1 = lidx[2 * a], l2 = lidx[2 * a + 1];
    const size_t vsz = (size_t)NP * NP;
    R *V1 = reinterpret_cast<R *>(fd_smem);
    R *V2 = l1 == l2 ? V1 : V1 + vsz;
    cx<R> *X = reinterpret_cast<cx<R> *>(fd_smem + 2 * vsz * sizeof(R));  // [NP][NP]
    const int tid = threadIdx.x, nt = blockDim.x;
    for (size_t t = tid; t < vsz; t += nt) {
        V1[t] = V[(size_t)l1 * vsz + t];
        if (l1 != l2) V2[t] = V[(size_t)l2 * vsz + t];
    }
    cx<R> *xa = x + (size_t)a * N * N;
    for (int t = tid; t < NP * NP; t += nt) {
        const int i = t / NP, j = t - i * NP;
        X[t] = (i < N && j < N) ? xa[(size_t)i * N + j] : mk<R>((R)0, (R)0);
    }
    __syncthreads();
    const int TN = NP / 4;
    const int ti = tid / TN, tj = tid - ti * TN;
    const bool act = ti < TN;
    const int i0 = 4 * ti, j0 = 4 * tj;
    cx<R> acc[4][4];
    auto zero = [&]() {
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int v = 0; v < 4; ++v) acc[u][v] = mk<R>((R)0, (R)0);
    };
    // step 1: T = V1^T X   (T[i][j] = sum_k V1[k][i] X[k][j])
    zero();
    if (act)
        for (int k = 0; k < NP; ++k) {
            R v[4];
            cx<R> xv[4];
            fd_ld4(V1 + (size_t)k * NP + i0, v);
            fd_ld4(X + (size_t)k * NP + j0, xv);
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int w = 0; w < 4; ++w) {
                    acc[u][w].x = fma(v[u], xv[w].x, acc[u][w].x);
                    acc[u][w].y = fma(v[u], xv[w].y, acc[u][w].y);
                }
        }
    __syncthreads();
    if (act)
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int w = 0; w < 4; ++w) X[(size_t)(i0 + u) * NP + j0 + w] = acc[u][w];
    __syncthreads();
    // step 2: T = D o (T V2)   (sum_k T[i][k] V2[k][j])
    zero();
    if (act)
        for (int k = 0; k < NP; ++k) {
            R v[4];
            fd_ld4(V2 + (size_t)k * NP + j0, v);
            cx<R> tv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) tv[u] = X[(size_t)(i0 + u) * NP + k];
#pragma unroll
            for (int w = 0; w < 4; ++w)
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    acc[u][w].x = fma(v[w], tv[u].x, acc[u][w].x);
                    acc[u][w].y = fma(v[w], tv[u].y, acc[u][w].y);
                }
        }
    __syncthreads();
    if (act) {
        const cx<R> *Da = D + (size_t)a * N * N;
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int w = 0; w < 4; ++w) {
                const int i = i0 + u, j = j0 + w;
                X[(size_t)i * NP + j] = (i < N && j < N) ? Da[(size_t)i * N + j] * acc[u][w] : mk<R>((R)0, (R)0);
            }
    }
    __syncthreads();
    // step 3: T = V1 T   (sum_k V1[i][k] T[k][j])
    zero();
    if (act)
        for (int k = 0; k < NP; ++k) {
            cx<R> xv[4];
            fd_ld4(X + (size_t)k * NP + j0, xv);
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const R v = V1[(size_t)(i0 + u) * NP + k];
#pragma unroll
                for (int w = 0; w < 4; ++w) {
                    acc[u][w].x = fma(v, xv[w].x, acc[u][w].x);
                    acc[u][w].y = fma(v, xv[w].y, acc[u][w].y);
                }
            }
        }
    __syncthreads();
    if (act)
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int w = 0; w < 4; ++w) X[(size_t)(i0 + u) * NP + j0 + w] = acc[u][w];
    __syncthreads();
    // step 4: Y = T V2^T   (sum_k T[i][k] V2[j][k]), straight to the channel's block
    zero();
    if (act)
        for (int k = 0; k < NP; ++k) {
#pragma unroll
            for (int w = 0; w < 4; ++w) {
                const R v = V2[(size_t)(j0 + w) * NP + k];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const cx<R> tv = X[(size_t)(i0 + u) * NP + k];
                    acc[u][w].x = fma(v, tv.x, acc[u][w].x);
                    acc[u][w].y = fma(v, tv.y, acc[u][w].y);
                }
            }
        }
    if (act)
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int w = 0; w < 4; ++w) {
                const int i = i0 + u, j = j0 + w;
                if (i < N && j < N) xa[(size_t)i * N + j] = acc[u][w];
            }
}

template <typename R>
size_t fd_smem(int NP)
{
    return 2 * (size_t)NP * NP * sizeof(R) + (size_t)NP * NP * sizeof(cx<R>);
}

// ---- radial sizes beyond the shared-memory kernel: the four products as batched GEMMs on
// planar (real, imaginary) copies in global memory. Batch z = 2 a + c (channel a, part c).
// x [A][N][N] complex <-> P [A][2][N][N] real
template <typename R>
__global__ void fd_split_kernel(const cx<R> *__restrict__ x, R *__restrict__ P, long long NN, long long total)
{
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        const long long a = t / NN, e = t - a * NN;
        const cx<R> v = x[t];
        P[(2 * a) * NN + e] = v.x;
        P[(2 * a + 1) * NN + e] = v.y;
    }
}
template <typename R>
__global__ void fd_merge_kernel(const R *__restrict__ P, cx<R> *__restrict__ x, long long NN, long long total)
{
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        const long long a = t / NN, e = t - a * NN;
        x[t] = mk<R>(P[(2 * a) * NN + e], P[(2 * a + 1) * NN + e]);
    }
}
// Q = D o P (complex, planar)
template <typename R>
__global__ void fd_dmul_kernel(const R *__restrict__ P, const cx<R> *__restrict__ D, R *__restrict__ Q, long long NN,
                               long long total)
{
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        const long long a = t / NN, e = t - a * NN;
        const R re = P[(2 * a) * NN + e], im = P[(2 * a + 1) * NN + e];
        const cx<R> d = D[t];
        Q[(2 * a) * NN + e] = d.x * re - d.y * im;
        Q[(2 * a + 1) * NN + e] = d.x * im + d.y * re;
    }
}

// Batched N x N products C_z = op(A_z) op(B_z), row-major. MODE picks the operands of batch
// z = 2a + c: 1: V_l1^T S_z, 2: S_z V_l2, 3: V_l1 S_z, 4: S_z V_l2^T (V the eigenvector set of
// the channel's electron). 64 x 64 outputs per CTA, 256 threads with 4 x 4 each, K in steps of 16.
template <typename R, int MODE>
__global__ void __launch_bounds__(256) fd_gemm_kernel(int N, const R *__restrict__ V, const int *__restrict__ lidx,
                                                      const R *__restrict__ S, R *__restrict__ C)
{
    constexpr int TM = 64, TK = 16;
    __shared__ R As[TK][TM + 4];
    __shared__ R Bs[TK][TM + 4];
    const int z = blockIdx.z, a = z >> 1;
    const size_t NN = (size_t)N * N;
    const R *Vm = V + (size_t)lidx[2 * a + ((MODE == 1 || MODE == 3) ? 0 : 1)] * NN;
    const R *Sm = S + (size_t)z * NN;
    R *Cm = C + (size_t)z * NN;
    const int i0 = blockIdx.y * TM, j0 = blockIdx.x * TM;
    const int tid = threadIdx.x, tr = tid / 16, tcol = tid % 16;
    R acc[4][4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = (R)0;
    for (int k0 = 0; k0 < N; k0 += TK) {
        // As[kk][ii] = opA[i0 + ii][k0 + kk], Bs[kk][jj] = opB[k0 + kk][j0 + jj]
        for (int t = tid; t < TK * TM; t += 256) {
            const int kk = t / TM, ii = t - kk * TM;
            const int i = i0 + ii, k = k0 + kk;
            R av = (R)0;
            if (i < N && k < N) {
                if (MODE == 1) av = Vm[(size_t)k * N + i];       // V^T
                else if (MODE == 3) av = Vm[(size_t)i * N + k];  // V
                else av = Sm[(size_t)i * N + k];                 // S
            }
            As[kk][ii] = av;
            const int j = j0 + ii;
            R bv = (R)0;
            if (j < N && k < N) {
                if (MODE == 2) bv = Vm[(size_t)k * N + j];       // V
                else if (MODE == 4) bv = Vm[(size_t)j * N + k];  // V^T
                else bv = Sm[(size_t)k * N + j];                 // S
            }
            Bs[kk][ii] = bv;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < TK; ++kk) {
            R ar[4], br[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) ar[u] = As[kk][tr * 4 + u];
#pragma unroll
            for (int v = 0; v < 4; ++v) br[v] = Bs[kk][tcol * 4 + v];
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] = fma(ar[u], br[v], acc[u][v]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int i = i0 + tr * 4 + u, j = j0 + tcol * 4 + v;
            if (i < N && j < N) Cm[(size_t)i * N + j] = acc[u][v];
        }
}

template <typename R>
int fd_apply_global(pg_banded *b, void *x)
{
    pg_ctx *ctx = b->op->ctx;
    const int A = b->op->shape[0], N = b->fdN;
    const long long NN = (long long)N * N, total = (long long)A * NN;
    cudaStream_t s = ctx->stream;
    const int eb = (int)std::min<long long>((total + 255) / 256, 152LL * 16);
    R *P0 = (R *)b->d_fdP0, *P1 = (R *)b->d_fdP1;
    const R *V = (const R *)b->d_fdV;
    dim3 g((N + 63) / 64, (N + 63) / 64, 2 * A);
    fd_split_kernel<R><<<eb, 256, 0, s>>>((const cx<R> *)x, P0, NN, total);
    fd_gemm_kernel<R, 1><<<g, 256, 0, s>>>(N, V, b->d_fdl, P0, P1);
    fd_gemm_kernel<R, 2><<<g, 256, 0, s>>>(N, V, b->d_fdl, P1, P0);
    fd_dmul_kernel<R><<<eb, 256, 0, s>>>(P0, (const cx<R> *)b->d_fdD, P1, NN, total);
    fd_gemm_kernel<R, 3><<<g, 256, 0, s>>>(N, V, b->d_fdl, P1, P0);
    fd_gemm_kernel<R, 4><<<g, 256, 0, s>>>(N, V, b->d_fdl, P0, P1);
    fd_merge_kernel<R><<<eb, 256, 0, s>>>(P1, (cx<R> *)x, NN, total);
    ctx->launches += 7;
    return pg_check_launch(ctx);
}

}  // namespace

int pg_fd_max_n(int precision)
{
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
    int n = 4;
    while (n + 4 <= 128 && (precision == PG_FP64 ? fd_smem<double>(n + 4) : fd_smem<float>(n + 4)) <= (size_t)optin)
        n += 4;
    return n;
}

int pg_fd_apply_dev(pg_banded *b, void *x)
{
    if (b->fdGlobal)
        return b->op->precision == PG_FP64 ? fd_apply_global<double>(b, x) : fd_apply_global<float>(b, x);
    pg_ctx *ctx = b->op->ctx;
    const int A = b->op->shape[0], NP = b->fdNP;
    const int TN = NP / 4;
    const int threads = ((TN * TN + 31) / 32) * 32;
    if (b->op->precision == PG_FP64)
        fd_solve_kernel<double><<<A, threads, fd_smem<double>(NP), ctx->stream>>>(
            b->fdN, NP, (const double *)b->d_fdV, (const cxd *)b->d_fdD, b->d_fdl, (cxd *)x);
    else
        fd_solve_kernel<float><<<A, threads, fd_smem<float>(NP), ctx->stream>>>(
            b->fdN, NP, (const float *)b->d_fdV, (const cxf *)b->d_fdD, b->d_fdl, (cxf *)x);
    ctx->launches++;
    return pg_check_launch(ctx);
}

int pg_fd_prepare(int precision, int NP)
{
    int dev = 0, optin = 0;
    PG_CUDA_TRY(cudaGetDevice(&dev));
    PG_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    const size_t need = precision == PG_FP64 ? fd_smem<double>(NP) : fd_smem<float>(NP);
    if (need > (size_t)optin || NP > 128) return PG_ERR_SHAPE;
    if (precision == PG_FP64)
        PG_CUDA_TRY(cudaFuncSetAttribute(fd_solve_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    else
        PG_CUDA_TRY(cudaFuncSetAttribute(fd_solve_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    return PG_OK;
}

int pg_fd_kernels(const pg_banded *b) { return b->fdGlobal ? 7 : 1; }
