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

namespace {

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
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const R v = V1[(size_t)k * NP + i0 + u];
#pragma unroll
                for (int w = 0; w < 4; ++w) {
                    const cx<R> xv = X[(size_t)k * NP + j0 + w];
                    acc[u][w].x = fma(v, xv.x, acc[u][w].x);
                    acc[u][w].y = fma(v, xv.y, acc[u][w].y);
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
    // step 2: T = D o (T V2)   (sum_k T[i][k] V2[k][j])
    zero();
    if (act)
        for (int k = 0; k < NP; ++k) {
#pragma unroll
            for (int w = 0; w < 4; ++w) {
                const R v = V2[(size_t)k * NP + j0 + w];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const cx<R> tv = X[(size_t)(i0 + u) * NP + k];
                    acc[u][w].x = fma(v, tv.x, acc[u][w].x);
                    acc[u][w].y = fma(v, tv.y, acc[u][w].y);
                }
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
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const R v = V1[(size_t)(i0 + u) * NP + k];
#pragma unroll
                for (int w = 0; w < 4; ++w) {
                    const cx<R> xv = X[(size_t)k * NP + j0 + w];
                    acc[u][w].x = fma(v, xv.x, acc[u][w].x);
                    acc[u][w].y = fma(v, xv.y, acc[u][w].y);
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
