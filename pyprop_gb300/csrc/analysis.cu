// Analysis of a final two-electron state: projections on products of single-electron radial
// states (examples/tensor/helium_stabilization/analysis.cpp:39-139). For the angular indices
// a of one (l1, l2) pair,
//     proj[a] = V1^H Psi_a conj(V2)                 (CalculateProjectionRadialProductStates)
//     psi_a  -= V1 proj[a] V2^T                     (RemoveProjectionRadialProductStates)
// with Psi_a the [N1][N2] radial block of the weighted wavefunction (the overlap applied on
// both radial ranks, as the reference's callers do) and V1 [N1][n1], V2 [N2][n2] the radial
// states as columns. Each is two batched complex FP64 products, one batch entry per angular
// index: small dense work next to a propagation, run once per analysed state.
#include "pg_internal.cuh"

#include <vector>

namespace {

// operand forms: element (i, k) of op(X) for row-major X with leading dimension ld
enum { OP_N = 0, OP_T = 1, OP_C = 2, OP_J = 3 };  // X, X^T, X^H, conj(X)

__device__ __forceinline__ cxd op_load(const cxd *X, long long ld, int op, int i, int k)
{
    const cxd v = (op == OP_N || op == OP_J) ? X[(size_t)i * ld + k] : X[(size_t)k * ld + i];
    return (op == OP_C || op == OP_J) ? mk<double>(v.x, -v.y) : v;
}

constexpr int ZT = 16;  // output tile (ZT x ZT), one element per thread; K staged in ZT chunks

// C_b = alpha op(A_b) op(B_b) + beta C_b for batch entry b = blockIdx.z; A_b = A + offA[b]
// (offA null: offset 0), B and C likewise. M x K times K x N, row-major, FP64 complex.
__global__ void __launch_bounds__(ZT *ZT) zgemm_batched_kernel(int M, int N, int K, cxd alpha, const cxd *A, long long lda,
                                                             int opa, const long long *offA, const cxd *B,
                                                             long long ldb, int opb, const long long *offB, cxd beta,
                                                             cxd *C, long long ldc, const long long *offC)
{
    __shared__ cxd As[ZT][ZT + 1];
    __shared__ cxd Bs[ZT][ZT + 1];
    const int b = blockIdx.z;
    const cxd *Ab = A + (offA ? offA[b] : 0);
    const cxd *Bb = B + (offB ? offB[b] : 0);
    cxd *Cb = C + (offC ? offC[b] : 0);
    const int tx = threadIdx.x % ZT, ty = threadIdx.x / ZT;
    const int i = blockIdx.y * ZT + ty, j = blockIdx.x * ZT + tx;
    cxd acc = mk<double>(0.0, 0.0);
    for (int k0 = 0; k0 < K; k0 += ZT) {
        const int ka = k0 + tx, kb = k0 + ty;
        As[ty][tx] = (i < M && ka < K) ? op_load(Ab, lda, opa, i, ka) : mk<double>(0.0, 0.0);
        Bs[ty][tx] = (kb < K && j < N) ? op_load(Bb, ldb, opb, kb, j) : mk<double>(0.0, 0.0);
        __syncthreads();
#pragma unroll
        for (int q = 0; q < ZT; ++q) cfma(acc, As[ty][q], Bs[q][tx]);
        __syncthreads();
    }
    if (i < M && j < N) {
        cxd out = alpha * acc;
        if (beta.x != 0.0 || beta.y != 0.0) out = out + beta * Cb[(size_t)i * ldc + j];
        Cb[(size_t)i * ldc + j] = out;
    }
}

int zgemm_batched(pg_ctx *ctx, int M, int N, int K, cxd alpha, const cxd *A, long long lda, int opa,
                  const long long *offA, const cxd *B, long long ldb, int opb, const long long *offB, cxd beta, cxd *C,
                  long long ldc, const long long *offC, int batch)
{
    if (M <= 0 || N <= 0 || batch <= 0) return PG_OK;
    if (batch > 65535) return PG_ERR_SHAPE;
    dim3 grid((N + ZT - 1) / ZT, (M + ZT - 1) / ZT, batch);
    zgemm_batched_kernel<<<grid, ZT * ZT, 0, ctx->stream>>>(M, N, K, alpha, A, lda, opa, offA, B, ldb, opb, offB, beta,
                                                            C, ldc, offC);
    ctx->launches++;
    return pg_check_launch(ctx);
}

struct DevBuf {
    void *p = nullptr;
    ~DevBuf() { cudaFree(p); }
};

int check_args(int nang, int N1, int N2, const int *angular, int nidx, const double *V1, int n1, const double *V2,
               int n2)
{
    if (nang < 1 || N1 < 1 || N2 < 1 || nidx < 0 || n1 < 0 || n2 < 0 || (nidx > 0 && !angular)) return PG_ERR_ARG;
    if ((n1 > 0 && !V1) || (n2 > 0 && !V2)) return PG_ERR_ARG;
    for (int q = 0; q < nidx; ++q)
        if (angular[q] < 0 || angular[q] >= nang) return PG_ERR_ARG;
    return PG_OK;
}

// upload V1, V2 and the batch offsets; proj_dev [nidx][n1][n2] = V1^H Psi_a conj(V2)
int project(pg_ctx *ctx, const cxd *psi_w, int N1, int N2, const int *angular, int nidx, const double *V1, int n1,
            const double *V2, int n2, DevBuf &dV1, DevBuf &dV2, DevBuf &dproj, DevBuf &doff)
{
    const size_t s1 = sizeof(cxd) * (size_t)N1 * n1, s2 = sizeof(cxd) * (size_t)N2 * n2;
    const size_t sp = sizeof(cxd) * (size_t)nidx * n1 * n2, st = sizeof(cxd) * (size_t)nidx * N1 * n2;
    PG_CUDA_TRY(cudaMalloc(&dV1.p, s1 + 16));
    PG_CUDA_TRY(cudaMalloc(&dV2.p, s2 + 16));
    PG_CUDA_TRY(cudaMalloc(&dproj.p, sp + st + 16));
    PG_CUDA_TRY(cudaMalloc(&doff.p, sizeof(long long) * 4 * (size_t)nidx + 16));
    PG_CUDA_TRY(cudaMemcpyAsync(dV1.p, V1, s1, cudaMemcpyHostToDevice, ctx->stream));
    PG_CUDA_TRY(cudaMemcpyAsync(dV2.p, V2, s2, cudaMemcpyHostToDevice, ctx->stream));
    // offsets: the psi block, the [N1][n2] intermediate, the [n1][n2] projection, the psi block
    std::vector<long long> off(4 * (size_t)nidx);
    for (int q = 0; q < nidx; ++q) {
        off[q] = (long long)angular[q] * N1 * N2;
        off[nidx + q] = (long long)q * N1 * n2;
        off[2 * nidx + q] = (long long)q * n1 * n2;
        off[3 * nidx + q] = off[q];
    }
    PG_CUDA_TRY(cudaMemcpyAsync(doff.p, off.data(), sizeof(long long) * off.size(), cudaMemcpyHostToDevice, ctx->stream));
    const long long *o = (const long long *)doff.p;
    cxd *proj = (cxd *)dproj.p, *tmp = proj + (size_t)nidx * n1 * n2;
    // tmp_a = Psi_a conj(V2)  [N1 x n2]
    PG_TRY(zgemm_batched(ctx, N1, n2, N2, mk<double>(1.0, 0.0), psi_w, N2, OP_N, o, (const cxd *)dV2.p, n2, OP_J,
                         nullptr, mk<double>(0.0, 0.0), tmp, n2, o + nidx, nidx));
    // proj_a = V1^H tmp_a  [n1 x n2]
    return zgemm_batched(ctx, n1, n2, N1, mk<double>(1.0, 0.0), (const cxd *)dV1.p, n1, OP_C, nullptr, tmp, n2, OP_N,
                         o + nidx, mk<double>(0.0, 0.0), proj, n2, o + 2 * nidx, nidx);
}

}  // namespace

extern "C" int pg_radial_products_project(pg_ctx *ctx, const void *psi_w, int nang, int N1, int N2, const int *angular,
                                          int nidx, const double *V1, int n1, const double *V2, int n2, double *proj)
{
    if (!ctx || !psi_w || (nidx > 0 && n1 > 0 && n2 > 0 && !proj)) return PG_ERR_ARG;
    PG_TRY(check_args(nang, N1, N2, angular, nidx, V1, n1, V2, n2));
    if (nidx == 0 || n1 == 0 || n2 == 0) return PG_OK;
    DevBuf dV1, dV2, dproj, doff;
    PG_TRY(project(ctx, (const cxd *)psi_w, N1, N2, angular, nidx, V1, n1, V2, n2, dV1, dV2, dproj, doff));
    PG_CUDA_TRY(cudaMemcpyAsync(proj, dproj.p, sizeof(cxd) * (size_t)nidx * n1 * n2, cudaMemcpyDeviceToHost,
                                ctx->stream));
    PG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return PG_OK;
}

extern "C" int pg_radial_products_remove(pg_ctx *ctx, const void *psi_w, void *psi, int nang, int N1, int N2,
                                         const int *angular, int nidx, const double *V1, int n1, const double *V2,
                                         int n2)
{
    if (!ctx || !psi_w || !psi) return PG_ERR_ARG;
    PG_TRY(check_args(nang, N1, N2, angular, nidx, V1, n1, V2, n2));
    if (nidx == 0 || n1 == 0 || n2 == 0) return PG_OK;
    DevBuf dV1, dV2, dproj, doff;
    PG_TRY(project(ctx, (const cxd *)psi_w, N1, N2, angular, nidx, V1, n1, V2, n2, dV1, dV2, dproj, doff));
    const long long *o = (const long long *)doff.p;
    cxd *proj = (cxd *)dproj.p, *tmp = proj + (size_t)nidx * n1 * n2;
    // tmp_a = V1 proj_a  [N1 x n2]
    PG_TRY(zgemm_batched(ctx, N1, n2, n1, mk<double>(1.0, 0.0), (const cxd *)dV1.p, n1, OP_N, nullptr, proj, n2, OP_N,
                         o + 2 * nidx, mk<double>(0.0, 0.0), tmp, n2, o + nidx, nidx));
    // psi_a -= tmp_a V2^T  [N1 x N2]
    PG_TRY(zgemm_batched(ctx, N1, N2, n2, mk<double>(-1.0, 0.0), tmp, n2, OP_N, o + nidx, (const cxd *)dV2.p, n2, OP_T,
                         nullptr, mk<double>(1.0, 0.0), (cxd *)psi, N2, o + 3 * nidx, nidx));
    PG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return PG_OK;
}
