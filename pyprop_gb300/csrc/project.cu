// Projection of functions on the quadrature grid into B-spline band rows: the step of the
// tensor-potential generator that represents a potential in the B-spline basis
// (pyprop/tensorpotential/TensorPotentialGenerator.py:80-274 through
// core/tensorpotential/basis_bspline.h:11-47 and BSplineGlobalOverlapIntegral,
// core/transform/bspline/bspline.cpp:373-466), without derivatives:
//     M[i][j] = sum_m sum_p w[m][p] B_i(x_mp) B_j(x_mp) f(x_mp),   |i - j| < k,
// stored as band rows out[i][(k - 1) + (j - i)]. Two calls make a two-electron radial factor
// f(r1, r2): along r2 for every r1 quadrature point, then along r1 for every (i2, j2) column of
// that result. Interval m carries the k splines first[m] + a (a < k); splines outside
// [0, N) have zero values in the tables. One CTA per batch row: the row's function values
// staged in shared memory, each (interval, pair a <= b) integrated by one thread and added
// to the row's band in shared memory (both (i, j) and (j, i): the matrix is symmetric).
#include "pg_internal.cuh"

#include <mutex>

namespace {

constexpr int PJ_THREADS = 256;

__global__ void __launch_bounds__(PJ_THREADS) band_project_kernel(
    const double *__restrict__ F, int bdiv, long long in_bstride, long long in_qstride, int nint, int k, int q,
    const int *__restrict__ first, const double *__restrict__ B, const double *__restrict__ w, int N,
    double *__restrict__ out, long long ob1, long long ob2, long long oi, long long od)
{
    extern __shared__ double pj_smem[];
    const int nq = nint * q, bw = 2 * k - 1;
    double *f = pj_smem;          // [nq] this row's function values times the weights
    double *acc = f + nq;         // [N][2k-1] the row's band
    const long long b = blockIdx.x;
    const double *Fb = F + b * in_bstride;
    for (int t = threadIdx.x; t < nq; t += PJ_THREADS) f[t] = Fb[(long long)t * in_qstride] * __ldg(w + t);
    for (int t = threadIdx.x; t < N * bw; t += PJ_THREADS) acc[t] = 0.0;
    __syncthreads();
    const int npair = k * (k + 1) / 2;
    for (int t = threadIdx.x; t < nint * npair; t += PJ_THREADS) {
        const int m = t / npair;
        int pr = t - m * npair, a = 0;
        while (pr >= k - a) {  // pair index -> (a, b), a <= b
            pr -= k - a;
            ++a;
        }
        const int bb = a + pr;
        const int i = __ldg(first + m) + a, j = __ldg(first + m) + bb;
        if (i < 0 || j >= N) continue;
        const double *Ba = B + ((size_t)m * k + a) * q, *Bb = B + ((size_t)m * k + bb) * q;
        const double *fm = f + (size_t)m * q;
        double s = 0.0;
        for (int p = 0; p < q; ++p) s = fma(__ldg(Ba + p) * __ldg(Bb + p), fm[p], s);
        atomicAdd(acc + (size_t)i * bw + (k - 1) + (j - i), s);
        if (bb != a) atomicAdd(acc + (size_t)j * bw + (k - 1) + (i - j), s);
    }
    __syncthreads();
    double *ob = out + (b / bdiv) * ob1 + (b % bdiv) * ob2;
    for (int t = threadIdx.x; t < N * bw; t += PJ_THREADS) {
        const int i = t / bw, d = t - i * bw;
        ob[i * oi + d * od] = acc[t];
    }
}

}  // namespace

extern "C" int pg_bspline_band_project(pg_ctx *ctx, const double *F, long long nbatch, int bdiv, long long in_bstride,
                                       long long in_qstride, int nint, int k, int q, const int *first,
                                       const double *B, const double *w, int N, double *out, long long ob1,
                                       long long ob2, long long oi, long long od)
{
    if (!ctx || !F || !first || !B || !w || !out || nbatch < 0 || bdiv < 1 || nint < 1 || k < 1 || k > 16 || q < 1 ||
        N < 1)
        return PG_ERR_ARG;
    if (nbatch == 0) return PG_OK;
    if (nbatch > 0x7fffffffLL) return PG_ERR_SHAPE;
    const size_t smem = sizeof(double) * ((size_t)nint * q + (size_t)N * (2 * k - 1));
    int optin = 0;
    PG_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
    if (smem > (size_t)optin) return PG_ERR_SHAPE;  // quadrature grid or basis too large for one row in shared memory
    if (smem > 48 * 1024) {  // the attribute only ever grows: another caller may rely on a larger one
        static std::mutex mu;
        static size_t configured = 0;
        std::lock_guard<std::mutex> lock(mu);
        if (configured < smem) {
            PG_CUDA_TRY(cudaFuncSetAttribute(band_project_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            configured = smem;
        }
    }
    band_project_kernel<<<(unsigned)nbatch, PJ_THREADS, smem, ctx->stream>>>(F, bdiv, in_bstride, in_qstride, nint, k, q,
                                                                            first, B, w, N, out, ob1, ob2, oi, od);
    ctx->launches++;
    return pg_check_launch(ctx);
}
