// Krylov vector kernels: block inner products (Gram-Schmidt), updates, norms, basis
// combinations, precision conversion.
//
// Reductions: every CTA reduces its contiguous chunk in the element precision (warp
// shuffles, then shared memory), stores one complex128 partial per column, and the last
// CTA to arrive (threadfence + atomic ticket, no waiting) sums the partials in FP64 and
// resets the ticket. The block inner product <V_j, w> for all j replaces the reference's
// conjugate-transpose zgemv + MPI_Allreduce (core/krylov/piram/piram/functors.h:197-240).
#include "pg_internal.cuh"

#include <algorithm>
#include <mutex>

static const int RED_THREADS = 128;
static const int RED_WARPS = RED_THREADS / 32;
static const int RED_ELEMS = 1;  // elements per thread before another CTA is added
static const int RED_CB = 16;    // columns per register block

static inline int red_blocks(pg_ctx *ctx, long long n)
{
    long long per = (long long)RED_THREADS * RED_ELEMS;
    long long nb = (n + per - 1) / per;
    int cap = std::min(ctx->red_max_blocks, 2 * std::max(1, ctx->num_sms));
    return (int)std::max<long long>(1, std::min<long long>(nb, cap));
}

template <typename R> __device__ __forceinline__ R warp_sum(R v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// acc += conj(a) * b
template <typename R> __device__ __forceinline__ void cdot_acc(R &ax, R &ay, cx<R> a, cx<R> b)
{
    ax = fma(a.x, b.x, ax);
    ax = fma(a.y, b.y, ax);
    ay = fma(a.x, b.y, ay);
    ay = fma(-a.y, b.x, ay);
}

// Column sums over this CTA's element range [lo, hi) for columns [jbeg, J]: column j < J is
// <V_j, w>, column J is ||w||^2. Each thread walks its elements once per block of RED_CB
// columns, so RED_CB independent loads are in flight per element. Only the columns in use
// are reduced across the warp (FP64 arithmetic is scarce on this GPU, so no work is spent
// on empty columns); the CTA sum of each column is formed in FP64 and either added to
// atomic_out (FP64 atomics; the consumer clears the buffer after reading it) or stored as
// partial[col][blockIdx] for the last-CTA pass.
template <typename R>
__device__ __forceinline__ void column_sums(const cx<R> *__restrict__ V, long long ldv, int J, int jbeg,
                                            const cx<R> *w, long long lo, long long hi, double (*red)[2 * PG_RED_COLS],
                                            double *partial, double *atomic_out)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int ncols = J + 1;
    for (int j0 = jbeg; j0 < ncols; j0 += RED_CB) {
        R ax[RED_CB], ay[RED_CB];
#pragma unroll
        for (int c = 0; c < RED_CB; ++c) ax[c] = ay[c] = (R)0;
        for (long long i = lo + threadIdx.x; i < hi; i += RED_THREADS) {
            const cx<R> b = w[i];
#pragma unroll
            for (int c = 0; c < RED_CB; ++c) {
                const int j = j0 + c;
                if (j < J) {
                    cdot_acc(ax[c], ay[c], V[(size_t)j * ldv + i], b);
                } else if (j == J) {
                    ax[c] = fma(b.x, b.x, ax[c]);
                    ax[c] = fma(b.y, b.y, ax[c]);
                }
            }
        }
#pragma unroll
        for (int c = 0; c < RED_CB; ++c) {
            const int j = j0 + c;
            if (j < ncols) {  // warp-uniform
                const R sx = warp_sum(ax[c]);
                const R sy = (j < J) ? warp_sum(ay[c]) : (R)0;
                if (lane == 0) {
                    red[warp][2 * j] = (double)sx;
                    red[warp][2 * j + 1] = (double)sy;
                }
            }
        }
    }
    __syncthreads();
    for (int j = jbeg + (int)threadIdx.x; j < ncols; j += RED_THREADS) {
        double sx = 0.0, sy = 0.0;
#pragma unroll
        for (int q = 0; q < RED_WARPS; ++q) {
            sx += red[q][2 * j];
            sy += red[q][2 * j + 1];
        }
        if (atomic_out) {
            atomicAdd(atomic_out + 2 * j, sx);
            if (j < J) atomicAdd(atomic_out + 2 * j + 1, sy);
        } else {
            partial[(size_t)(2 * j) * gridDim.x + blockIdx.x] = sx;
            partial[(size_t)(2 * j + 1) * gridDim.x + blockIdx.x] = sy;
        }
    }
}

__device__ __forceinline__ bool arrive_last(unsigned int *counter)
{
    __shared__ bool is_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int ticket = atomicAdd(counter, 1u);
        is_last = (ticket == gridDim.x - 1);
    }
    __syncthreads();
    return is_last;
}

// Final cross-CTA reduction by the last CTA to arrive: one warp per column, lanes reading
// consecutive CTAs' partials (from L2: other CTAs wrote them), FP64 throughout. Columns
// below jbeg are zero. out[2J+1] = sqrt(out[2J]); the ticket is reset for the next launch.
__device__ void finish_reduction(const double *partial, int J, int jbeg, unsigned int *counter, double *out)
{
    __threadfence();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int ncols = J + 1;
    const int nb = (int)gridDim.x;
    for (int j = warp; j < ncols; j += RED_WARPS) {
        double sx = 0.0, sy = 0.0;
        if (j >= jbeg) {
            const double *px = partial + (size_t)(2 * j) * nb;
            const double *py = partial + (size_t)(2 * j + 1) * nb;
            double ax[4] = {0.0, 0.0, 0.0, 0.0}, ay[4] = {0.0, 0.0, 0.0, 0.0};
            for (int b0 = 0; b0 < nb; b0 += 128) {
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int blk = b0 + 32 * u + lane;
                    if (blk < nb) {
                        ax[u] += __ldcg(px + blk);
                        ay[u] += __ldcg(py + blk);
                    }
                }
            }
            sx = warp_sum((ax[0] + ax[1]) + (ax[2] + ax[3]));
            sy = warp_sum((ay[0] + ay[1]) + (ay[2] + ay[3]));
        }
        if (lane == 0) {
            out[2 * j] = sx;
            out[2 * j + 1] = sy;
            if (j == J) out[2 * J + 1] = sqrt(sx);
        }
    }
    if (threadIdx.x == 0) *counter = 0;
}

// out[2j..2j+1] = <V_j, w> (j < J); out[2J] = ||w||^2, out[2J+1] = ||w||.
// With atomic_out the CTA sums are added to atomic_out (zero on entry; no square root).
template <typename R>
__global__ void __launch_bounds__(RED_THREADS) multidot_kernel(const cx<R> *__restrict__ V, long long ldv, int J,
                                                               const int *__restrict__ Jdev, const cx<R> *__restrict__ w,
                                                               long long n, double *partial, unsigned int *counter,
                                                               double *out, double *atomic_out)
{
    __shared__ double red[RED_WARPS][2 * PG_RED_COLS];
    if (Jdev) J = min(*Jdev + 1, J);  // device count, bounded by the host-checked maximum
    const long long chunk = (n + gridDim.x - 1) / gridDim.x;
    const long long lo = (long long)blockIdx.x * chunk;
    const long long hi = min(n, lo + chunk);
    column_sums<R>(V, ldv, J, 0, w, lo, hi, red, partial, atomic_out);
    if (atomic_out) return;
    if (arrive_last(counter)) finish_reduction(partial, J, 0, counter, out);
}

// w -= sum_j V_j h_j (h complex128 on device); then the dots <V_j, w> (j < J, when
// want_dots) and ||w||^2 into out exactly as multidot_kernel.
template <typename R>
__global__ void __launch_bounds__(RED_THREADS) gs_update_kernel(const cx<R> *__restrict__ V, long long ldv, int J,
                                                                const int *__restrict__ Jdev,
                                                                const double *__restrict__ h, cx<R> *__restrict__ w,
                                                                long long n, int want_dots, double *partial,
                                                                unsigned int *counter, double *out, double *atomic_out)
{
    __shared__ double red[RED_WARPS][2 * PG_RED_COLS];
    __shared__ cx<R> hs[PG_RED_COLS];
    if (Jdev) J = min(*Jdev + 1, J);  // device count, bounded by the host-checked maximum
    for (int j = threadIdx.x; j < J; j += blockDim.x) hs[j] = mk<R>((R)h[2 * j], (R)h[2 * j + 1]);
    __syncthreads();
    const long long chunk = (n + gridDim.x - 1) / gridDim.x;
    const long long lo = (long long)blockIdx.x * chunk;
    const long long hi = min(n, lo + chunk);
    for (long long i = lo + threadIdx.x; i < hi; i += RED_THREADS) {
        cx<R> acc = w[i];
        for (int j0 = 0; j0 < J; j0 += RED_CB) {
            cx<R> v[RED_CB];
#pragma unroll
            for (int c = 0; c < RED_CB; ++c)
                v[c] = (j0 + c < J) ? V[(size_t)(j0 + c) * ldv + i] : mk<R>((R)0, (R)0);
#pragma unroll
            for (int c = 0; c < RED_CB; ++c)
                if (j0 + c < J) {
                    const cx<R> hc = hs[j0 + c];
                    acc.x = fma(-v[c].x, hc.x, acc.x);
                    acc.x = fma(v[c].y, hc.y, acc.x);
                    acc.y = fma(-v[c].x, hc.y, acc.y);
                    acc.y = fma(-v[c].y, hc.x, acc.y);
                }
        }
        w[i] = acc;  // read back below by this same thread only
    }
    const int jbeg = want_dots ? 0 : J;
    column_sums<R>(V, ldv, J, jbeg, w, lo, hi, red, partial, atomic_out);
    if (atomic_out) return;
    if (arrive_last(counter)) finish_reduction(partial, J, jbeg, counter, out);
}

template <typename R>
int pg_multidot(pg_ctx *ctx, const cx<R> *V, long long ldv, int J, const cx<R> *w, long long n, double *out_dev,
                const int *Jdev, int atomic)
{
    if (J + 1 > ctx->red_max_cols) return PG_ERR_ARG;
    const int nb = red_blocks(ctx, n);
    multidot_kernel<R><<<nb, RED_THREADS, 0, ctx->stream>>>(V, ldv, J, Jdev, w, n, ctx->red_partial, ctx->red_counter,
                                                            out_dev, atomic ? out_dev : nullptr);
    ctx->launches++;
    return pg_check_launch(ctx);
}

template <typename R>
int pg_gs_update(pg_ctx *ctx, const cx<R> *V, long long ldv, int J, const double *h_dev, cx<R> *w, long long n,
                 int want_dots, double *out_dev, const int *Jdev, int atomic)
{
    if (J + 1 > ctx->red_max_cols) return PG_ERR_ARG;
    const int nb = red_blocks(ctx, n);
    gs_update_kernel<R><<<nb, RED_THREADS, 0, ctx->stream>>>(V, ldv, J, Jdev, h_dev, w, n, want_dots, ctx->red_partial,
                                                            ctx->red_counter, out_dev, atomic ? out_dev : nullptr);
    ctx->launches++;
    return pg_check_launch(ctx);
}

template int pg_multidot<double>(pg_ctx *, const cxd *, long long, int, const cxd *, long long, double *, const int *,
                                 int);
template int pg_multidot<float>(pg_ctx *, const cxf *, long long, int, const cxf *, long long, double *, const int *,
                                int);
template int pg_gs_update<double>(pg_ctx *, const cxd *, long long, int, const double *, cxd *, long long, int, double *,
                                  const int *, int);
template int pg_gs_update<float>(pg_ctx *, const cxf *, long long, int, const double *, cxf *, long long, int, double *,
                                 const int *, int);

// ------------------------------------------------------------------------------------
// elementwise helpers
// ------------------------------------------------------------------------------------
// dst (Rd) = src (Rs) * (1/scale_dev[0]) (or * mul when scale_dev is null); dst2 gets a copy
template <typename Rd, typename Rs>
__global__ void scale_copy_kernel(const cx<Rs> *__restrict__ src, cx<Rd> *__restrict__ dst, cx<Rd> *__restrict__ dst2,
                                  long long n, const double *__restrict__ inv_scale_dev, double mul)
{
    double s = mul;
    if (inv_scale_dev) {
        const double b = inv_scale_dev[0];
        s = b > 0.0 ? 1.0 / b : 0.0;  // a zero norm gives a zero vector, never inf/NaN
    }
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const cx<Rs> a = src[i];
        const cx<Rd> v = mk<Rd>((Rd)((double)a.x * s), (Rd)((double)a.y * s));
        dst[i] = v;
        if (dst2) dst2[i] = v;
    }
}

template <typename Rd, typename Rs>
int pg_scale_copy(pg_ctx *ctx, const cx<Rs> *src, cx<Rd> *dst, cx<Rd> *dst2, long long n, const double *inv_scale_dev,
                  double mul)
{
    int nb = (int)std::min<long long>((n + 255) / 256, 4LL * std::max(1, ctx->num_sms));
    if (nb < 1) nb = 1;
    scale_copy_kernel<Rd, Rs><<<nb, 256, 0, ctx->stream>>>(src, dst, dst2, n, inv_scale_dev, mul);
    ctx->launches++;
    return pg_check_launch(ctx);
}
template int pg_scale_copy<double, double>(pg_ctx *, const cxd *, cxd *, cxd *, long long, const double *, double);
template int pg_scale_copy<float, double>(pg_ctx *, const cxd *, cxf *, cxf *, long long, const double *, double);
template int pg_scale_copy<double, float>(pg_ctx *, const cxf *, cxd *, cxd *, long long, const double *, double);
template int pg_scale_copy<float, float>(pg_ctx *, const cxf *, cxf *, cxf *, long long, const double *, double);

// out (complex128) = alpha * sum_{j<k} V_j c_j (+ beta_acc * out); c complex128 on device.
template <typename R>
__global__ void combine_kernel(const cx<R> *__restrict__ V, long long ldv, int k, const double *__restrict__ c,
                               double alpha, cxd *__restrict__ out, long long n, int accumulate)
{
    __shared__ cxd cs[PG_RED_COLS];
    for (int j = threadIdx.x; j < k; j += blockDim.x) cs[j] = mk<double>(c[2 * j], c[2 * j + 1]);
    __syncthreads();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double ax = 0, ay = 0;
        for (int j = 0; j < k; ++j) {
            const cx<R> v = V[(size_t)j * ldv + i];
            const cxd q = cs[j];
            ax = fma((double)v.x, q.x, ax); ax = fma(-(double)v.y, q.y, ax);
            ay = fma((double)v.x, q.y, ay); ay = fma((double)v.y, q.x, ay);
        }
        cxd o = mk<double>(alpha * ax, alpha * ay);
        if (accumulate) o = o + out[i];
        out[i] = o;
    }
}

template <typename R>
int pg_combine(pg_ctx *ctx, const cx<R> *V, long long ldv, int k, const double *c_dev, double alpha, cxd *out,
               long long n, int accumulate)
{
    if (k > PG_RED_COLS) return PG_ERR_ARG;
    int nb = (int)std::min<long long>((n + 255) / 256, 4LL * std::max(1, ctx->num_sms));
    if (nb < 1) nb = 1;
    combine_kernel<R><<<nb, 256, 0, ctx->stream>>>(V, ldv, k, c_dev, alpha, out, n, accumulate);
    ctx->launches++;
    return pg_check_launch(ctx);
}
template int pg_combine<double>(pg_ctx *, const cxd *, long long, int, const double *, double, cxd *, long long, int);
template int pg_combine<float>(pg_ctx *, const cxf *, long long, int, const double *, double, cxd *, long long, int);

// y = a*x + y with complex a (host value), complex128 vectors
__global__ void axpy_kernel(cxd a, const cxd *__restrict__ x, cxd *__restrict__ y, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        cfma(y[i], a, x[i]);
}
int pg_axpy(pg_ctx *ctx, cxd a, const cxd *x, cxd *y, long long n)
{
    int nb = (int)std::min<long long>((n + 255) / 256, 4LL * std::max(1, ctx->num_sms));
    if (nb < 1) nb = 1;
    axpy_kernel<<<nb, 256, 0, ctx->stream>>>(a, x, y, n);
    ctx->launches++;
    return pg_check_launch(ctx);
}

// ------------------------------------------------------------------------------------
// ABI
// ------------------------------------------------------------------------------------
extern "C" int pg_vec_dot(pg_ctx *ctx, int precision, const void *x, const void *y, long long n, double *out)
{
    if (!ctx || !x || !y || !out || n < 0) return PG_ERR_ARG;
    int st;
    if (precision == PG_FP64) st = pg_multidot<double>(ctx, (const cxd *)x, 0, 1, (const cxd *)y, n, ctx->red_out);
    else if (precision == PG_FP32) st = pg_multidot<float>(ctx, (const cxf *)x, 0, 1, (const cxf *)y, n, ctx->red_out);
    else return PG_ERR_ARG;
    if (st != PG_OK) return st;
    PG_CUDA_TRY(cudaMemcpyAsync(ctx->h_pinned, ctx->red_out, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    PG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    out[0] = ctx->h_pinned[0];
    out[1] = ctx->h_pinned[1];
    return PG_OK;
}

extern "C" int pg_vec_convert(pg_ctx *ctx, int src_precision, const void *x, int dst_precision, void *y, long long n)
{
    if (!ctx || !x || !y || n < 0) return PG_ERR_ARG;
    if (src_precision == PG_FP64 && dst_precision == PG_FP32)
        return pg_scale_copy<float, double>(ctx, (const cxd *)x, (cxf *)y, nullptr, n, nullptr, 1.0);
    if (src_precision == PG_FP32 && dst_precision == PG_FP64)
        return pg_scale_copy<double, float>(ctx, (const cxf *)x, (cxd *)y, nullptr, n, nullptr, 1.0);
    if (src_precision == PG_FP64 && dst_precision == PG_FP64)
        return pg_scale_copy<double, double>(ctx, (const cxd *)x, (cxd *)y, nullptr, n, nullptr, 1.0);
    if (src_precision == PG_FP32 && dst_precision == PG_FP32)
        return pg_scale_copy<float, float>(ctx, (const cxf *)x, (cxf *)y, nullptr, n, nullptr, 1.0);
    return PG_ERR_ARG;
}

extern "C" int pg_vec_combine(pg_ctx *ctx, void *V, long long n, int m, const double *Q, int k)
{
    // V[:k] <- V[:m] Q  (column q of Q gives new vector q); done through a temporary
    if (!ctx || !V || !Q || m <= 0 || k <= 0 || k > m || m > PG_RED_COLS) return PG_ERR_ARG;
    cxd *tmp = nullptr;
    double *dQ = nullptr;
    PG_CUDA_TRY(cudaMalloc(&tmp, sizeof(cxd) * (size_t)n * k));
    PG_CUDA_TRY(cudaMalloc(&dQ, sizeof(double) * 2 * (size_t)m * k));
    std::vector<double> colmaj(2 * (size_t)m * k);
    for (int q = 0; q < k; ++q)
        for (int j = 0; j < m; ++j) {
            colmaj[2 * ((size_t)q * m + j)] = Q[2 * ((size_t)j * k + q)];
            colmaj[2 * ((size_t)q * m + j) + 1] = Q[2 * ((size_t)j * k + q) + 1];
        }
    PG_CUDA_TRY(cudaMemcpyAsync(dQ, colmaj.data(), colmaj.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    for (int q = 0; q < k; ++q)
        PG_TRY(pg_combine<double>(ctx, (const cxd *)V, n, m, dQ + 2 * (size_t)q * m, 1.0, tmp + (size_t)q * n, n, 0));
    PG_CUDA_TRY(cudaMemcpyAsync(V, tmp, sizeof(cxd) * (size_t)n * k, cudaMemcpyDeviceToDevice, ctx->stream));
    PG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    cudaFree(tmp);
    cudaFree(dQ);
    return PG_OK;
}

// ------------------------------------------------------------------------------------
// allocation-free block inner product
// ------------------------------------------------------------------------------------
// Same multidot kernel, but its per-CTA partials, arrival ticket and nothing else live in
// file-scope device arrays instead of memory from cudaMalloc. Every GPU that loads this
// library holds these ~320 KB until the process exits. Host code cannot use the arrays'
// names as device addresses, so their addresses are looked up once per device with
// cudaGetSymbolAddress (on the first call on that device) and passed to the kernel.
static const int NOALLOC_MAX_VECTORS = 64;
static const int NOALLOC_BLOCKS = PG_RED_BLOCKS;
static const int NOALLOC_MAX_DEVICES = 64;

static __device__ __align__(256) double g_noalloc_partial[2 * NOALLOC_BLOCKS * (NOALLOC_MAX_VECTORS + 1)];
static __device__ __align__(256) unsigned int g_noalloc_ticket[64];

namespace {
struct NoallocDevice {
    bool ready = false;
    double *partial = nullptr;
    unsigned int *ticket = nullptr;
    int max_blocks = 1;
};
NoallocDevice g_noalloc_dev[NOALLOC_MAX_DEVICES];
std::mutex g_noalloc_mutex;
}  // namespace

// First call on a device: resolve the scratch addresses with that device current.
static int noalloc_setup(int device, NoallocDevice **out)
{
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    NoallocDevice &d = g_noalloc_dev[device];
    if (!d.ready) {
        PG_CUDA_TRY(cudaGetSymbolAddress((void **)&d.partial, g_noalloc_partial));
        PG_CUDA_TRY(cudaGetSymbolAddress((void **)&d.ticket, g_noalloc_ticket));
        int sms = 0;
        PG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
        d.max_blocks = std::max(1, std::min(NOALLOC_BLOCKS, 2 * std::max(1, sms)));
        d.ready = true;
    }
    *out = &d;
    return PG_OK;
}

extern "C" int pg_vec_multidot_noalloc(int precision, const void *V, long long ldv, int J, const void *w, long long n,
                                       double *out, void *stream)
{
    if (!w || !out || n < 0 || J < 0 || (J > 0 && !V)) return PG_ERR_ARG;
    if (J > NOALLOC_MAX_VECTORS) return PG_ERR_ARG;  // more columns than the static scratch holds
    if (J > 1 && ldv < n) return PG_ERR_ARG;
    if (precision != PG_FP64 && precision != PG_FP32) return PG_ERR_ARG;
    int device = 0;
    PG_CUDA_TRY(cudaGetDevice(&device));
    if (device < 0 || device >= NOALLOC_MAX_DEVICES) return PG_ERR_ARG;
    NoallocDevice *d = nullptr;
    PG_TRY(noalloc_setup(device, &d));
    cudaStream_t s = (cudaStream_t)stream;
    // the ticket must start at zero; the last CTA leaves it at zero, this clears any leftover
    PG_CUDA_TRY(cudaMemsetAsync(d->ticket, 0, sizeof(unsigned int), s));
    const long long per = (long long)RED_THREADS * RED_ELEMS;
    const int nb = (int)std::max<long long>(1, std::min<long long>((n + per - 1) / per, d->max_blocks));
    if (precision == PG_FP64)
        multidot_kernel<double><<<nb, RED_THREADS, 0, s>>>((const cxd *)V, ldv, J, nullptr, (const cxd *)w, n,
                                                           d->partial, d->ticket, out, nullptr);
    else
        multidot_kernel<float><<<nb, RED_THREADS, 0, s>>>((const cxf *)V, ldv, J, nullptr, (const cxf *)w, n,
                                                          d->partial, d->ticket, out, nullptr);
    PG_CUDA_TRY(cudaGetLastError());
    return PG_OK;
}

// ------------------------------------------------------------------------------------
// swap of the last two ranks: y[a][j][i] = x[a][i][j] (x: [n0][n1][n2])
// ------------------------------------------------------------------------------------
// Two-electron wavefunctions [Nang][N][N] keep their fibres along the last rank; operations
// along the middle rank (the first electron's overlap) run on the swapped copy. 32x32 tiles
// through shared memory, both global sides coalesced.
template <typename R>
__global__ void swap_last2_kernel(const cx<R> *__restrict__ x, cx<R> *__restrict__ y, int n1, int n2)
{
    __shared__ cx<R> tile[32][33];
    const int a = blockIdx.z;
    const int i0 = blockIdx.y * 32, j0 = blockIdx.x * 32;
    const cx<R> *xa = x + (size_t)a * n1 * n2;
    cx<R> *ya = y + (size_t)a * n1 * n2;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int i = i0 + r, j = j0 + threadIdx.x;
        if (i < n1 && j < n2) tile[r][threadIdx.x] = xa[(size_t)i * n2 + j];
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int j = j0 + r, i = i0 + threadIdx.x;
        if (i < n1 && j < n2) ya[(size_t)j * n1 + i] = tile[threadIdx.x][r];
    }
}

extern "C" int pg_vec_swap_last2(pg_ctx *ctx, int precision, const void *x, void *y, int n0, int n1, int n2)
{
    if (!ctx || !x || !y || n0 < 0 || n1 < 0 || n2 < 0 || x == y) return PG_ERR_ARG;
    if (precision != PG_FP64 && precision != PG_FP32) return PG_ERR_ARG;
    return pg_swap_last2_dev(ctx, precision, x, y, n0, n1, n2);
}

int pg_swap_last2_dev(pg_ctx *ctx, int precision, const void *x, void *y, int n0, int n1, int n2)
{
    if (n0 == 0 || n1 == 0 || n2 == 0) return PG_OK;
    if (n0 > 65535) return PG_ERR_SHAPE;
    dim3 grid((n2 + 31) / 32, (n1 + 31) / 32, n0), block(32, 8);
    if (precision == PG_FP64)
        swap_last2_kernel<double><<<grid, block, 0, ctx->stream>>>((const cxd *)x, (cxd *)y, n1, n2);
    else
        swap_last2_kernel<float><<<grid, block, 0, ctx->stream>>>((const cxf *)x, (cxf *)y, n1, n2);
    ctx->launches++;
    return pg_check_launch(ctx);
}
