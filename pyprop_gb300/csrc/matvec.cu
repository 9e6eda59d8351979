// Tensor-potential matvec on sm_103a.
//
// Two families:
//  * reference-layout kernels (pg_tensor_multiply_*): read the potential exactly as the
//    reference stores it ([pairs][N*(2k+1)], BandNH slot j*(2k+1) + (k+i-j)) and do
//    dest += scaling * V * source, the contract of the generated Fortran
//    TensorPotentialMultiply_{Diag,Simp,Ident}_BandNH (tensorpotentialmultiply_generator.py
//    :302-462 storage snippets, :622-762 BandNH with zgbmv);
//  * the fused operator (pg_op_*): all consolidated terms of H in one launch, bands stored
//    diagonal-major [band][d][i] so that consecutive threads (radial rows i) read
//    consecutive addresses for every diagonal d, complex64 or complex128.
#include "pg_internal.cuh"

#include <algorithm>
#include <cstring>
#include <numeric>

// ------------------------------------------------------------------------------------
// reference-layout kernels (complex128)
// ------------------------------------------------------------------------------------
// mode 0: Diag (pairs (l,l), potential row l), 1: Simp (pair list), 2: Ident (one band)
__global__ void ref_bandnh_kernel(int mode, const cxd *__restrict__ pot, int npairs, int potStride,
                                  double scaling, const cxd *__restrict__ src, cxd *__restrict__ dst,
                                  int nrows, int N, int kb, const int *__restrict__ pairs)
{
    const int r = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N || r >= nrows) return;
    const int b = 2 * kb + 1;
    cxd acc = mk<double>(0.0, 0.0);
    auto band_row = [&](const cxd *V, const cxd *x) {
        cxd t = mk<double>(0.0, 0.0);
        for (int d = 0; d < b; ++d) {
            const int j = i + d - kb;
            if (j >= 0 && j < N) cfma(t, V[(size_t)j * b + (2 * kb - d)], x[j]);
        }
        return t;
    };
    if (mode == 0) {
        acc = band_row(pot + (size_t)r * potStride, src + (size_t)r * N);
    } else if (mode == 2) {
        acc = band_row(pot, src + (size_t)r * N);
    } else {
        for (int p = 0; p < npairs; ++p) {
            if (pairs[2 * p] != r) continue;
            const int c = pairs[2 * p + 1];
            if (c < 0 || c >= nrows) continue;  // pair lists come from device memory: never index past psi
            acc = acc + band_row(pot + (size_t)p * potStride, src + (size_t)c * N);
        }
    }
    cxd o = dst[(size_t)r * N + i];
    o.x = fma(scaling, acc.x, o.x);
    o.y = fma(scaling, acc.y, o.y);
    dst[(size_t)r * N + i] = o;
}

static int ref_bandnh_launch(int mode, const double *potential, int e0, int e1, double scaling,
                             const double *source, int s0, int s1, double *dest, int d0, int d1,
                             const int *pairs, int p0, int p1, int bandCount, void *stream)
{
    if (!potential || !source || !dest || bandCount < 0) return PG_ERR_ARG;
    const int b = 2 * bandCount + 1;
    if (s0 != d0 || s1 != d1 || s0 <= 0 || s1 <= 0) return PG_ERR_SHAPE;
    if (e1 != s1 * b) return PG_ERR_SHAPE;
    if (mode == 0 && e0 != s0) return PG_ERR_SHAPE;
    if (mode == 2 && e0 != 1) return PG_ERR_SHAPE;
    if (mode == 1) {
        if (!pairs || p1 != 2 || p0 != e0) return PG_ERR_SHAPE;
    }
    dim3 block(128);
    dim3 grid((s1 + 127) / 128, s0);
    ref_bandnh_kernel<<<grid, block, 0, (cudaStream_t)stream>>>(
        mode, (const cxd *)potential, e0, e1, scaling, (const cxd *)source, (cxd *)dest, s0, s1, bandCount, pairs);
    PG_CUDA_TRY(cudaGetLastError());
    return PG_OK;
}

extern "C" int pg_tensor_multiply_diag_bandnh(const double *potential, int potExtent0, int potExtent1,
                                              double scaling, const double *source, int srcExtent0,
                                              int srcExtent1, double *dest, int dstExtent0, int dstExtent1,
                                              int bandCount, void *stream)
{
    return ref_bandnh_launch(0, potential, potExtent0, potExtent1, scaling, source, srcExtent0, srcExtent1, dest,
                             dstExtent0, dstExtent1, nullptr, 0, 0, bandCount, stream);
}

extern "C" int pg_tensor_multiply_simp_bandnh(const double *potential, int potExtent0, int potExtent1,
                                              double scaling, const double *source, int srcExtent0,
                                              int srcExtent1, double *dest, int dstExtent0, int dstExtent1,
                                              const int *pair0, int pair0Extent0, int pair0Extent1, int bandCount,
                                              void *stream)
{
    return ref_bandnh_launch(1, potential, potExtent0, potExtent1, scaling, source, srcExtent0, srcExtent1, dest,
                             dstExtent0, dstExtent1, pair0, pair0Extent0, pair0Extent1, bandCount, stream);
}

extern "C" int pg_tensor_multiply_ident_bandnh(const double *potential, int potExtent0, int potExtent1,
                                               double scaling, const double *source, int srcExtent0,
                                               int srcExtent1, double *dest, int dstExtent0, int dstExtent1,
                                               int bandCount, void *stream)
{
    return ref_bandnh_launch(2, potential, potExtent0, potExtent1, scaling, source, srcExtent0, srcExtent1, dest,
                             dstExtent0, dstExtent1, nullptr, 0, 0, bandCount, stream);
}

// ------------------------------------------------------------------------------------
// fused operator
// ------------------------------------------------------------------------------------
// One CTA covers TILE radial rows of one angular row r. For every entry (col, band, slot)
// of row r: t = sum_d band[d][i] * src[col][i+d-kb], acc += scale[slot] * t.
// The scale is applied per entry in the compute precision.
template <typename R, int KB>
__global__ void __launch_bounds__(128) op_matvec_kernel(OpDev op, pg_scales scales, const cxd *__restrict__ scales_dev,
                                                        const cx<R> *__restrict__ src, cx<R> *__restrict__ dst,
                                                        int accumulate, const double *__restrict__ src_inv_scale,
                                                        cx<R> *__restrict__ src_copy_out)
{
    const int r = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int N = op.N;
    if (i >= N) return;
    const int kb = (KB >= 0) ? KB : op.kb;
    const int b = 2 * kb + 1;
    const cx<R> *bands = (const cx<R> *)op.bands;
    R sc = (R)1;
    if (src_inv_scale) sc = (R)(1.0 / *src_inv_scale);
    cx<R> acc = mk<R>((R)0, (R)0);
    const int e_begin = op.row_ptr[r], e_end = op.row_ptr[r + 1];
    for (int e = e_begin; e < e_end; ++e) {
        const int col = op.ent_col[e];
        const cx<R> *__restrict__ V = bands + (size_t)op.ent_band[e] * b * op.ld;
        const cx<R> *__restrict__ x = src + (size_t)col * N;
        cx<R> t = mk<R>((R)0, (R)0);
        if (KB >= 0) {
#pragma unroll
            for (int d = 0; d < 2 * KB + 1; ++d) {
                const int j = i + d - KB;
                if (j >= 0 && j < N) cfma(t, V[(size_t)d * op.ld + i], x[j]);
            }
        } else {
            for (int d = 0; d < b; ++d) {
                const int j = i + d - kb;
                if (j >= 0 && j < N) cfma(t, V[(size_t)d * op.ld + i], x[j]);
            }
        }
        const int slot = op.ent_slot[e];
        const cx<R> s = scales_dev ? cvt<R>(scales_dev[slot]) : cvt<R>(scales.s[slot]);
        cfma(acc, s, t);
    }
    const size_t o = (size_t)r * N + i;
    if (src_inv_scale) {
        acc = sc * acc;
        if (src_copy_out) src_copy_out[o] = sc * src[o];
    }
    if (accumulate) acc = acc + dst[o];
    dst[o] = acc;
}

// ------------------------------------------------------------------------------------
// fused operator, bulk-copy staged variant
// ------------------------------------------------------------------------------------
// One CTA = BT radial rows of one angular row. Thread 0 issues one cp.async.bulk per
// (entry, diagonal) band slab [d][i0 .. i0+BT) into shared memory, all completing on one
// mbarrier (expected bytes), while all threads load the source slabs x[col][i0-kb .. i0+BT+kb)
// with ordinary coalesced loads. The whole CTA's operator tile is in flight at once, so the
// kernel is bound by HBM rather than by load latency. Entries of a row are processed in
// groups of BMAXE. Requires band leading dimension ld (>= N) with 16-byte aligned slabs.
static const int BT = 64;
static const int BMAXE = 4;

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity)
{
    unsigned ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// bounded wait: gives up after `limit` polls and reports through *err
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, unsigned parity, int *err)
{
    for (long long it = 0; it < (1LL << 26); ++it)
        if (mbar_try_wait(bar, parity)) return true;
    if (err) atomicExch(err, 1);
    return false;
}

template <typename R, int KB>
__global__ void __launch_bounds__(BT) op_matvec_bulk_kernel(OpDev op, pg_scales scales, const cxd *__restrict__ scales_dev,
                                                            const cx<R> *__restrict__ src, cx<R> *__restrict__ dst,
                                                            int accumulate, int *err)
{
    constexpr int B = 2 * KB + 1;
    extern __shared__ __align__(128) unsigned char mv_smem[];
    unsigned long long *bar = (unsigned long long *)mv_smem;
    cx<R> *bs = (cx<R> *)(mv_smem + 128);            // [BMAXE][B][BT]
    cx<R> *xs = bs + (size_t)BMAXE * B * BT;          // [BMAXE][BT + 2KB]
    const int r = blockIdx.y;
    const int i0 = blockIdx.x * BT;
    const int t = threadIdx.x;
    const int N = op.N;
    const int ld = op.ld;
    const int cnt = min(BT, N - i0);
    const unsigned slab_bytes = (unsigned)(((size_t)cnt * sizeof(cx<R>) + 15) & ~(size_t)15);
    const cx<R> *bands = (const cx<R> *)op.bands;
    if (t == 0) {
        mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    cx<R> acc = mk<R>((R)0, (R)0);
    const int e_begin = op.row_ptr[r], e_end = op.row_ptr[r + 1];
    unsigned phase = 0;
    for (int e0 = e_begin; e0 < e_end; e0 += BMAXE) {
        const int ne = min(BMAXE, e_end - e0);
        if (t == 0) {
            mbar_arrive_expect_tx(bar, slab_bytes * (unsigned)(ne * B));
            for (int q = 0; q < ne; ++q) {
                const cx<R> *V = bands + (size_t)op.ent_band[e0 + q] * B * ld + i0;
                for (int d = 0; d < B; ++d)
                    bulk_g2s(bs + ((size_t)q * B + d) * BT, V + (size_t)d * ld, slab_bytes, bar);
            }
        }
        for (int q = 0; q < ne; ++q) {
            const cx<R> *x = src + (size_t)op.ent_col[e0 + q] * N;
            for (int u = t; u < BT + 2 * KB; u += BT) {
                const int j = i0 - KB + u;
                xs[q * (BT + 2 * KB) + u] = (j >= 0 && j < N) ? x[j] : mk<R>((R)0, (R)0);
            }
        }
        __syncthreads();
        const bool ok = mbar_wait_bounded(bar, phase, err);
        // CTA-uniform decision: a thread whose wait ran out waits once more (bounded) for the
        // copies still in flight, then the whole CTA leaves without computing
        if (__syncthreads_or(ok ? 0 : 1)) {
            if (!ok) mbar_wait_bounded(bar, phase, err);
            return;
        }
        phase ^= 1u;
        if (t < cnt) {
            for (int q = 0; q < ne; ++q) {
                const cx<R> *Vb = bs + (size_t)q * B * BT;
                const cx<R> *xb = xs + q * (BT + 2 * KB) + t;
                cx<R> tq = mk<R>((R)0, (R)0);
#pragma unroll
                for (int d = 0; d < B; ++d) cfma(tq, Vb[d * BT + t], xb[d]);
                const int slot = op.ent_slot[e0 + q];
                const cx<R> sc = scales_dev ? cvt<R>(scales_dev[slot]) : cvt<R>(scales.s[slot]);
                cfma(acc, sc, tq);
            }
        }
        __syncthreads();  // shared slabs are refilled by the next group
    }
    if (t < cnt) {
        const size_t o = (size_t)r * N + i0 + t;
        if (accumulate) acc = acc + dst[o];
        dst[o] = acc;
    }
}

template <typename R, int KB>
static int launch_bulk(pg_op *op, const pg_scales &scales, const cxd *scales_dev, const void *src, void *dst,
                       int accumulate)
{
    constexpr int B = 2 * KB + 1;
    const size_t smem = 128 + sizeof(cx<R>) * ((size_t)BMAXE * B * BT + (size_t)BMAXE * (BT + 2 * KB));
    static bool configured[2] = {false, false};
    const int which = sizeof(R) == 8 ? 1 : 0;
    if (!configured[which]) {
        PG_CUDA_TRY(cudaFuncSetAttribute(op_matvec_bulk_kernel<R, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem));
        configured[which] = true;
    }
    dim3 grid((op->N + BT - 1) / BT, op->nrows);
    op_matvec_bulk_kernel<R, KB><<<grid, BT, smem, op->ctx->stream>>>(op->dev(), scales, scales_dev, (const cx<R> *)src,
                                                                       (cx<R> *)dst, accumulate, op->ctx->d_err);
    op->ctx->launches++;
    return pg_check_launch(op->ctx);
}

template <typename R>
static int launch_op_matvec(pg_op *op, const pg_scales &scales, const cxd *scales_dev, const void *src, void *dst,
                            int accumulate, const double *inv_scale, void *copy_out)
{
    dim3 block(128);
    dim3 grid((op->N + 127) / 128, op->nrows);
    cudaStream_t s = op->ctx->stream;
    const OpDev d = op->dev();
    const cx<R> *x = (const cx<R> *)src;
    cx<R> *y = (cx<R> *)dst;
    cx<R> *c = (cx<R> *)copy_out;
    switch (op->kb) {
    case 6: op_matvec_kernel<R, 6><<<grid, block, 0, s>>>(d, scales, scales_dev, x, y, accumulate, inv_scale, c); break;
    case 8: op_matvec_kernel<R, 8><<<grid, block, 0, s>>>(d, scales, scales_dev, x, y, accumulate, inv_scale, c); break;
    case 4: op_matvec_kernel<R, 4><<<grid, block, 0, s>>>(d, scales, scales_dev, x, y, accumulate, inv_scale, c); break;
    default: op_matvec_kernel<R, -1><<<grid, block, 0, s>>>(d, scales, scales_dev, x, y, accumulate, inv_scale, c); break;
    }
    op->ctx->launches++;
    return pg_check_launch(op->ctx);
}

int pg_op_matvec_dev(pg_op *op, const pg_scales &scales, const cxd *scales_dev, const void *src, void *dst,
                     int accumulate, const double *src_inv_scale_dev, void *src_copy_out)
{
    if (!op || !op->finalized) return PG_ERR_STATE;
    if (op->kb == 6 && !src_inv_scale_dev && !src_copy_out && op->use_bulk) {
        if (op->precision == PG_FP64) return launch_bulk<double, 6>(op, scales, scales_dev, src, dst, accumulate);
        return launch_bulk<float, 6>(op, scales, scales_dev, src, dst, accumulate);
    }
    if (op->precision == PG_FP64)
        return launch_op_matvec<double>(op, scales, scales_dev, src, dst, accumulate, src_inv_scale_dev, src_copy_out);
    return launch_op_matvec<float>(op, scales, scales_dev, src, dst, accumulate, src_inv_scale_dev, src_copy_out);
}

extern "C" int pg_op_create(pg_ctx *ctx, int rank, const int *shape, int bandCount, int precision, pg_op **out)
{
    if (!ctx || !shape || !out || bandCount < 0) return PG_ERR_ARG;
    if (rank != 2) return PG_ERR_STORAGE;
    if (precision != PG_FP64 && precision != PG_FP32) return PG_ERR_ARG;
    if (shape[0] <= 0 || shape[1] <= 2 * bandCount) return PG_ERR_SHAPE;
    pg_op *op = new pg_op();
    op->ctx = ctx;
    op->rank = rank;
    op->nrows = shape[0];
    op->N = shape[1];
    op->kb = bandCount;
    op->b = 2 * bandCount + 1;
    op->ld = (op->N + 3) & ~3;
    op->use_bulk = 1;
    op->precision = precision;
    *out = op;
    return PG_OK;
}

extern "C" int pg_op_destroy(pg_op *op)
{
    if (!op) return PG_ERR_ARG;
    cudaFree(op->d_row_ptr);
    cudaFree(op->d_ent_col);
    cudaFree(op->d_ent_band);
    cudaFree(op->d_ent_slot);
    cudaFree(op->d_bands);
    delete op;
    return PG_OK;
}

extern "C" int pg_op_add_term(pg_op *op, const char *storage, const double *potential, int potExtent0,
                              int potExtent1, const int *pairs0, int npairs0, int slot)
{
    if (!op || !storage || (!potential && potExtent0 > 0)) return PG_ERR_ARG;
    if (op->finalized) return PG_ERR_STATE;
    if (slot < 0 || slot >= PG_MAX_SLOTS) return PG_ERR_ARG;
    HostTerm t;
    t.storage = storage;
    if (t.storage != "Diag_BandNH" && t.storage != "Simp_BandNH" && t.storage != "Ident_BandNH") return PG_ERR_STORAGE;
    if (potExtent1 != op->N * op->b) return PG_ERR_SHAPE;
    if (t.storage == "Diag_BandNH" && potExtent0 != op->nrows) return PG_ERR_SHAPE;
    if (t.storage == "Ident_BandNH" && potExtent0 != 1) return PG_ERR_SHAPE;
    if (t.storage == "Simp_BandNH") {
        if (npairs0 != potExtent0 || (npairs0 > 0 && !pairs0)) return PG_ERR_SHAPE;
        for (int p = 0; p < npairs0; ++p) {
            const int rr = pairs0[2 * p], cc = pairs0[2 * p + 1];
            if (rr < 0 || rr >= op->nrows || cc < 0 || cc >= op->nrows) return PG_ERR_SHAPE;
        }
        t.pairs.assign(pairs0, pairs0 + 2 * npairs0);
    }
    t.e0 = potExtent0;
    t.e1 = potExtent1;
    if (potExtent0 > 0) t.pot.assign(potential, potential + 2 * (size_t)potExtent0 * potExtent1);
    t.slot = slot;
    op->terms.push_back(std::move(t));
    return PG_OK;
}

template <typename R>
static int upload_bands(pg_op *op)
{
    // device rows of length ld (>= N, multiple of 4): every slab starts 16-byte aligned
    const size_t rows = op->h_bands.size() / (size_t)op->N;
    const size_t n = rows * (size_t)op->ld;
    std::vector<cx<R>> tmp(n, mk<R>((R)0, (R)0));
    for (size_t q = 0; q < rows; ++q)
        for (int i = 0; i < op->N; ++i) {
            const std::complex<double> v = op->h_bands[q * op->N + i];
            tmp[q * op->ld + i] = mk<R>((R)v.real(), (R)v.imag());
        }
    PG_CUDA_TRY(cudaMalloc(&op->d_bands, std::max<size_t>(1, n) * sizeof(cx<R>)));
    PG_CUDA_TRY(cudaMemcpy(op->d_bands, tmp.data(), n * sizeof(cx<R>), cudaMemcpyHostToDevice));
    return PG_OK;
}

extern "C" int pg_op_finalize(pg_op *op)
{
    if (!op) return PG_ERR_ARG;
    if (op->finalized) return PG_ERR_STATE;
    const int N = op->N, b = op->b, kb = op->kb, nrows = op->nrows;
    struct Ent { int row, col, band, slot; };
    std::vector<Ent> ents;
    std::vector<std::complex<double>> bands;
    auto add_band = [&](const double *pot) {
        // reference slot j*b + (kb + i - j) -> device [d][i], d = j - i + kb
        const int id = (int)(bands.size() / ((size_t)b * N));
        bands.resize(bands.size() + (size_t)b * N);
        std::complex<double> *B = bands.data() + (size_t)id * b * N;
        for (int d = 0; d < b; ++d)
            for (int i = 0; i < N; ++i) {
                const int j = i + d - kb;
                std::complex<double> v(0.0, 0.0);
                if (j >= 0 && j < N) {
                    const size_t s = (size_t)j * b + (kb + i - j);
                    v = std::complex<double>(pot[2 * s], pot[2 * s + 1]);
                }
                B[(size_t)d * N + i] = v;
            }
        return id;
    };
    for (const HostTerm &t : op->terms) {
        const size_t stride = (size_t)t.e1;
        if (t.storage == "Diag_BandNH") {
            for (int l = 0; l < nrows; ++l) ents.push_back({l, l, add_band(t.pot.data() + 2 * stride * l), t.slot});
        } else if (t.storage == "Ident_BandNH") {
            const int id = add_band(t.pot.data());
            for (int l = 0; l < nrows; ++l) ents.push_back({l, l, id, t.slot});
        } else {
            for (int p = 0; p < t.e0; ++p)
                ents.push_back({t.pairs[2 * p], t.pairs[2 * p + 1], add_band(t.pot.data() + 2 * stride * p), t.slot});
        }
    }
    std::stable_sort(ents.begin(), ents.end(), [](const Ent &a, const Ent &c) { return a.row < c.row; });
    op->h_row_ptr.assign(nrows + 1, 0);
    for (const Ent &e : ents) op->h_row_ptr[e.row + 1]++;
    for (int r = 0; r < nrows; ++r) op->h_row_ptr[r + 1] += op->h_row_ptr[r];
    op->h_ent_col.clear(); op->h_ent_band.clear(); op->h_ent_slot.clear();
    for (const Ent &e : ents) {
        op->h_ent_col.push_back(e.col);
        op->h_ent_band.push_back(e.band);
        op->h_ent_slot.push_back(e.slot);
    }
    op->nentries = (long long)ents.size();
    op->nbands = (int)(bands.size() / ((size_t)b * N));
    op->h_bands.swap(bands);
    const size_t ne = std::max<size_t>(1, ents.size());
    PG_CUDA_TRY(cudaMalloc(&op->d_row_ptr, (nrows + 1) * sizeof(int)));
    PG_CUDA_TRY(cudaMalloc(&op->d_ent_col, ne * sizeof(int)));
    PG_CUDA_TRY(cudaMalloc(&op->d_ent_band, ne * sizeof(int)));
    PG_CUDA_TRY(cudaMalloc(&op->d_ent_slot, ne * sizeof(int)));
    PG_CUDA_TRY(cudaMemcpy(op->d_row_ptr, op->h_row_ptr.data(), (nrows + 1) * sizeof(int), cudaMemcpyHostToDevice));
    if (!ents.empty()) {
        PG_CUDA_TRY(cudaMemcpy(op->d_ent_col, op->h_ent_col.data(), ents.size() * sizeof(int), cudaMemcpyHostToDevice));
        PG_CUDA_TRY(cudaMemcpy(op->d_ent_band, op->h_ent_band.data(), ents.size() * sizeof(int), cudaMemcpyHostToDevice));
        PG_CUDA_TRY(cudaMemcpy(op->d_ent_slot, op->h_ent_slot.data(), ents.size() * sizeof(int), cudaMemcpyHostToDevice));
    }
    int st = (op->precision == PG_FP64) ? upload_bands<double>(op) : upload_bands<float>(op);
    if (st != PG_OK) return st;
    op->finalized = true;
    return PG_OK;
}

extern "C" long long pg_op_stored_elements(const pg_op *op)
{
    if (!op) return -1;
    return (long long)op->nbands * op->b * op->N;
}

extern "C" int pg_op_matvec(pg_op *op, const double *scales, int nscales, const void *src, void *dst, int accumulate)
{
    if (!op || !src || !dst) return PG_ERR_ARG;
    if (nscales < 0 || nscales > PG_MAX_SLOTS || (nscales > 0 && !scales)) return PG_ERR_ARG;
    pg_scales sc;
    for (int k = 0; k < PG_MAX_SLOTS; ++k) sc.s[k] = mk<double>(k < nscales ? scales[2 * k] : 0.0, k < nscales ? scales[2 * k + 1] : 0.0);
    return pg_op_matvec_dev(op, sc, nullptr, src, dst, accumulate, nullptr, nullptr);
}
