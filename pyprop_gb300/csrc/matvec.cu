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

#include <map>

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
    const int r = pg_grid_row();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int N = op.N;
    if (i >= N || r >= op.nrows) return;
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
// dense radial blocks (radial storage "Dense"): dst[r][i] += sum_e s_e sum_j D_e[i][j] x_e[j],
// x_e = src[col_e] (times 1/src_inv_scale when given). One CTA = 128 radial rows of one
// angular row; the source row is staged through shared memory in tiles of 128, and D is
// stored transposed ([j][i]) so the threads of a warp read consecutive i.
template <typename R>
__global__ void __launch_bounds__(128) op_dense_kernel(int N, int nrows, const int *__restrict__ row_ptr,
                                                       const int *__restrict__ ent_col, const int *__restrict__ ent_mat,
                                                       const int *__restrict__ ent_slot, const cx<R> *__restrict__ dense,
                                                       pg_scales scales, const cxd *__restrict__ scales_dev,
                                                       const cx<R> *__restrict__ src, cx<R> *__restrict__ dst,
                                                       const double *__restrict__ src_inv_scale)
{
    __shared__ cx<R> xs[128];
    const int r = pg_grid_row();
    if (r >= nrows) return;
    const int i = blockIdx.x * 128 + threadIdx.x;
    const R sc = src_inv_scale ? (R)(1.0 / *src_inv_scale) : (R)1;
    cx<R> acc = mk<R>((R)0, (R)0);
    for (int e = row_ptr[r]; e < row_ptr[r + 1]; ++e) {
        const cx<R> *__restrict__ D = dense + (size_t)ent_mat[e] * N * N;
        const cx<R> *__restrict__ x = src + (size_t)ent_col[e] * N;
        cx<R> t = mk<R>((R)0, (R)0);
        for (int j0 = 0; j0 < N; j0 += 128) {
            __syncthreads();
            const int jj = j0 + threadIdx.x;
            xs[threadIdx.x] = jj < N ? x[jj] : mk<R>((R)0, (R)0);
            __syncthreads();
            const int jn = min(128, N - j0);
            if (i < N)
                for (int q = 0; q < jn; ++q) cfma(t, D[(size_t)(j0 + q) * N + i], xs[q]);
        }
        const int slot = ent_slot[e];
        const cx<R> s = scales_dev ? cvt<R>(scales_dev[slot]) : cvt<R>(scales.s[slot]);
        cfma(acc, s, t);
    }
    if (i < N) {
        const size_t o = (size_t)r * N + i;
        dst[o] = dst[o] + sc * acc;
    }
}

// ------------------------------------------------------------------------------------
// fused operator, bulk-copy staged variant
// ------------------------------------------------------------------------------------
// One CTA = BT radial rows of one angular row. Warp 0 issues one cp.async.bulk per
// (entry, diagonal) band slab [d][i0 .. i0+BT) into shared memory, all completing on one
// mbarrier (expected bytes), while all threads load the source slabs x[col][i0-kb .. i0+BT+kb)
// with ordinary coalesced loads. The whole CTA's operator tile is in flight at once, so the
// kernel is bound by HBM rather than by load latency. Entries of a row are processed in
// groups of BMAXE. Requires band leading dimension ld (>= N) with 16-byte aligned slabs.
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

// 3-D tensor copy of one box into shared memory, completing on the mbarrier
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int c0, int c1, int c2,
                                            unsigned long long *bar)
{
    asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n"
                 ::"r"(smem_u32(dst)), "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
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

template <typename R, int KB, int BT, int MODE, int GE>
__global__ void __launch_bounds__(BT) op_matvec_bulk_kernel(OpDev op, pg_scales scales, const cxd *__restrict__ scales_dev,
                                                            const cx<R> *__restrict__ src, cx<R> *__restrict__ dst,
                                                            int accumulate, int *err,
                                                            const __grid_constant__ CUtensorMap tmap,
                                                            const cx<R> *__restrict__ rowmajor)
{
    constexpr int B = 2 * KB + 1;
    extern __shared__ __align__(128) unsigned char mv_smem[];
    unsigned long long *bar = (unsigned long long *)mv_smem;
    cx<R> *bs = (cx<R> *)(mv_smem + 128);            // [GE][B][BT]
    cx<R> *xs = bs + (size_t)GE * B * BT;          // [GE][BT + 2KB]
    const int r = pg_grid_row();
    if (r >= op.nrows) return;  // CTA-uniform, before any barrier
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
    for (int e0 = e_begin; e0 < e_end; e0 += GE) {
        const int ne = min(GE, e_end - e0);
        if (MODE == 2) {
            // row-major band copy [band][ld][B]: one contiguous bulk copy per entry (the rows up
            // to the band's padded end ld, so the last tile stays inside its band)
            const int rows = min(BT, ld - i0);
            const unsigned bytes = (unsigned)(rows * B * sizeof(cx<R>));
            if (t < 32) {
                if (t == 0) mbar_arrive_expect_tx(bar, bytes * (unsigned)ne);
                __syncwarp();
                if (t < ne)
                    bulk_g2s(bs + (size_t)t * B * BT, rowmajor + ((size_t)op.ent_band[e0 + t] * ld + i0) * B, bytes, bar);
            }
        } else if (MODE == 1) {
            // one tensor copy per entry: the box [B diagonals][BT rows] of band ent_band (the
            // box is always full: rows past the band's end read as zero)
            if (t < 32) {
                if (t == 0) mbar_arrive_expect_tx(bar, (unsigned)(ne * B * BT * sizeof(cx<R>)));
                __syncwarp();
                if (t < ne) {
                    const int x0 = (sizeof(R) == 8 ? 2 : 1) * i0;
                    tma_load_3d(bs + (size_t)t * B * BT, &tmap, x0, 0, op.ent_band[e0 + t], bar);
                }
            }
        } else if (t < 32) {
            // lane 0 announces the bytes, then the 32 lanes of warp 0 issue the slab copies
            if (t == 0) mbar_arrive_expect_tx(bar, slab_bytes * (unsigned)(ne * B));
            __syncwarp();
            for (int sl = t; sl < ne * B; sl += 32) {
                const int q = sl / B, d = sl - q * B;
                const cx<R> *V = bands + (size_t)op.ent_band[e0 + q] * B * ld + i0;
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
                for (int d = 0; d < B; ++d) cfma(tq, MODE == 2 ? Vb[t * B + d] : Vb[d * BT + t], xb[d]);
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

// ------------------------------------------------------------------------------------
// persistent TMA variant: each CTA walks tiles (64 rows of one angular row) with a stride of
// the grid, the next unit's band boxes (TMA) and source halo (cp.async, zero-filled outside
// the fibre) in flight in one shared-memory stage while the current unit is computed from the
// other. A unit is a tile's group of up to BMAXE entries.
// ------------------------------------------------------------------------------------
__device__ __forceinline__ void cp_async_8(void *smem, const void *gmem, bool valid)
{
    const unsigned s = smem_u32(smem);
    const int n = valid ? 8 : 0;  // source size 0: the 8 bytes are zero-filled
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gmem), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async_16z(void *smem, const void *gmem, bool valid)
{
    const unsigned s = smem_u32(smem);
    const int n = valid ? 16 : 0;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async_commit_mv() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_mv(int pending)
{
    if (pending) asm volatile("cp.async.wait_group 1;\n" ::);
    else asm volatile("cp.async.wait_group 0;\n" ::);
}

template <typename R, int KB>
__global__ void __launch_bounds__(64) op_matvec_tma_persistent_kernel(OpDev op, pg_scales scales,
                                                                       const cxd *__restrict__ scales_dev,
                                                                       const cx<R> *__restrict__ src,
                                                                       cx<R> *__restrict__ dst, int accumulate,
                                                                       int *err, const __grid_constant__ CUtensorMap tmap)
{
    constexpr int BT = 64, B = 2 * KB + 1, XW = BT + 2 * KB;
    extern __shared__ __align__(128) unsigned char mv_smem[];
    unsigned long long *bar = (unsigned long long *)mv_smem;          // [2]
    cx<R> *bs = (cx<R> *)(mv_smem + 128);                             // [2][BMAXE][B][BT]
    cx<R> *xs = bs + (size_t)2 * BMAXE * B * BT;                      // [2][BMAXE][XW]
    const int t = threadIdx.x;
    const int N = op.N;
    const int tiles_i = (N + BT - 1) / BT;
    const long long ntiles = (long long)op.nrows * tiles_i;
    if (t == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    // unit iterator: (tile u, group g)
    auto ngroups = [&](long long u) {
        const int r = (int)(u / tiles_i);
        const int ne = op.row_ptr[r + 1] - op.row_ptr[r];
        return max(1, (ne + BMAXE - 1) / BMAXE);
    };
    auto issue = [&](long long u, int g, int stage) {
        const int r = (int)(u / tiles_i), i0 = (int)(u % tiles_i) * BT;
        const int e0 = op.row_ptr[r] + g * BMAXE;
        const int ne = max(0, min(BMAXE, op.row_ptr[r + 1] - e0));
        if (t < 32) {
            if (t == 0) mbar_arrive_expect_tx(&bar[stage], (unsigned)(ne * B * BT * sizeof(cx<R>)));
            __syncwarp();
            if (t < ne) {
                const int x0 = (sizeof(R) == 8 ? 2 : 1) * i0;
                tma_load_3d(bs + ((size_t)stage * BMAXE + t) * B * BT, &tmap, x0, 0, op.ent_band[e0 + t], &bar[stage]);
            }
        }
        for (int q = 0; q < ne; ++q) {
            const cx<R> *x = src + (size_t)op.ent_col[e0 + q] * N;
            cx<R> *xd = xs + ((size_t)stage * BMAXE + q) * XW;
            for (int u2 = t; u2 < XW; u2 += BT) {
                const int j = i0 - KB + u2;
                const bool ok = j >= 0 && j < N;
                if (sizeof(cx<R>) == 8) cp_async_8(xd + u2, ok ? (const void *)(x + j) : (const void *)x, ok);
                else cp_async_16z(xd + u2, ok ? (const void *)(x + j) : (const void *)x, ok);
            }
        }
        cp_async_commit_mv();
    };
    long long u = blockIdx.x;
    int g = 0;
    if (u >= ntiles) return;
    unsigned phase[2] = {0u, 0u};
    issue(u, 0, 0);
    int stage = 0;
    cx<R> acc = mk<R>((R)0, (R)0);
    for (;;) {
        // the unit after this one
        long long un = u;
        int gn = g + 1;
        if (gn >= ngroups(u)) {
            un = u + gridDim.x;
            gn = 0;
        }
        const bool more = un < ntiles;
        if (more) issue(un, gn, stage ^ 1);
        const bool ok = mbar_wait_bounded(&bar[stage], phase[stage], err);
        cp_async_wait_mv(more ? 1 : 0);
        if (__syncthreads_or(ok ? 0 : 1)) {
            // give up uniformly: wait (bounded) for the copies still in flight, then leave
            if (!ok) mbar_wait_bounded(&bar[stage], phase[stage], err);
            if (more) mbar_wait_bounded(&bar[stage ^ 1], phase[stage ^ 1], err);
            cp_async_wait_mv(0);
            return;
        }
        phase[stage] ^= 1u;
        const int r = (int)(u / tiles_i), i0 = (int)(u % tiles_i) * BT;
        const int e0 = op.row_ptr[r] + g * BMAXE;
        const int ne = max(0, min(BMAXE, op.row_ptr[r + 1] - e0));
        const int cnt = min(BT, N - i0);
        if (t < cnt) {
            for (int q = 0; q < ne; ++q) {
                const cx<R> *Vb = bs + ((size_t)stage * BMAXE + q) * B * BT;
                const cx<R> *xb = xs + ((size_t)stage * BMAXE + q) * XW + t;
                cx<R> tq = mk<R>((R)0, (R)0);
#pragma unroll
                for (int d = 0; d < B; ++d) cfma(tq, Vb[d * BT + t], xb[d]);
                const int slot = op.ent_slot[e0 + q];
                const cx<R> sc = scales_dev ? cvt<R>(scales_dev[slot]) : cvt<R>(scales.s[slot]);
                cfma(acc, sc, tq);
            }
        }
        if (gn == 0) {  // last group of this tile: store
            if (t < cnt) {
                const size_t o = (size_t)r * N + i0 + t;
                dst[o] = accumulate ? acc + dst[o] : acc;
            }
            acc = mk<R>((R)0, (R)0);
        }
        __syncthreads();  // this stage is refilled two units from now
        if (!more) break;
        u = un;
        g = gn;
        stage ^= 1;
    }
}

template <typename R, int KB>
static int launch_tma_persistent(pg_op *op, const pg_scales &scales, const cxd *scales_dev, const void *src, void *dst,
                                 int accumulate)
{
    constexpr int B = 2 * KB + 1, BT = 64;
    const size_t smem = 128 + sizeof(cx<R>) * ((size_t)2 * BMAXE * B * BT + (size_t)2 * BMAXE * (BT + 2 * KB));
    static bool configured = false;
    if (!configured) {
        PG_CUDA_TRY(cudaFuncSetAttribute(op_matvec_tma_persistent_kernel<R, KB>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        configured = true;
    }
    const long long ntiles = (long long)op->nrows * ((op->N + BT - 1) / BT);
    int per_sm = 1;
    PG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, op_matvec_tma_persistent_kernel<R, KB>, BT, smem));
    const long long grid = std::max<long long>(1, std::min<long long>(ntiles, (long long)std::max(1, per_sm) *
                                                                                  std::max(1, op->ctx->num_sms)));
    op_matvec_tma_persistent_kernel<R, KB><<<(unsigned)grid, BT, smem, op->ctx->stream>>>(
        op->dev(), scales, scales_dev, (const cx<R> *)src, (cx<R> *)dst, accumulate, op->ctx->d_err, op->tmap);
    op->ctx->launches++;
    return pg_check_launch(op->ctx);
}

template <typename R, int KB, int BT, int MODE, int GE = BMAXE>
static int launch_bulk_bt(pg_op *op, const pg_scales &scales, const cxd *scales_dev, const void *src, void *dst,
                          int accumulate)
{
    constexpr int B = 2 * KB + 1;
    const size_t smem = 128 + sizeof(cx<R>) * ((size_t)GE * B * BT + (size_t)GE * (BT + 2 * KB));
    static bool configured = false;
    if (!configured) {
        PG_CUDA_TRY(cudaFuncSetAttribute(op_matvec_bulk_kernel<R, KB, BT, MODE, GE>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        configured = true;
    }
    const dim3 grid = pg_row_grid((op->N + BT - 1) / BT, op->nrows);
    op_matvec_bulk_kernel<R, KB, BT, MODE, GE><<<grid, BT, smem, op->ctx->stream>>>(
        op->dev(), scales, scales_dev, (const cx<R> *)src, (cx<R> *)dst, accumulate, op->ctx->d_err, op->tmap,
        (const cx<R> *)op->d_bands_rm);
    op->ctx->launches++;
    return pg_check_launch(op->ctx);
}

// tile width by the operator's tuned variant (64-row tiles: more CTAs; 128-row: fewer, larger copies)
template <typename R, int KB>
static int launch_bulk(pg_op *op, const pg_scales &scales, const cxd *scales_dev, const void *src, void *dst,
                       int accumulate)
{
    if (op->variant == 2) return launch_bulk_bt<R, KB, 128, 0>(op, scales, scales_dev, src, dst, accumulate);
    if (op->variant == 4 && op->has_tmap) return launch_bulk_bt<R, KB, 64, 1>(op, scales, scales_dev, src, dst, accumulate);
    if (op->variant == 5 && op->has_tmap) return launch_tma_persistent<R, KB>(op, scales, scales_dev, src, dst, accumulate);
    if (op->variant == 6 && op->d_bands_rm) return launch_bulk_bt<R, KB, 64, 2>(op, scales, scales_dev, src, dst, accumulate);
    if (op->variant == 7 && op->has_tmap) return launch_bulk_bt<R, KB, 64, 1, 2>(op, scales, scales_dev, src, dst, accumulate);
    if (op->variant == 8 && op->has_tmap) return launch_bulk_bt<R, KB, 64, 1, 1>(op, scales, scales_dev, src, dst, accumulate);
    return launch_bulk_bt<R, KB, 64, 0>(op, scales, scales_dev, src, dst, accumulate);
}

template <typename R>
static int launch_op_matvec(pg_op *op, const pg_scales &scales, const cxd *scales_dev, const void *src, void *dst,
                            int accumulate, const double *inv_scale, void *copy_out)
{
    dim3 block(128);
    const dim3 grid = pg_row_grid((op->N + 127) / 128, op->nrows);
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

template <typename R>
static int launch_dense(pg_op *op, const pg_scales &scales, const cxd *scales_dev, const void *src, void *dst,
                        const double *inv_scale)
{
    const dim3 grid = pg_row_grid((op->N + 127) / 128, op->nrows);
    op_dense_kernel<R><<<grid, 128, 0, op->ctx->stream>>>(op->N, op->nrows, op->d_drow_ptr, op->d_dent_col, op->d_dent_mat,
                                                          op->d_dent_slot, (const cx<R> *)op->d_dense, scales,
                                                          scales_dev, (const cx<R> *)src, (cx<R> *)dst, inv_scale);
    op->ctx->launches++;
    return pg_check_launch(op->ctx);
}

int pg_op_matvec_kernels(const pg_op *op) { return (op->ndense_entries > 0 ? 2 : 1) + (op->fact.Q > 0 ? 2 : 0); }

int pg_op_matvec_dev(pg_op *op, const pg_scales &scales, const cxd *scales_dev, const void *src, void *dst,
                     int accumulate, const double *src_inv_scale_dev, void *src_copy_out)
{
    if (!op || !op->finalized) return PG_ERR_STATE;
    const bool fp64 = op->precision == PG_FP64;
    if (op->kb == 6 && !src_inv_scale_dev && !src_copy_out && op->use_bulk && op->variant != 3) {
        PG_TRY(fp64 ? launch_bulk<double, 6>(op, scales, scales_dev, src, dst, accumulate)
                    : launch_bulk<float, 6>(op, scales, scales_dev, src, dst, accumulate));
    } else {
        PG_TRY(fp64 ? launch_op_matvec<double>(op, scales, scales_dev, src, dst, accumulate, src_inv_scale_dev,
                                               src_copy_out)
                    : launch_op_matvec<float>(op, scales, scales_dev, src, dst, accumulate, src_inv_scale_dev,
                                              src_copy_out));
    }
    if (op->ndense_entries > 0)
        PG_TRY(fp64 ? launch_dense<double>(op, scales, scales_dev, src, dst, src_inv_scale_dev)
                    : launch_dense<float>(op, scales, scales_dev, src, dst, src_inv_scale_dev));
    if (op->fact.Q > 0 && !op->tuning) PG_TRY(pg_factored_apply(op, scales, scales_dev, src, dst, src_inv_scale_dev));
    return PG_OK;
}

extern "C" int pg_op_create(pg_ctx *ctx, int rank, const int *shape, int bandCount, int precision, pg_op **out)
{
    if (!ctx || !shape || !out || bandCount < 0) return PG_ERR_ARG;
    if (rank != 2 && rank != 3) return PG_ERR_STORAGE;
    if (precision != PG_FP64 && precision != PG_FP32) return PG_ERR_ARG;
    long long rows = 1;
    for (int r = 0; r < rank - 1; ++r) {
        if (shape[r] <= 0) return PG_ERR_SHAPE;
        rows *= shape[r];
    }
    if (rows > (1LL << 30) || shape[rank - 1] <= 2 * bandCount) return PG_ERR_SHAPE;
    pg_op *op = new pg_op();
    op->ctx = ctx;
    op->rank = rank;
    op->shape.assign(shape, shape + rank);
    // the last rank is the banded fibre; all other ranks together index the fibres
    op->nrows = (int)rows;
    op->N = shape[rank - 1];
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
    cudaFree(op->d_bands_rm);
    cudaFree(op->d_drow_ptr);
    cudaFree(op->d_dent_col);
    cudaFree(op->d_dent_mat);
    cudaFree(op->d_dent_slot);
    cudaFree(op->d_dense);
    pg_factored_free(op);
    delete op;
    return PG_OK;
}

// Storage ids "<rank 0>_<rank 1>[_<rank 2>]" of the reference's generated multiply kernels
// (core/tensorpotential/tensorpotentialmultiply_generator.py): every rank but the last is
// Simp, Herm, Diag, Ident, Band, BandNH or Dense (:302-462, :467-618, :622-762, :1227-1330);
// the last (fibre) rank is BandNH, Band, Dense, Diag, Ident or Simp. potential holds
// prod(extents) complex128 in the reference's layout; pairs lists (row, col) of every Simp or
// Herm rank, in rank order.
static bool outer_kind(const std::string &s)
{
    return s == "Simp" || s == "Herm" || s == "Diag" || s == "Ident" || s == "Band" || s == "BandNH" || s == "Dense";
}
static bool inner_kind(const std::string &s)
{
    return s == "BandNH" || s == "Band" || s == "Dense" || s == "Diag" || s == "Ident" || s == "Simp";
}
static bool has_pairs(const std::string &s) { return s == "Simp" || s == "Herm"; }

static int add_term(pg_op *op, const char *storage, const double *potential, const int *extents, const int *pairs,
                    const int *npairs, int slot)
{
    if (!op || !storage || !extents) return PG_ERR_ARG;
    if (op->finalized) return PG_ERR_STATE;
    if (slot < 0 || slot >= PG_MAX_SLOTS) return PG_ERR_ARG;
    const int R = op->rank;
    HostTerm t;
    t.storage = storage;
    size_t start = 0;
    for (;;) {
        const size_t us = t.storage.find('_', start);
        t.kinds.push_back(t.storage.substr(start, us == std::string::npos ? std::string::npos : us - start));
        if (us == std::string::npos) break;
        start = us + 1;
    }
    if ((int)t.kinds.size() != R) return PG_ERR_STORAGE;
    for (int r = 0; r < R - 1; ++r)
        if (!outer_kind(t.kinds[r])) return PG_ERR_STORAGE;
    if (!inner_kind(t.kinds[R - 1])) return PG_ERR_STORAGE;
    size_t total = 1;
    const int *pp = pairs;
    t.pairs.resize(R);
    for (int r = 0; r < R; ++r) {
        const std::string &k = t.kinds[r];
        const int e = extents[r], n = op->shape[r];
        if (e < 0) return PG_ERR_SHAPE;
        total *= (size_t)e;
        if (has_pairs(k)) {
            if (!npairs || npairs[r] != e || (e > 0 && !pp)) return PG_ERR_SHAPE;
            if (r == R - 1 && k == "Herm") return PG_ERR_STORAGE;
            for (int q = 0; q < e; ++q)
                if (pp[2 * q] < 0 || pp[2 * q] >= n || pp[2 * q + 1] < 0 || pp[2 * q + 1] >= n) return PG_ERR_SHAPE;
            t.pairs[r].assign(pp, pp + 2 * (size_t)e);
            pp += 2 * (size_t)e;
        } else if (k == "Diag") {
            if (e != n) return PG_ERR_SHAPE;
        } else if (k == "Ident") {
            if (e != 1) return PG_ERR_SHAPE;
        } else if (k == "Dense") {
            if (e != n * n) return PG_ERR_SHAPE;
        } else if (r == R - 1) {  // banded fibre storage
            if (k == "BandNH" && e != n * op->b) return PG_ERR_SHAPE;
            if (k == "Band" && e != n * (op->kb + 1)) return PG_ERR_SHAPE;
        } else {  // Band / BandNH outer: extent n * bandCount
            if (e <= 0 || e % n != 0) return PG_ERR_SHAPE;
            if (k == "BandNH" && (e / n) % 2 == 0) return PG_ERR_SHAPE;
        }
    }
    if (total > 0 && !potential) return PG_ERR_ARG;
    t.ext.assign(extents, extents + R);
    if (total > 0) t.pot.assign(potential, potential + 2 * total);
    t.slot = slot;
    op->terms.push_back(std::move(t));
    return PG_OK;
}

extern "C" int pg_op_add_term(pg_op *op, const char *storage, const double *potential, int potExtent0,
                              int potExtent1, const int *pairs0, int npairs0, int slot)
{
    if (!op) return PG_ERR_ARG;
    if (op->rank != 2) return PG_ERR_STATE;  // rank-3 operators take pg_op_add_term_ranks
    const int ext[2] = {potExtent0, potExtent1};
    const int np[2] = {npairs0, 0};
    return add_term(op, storage, potential, ext, pairs0, np, slot);
}

extern "C" int pg_op_add_term_ranks(pg_op *op, const char *storage, const double *potential, const int *extents,
                                    const int *pairs, const int *npairs, int slot)
{
    return add_term(op, storage, potential, extents, pairs, npairs, slot);
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

// One angular (row, col) block of a term: the radial data at index i0 of the angular rank,
// complex conjugated when the reference's loop passes conjugate = true (the mirrored half of
// Herm and Band angular storage).
struct BlockRef {
    int row, col;
    size_t i0;
    bool conj;
};

// Expansion of one non-fibre rank, following the generator's loops for each storage: the
// (row, col) blocks with the potential index along that rank and the conjugate flag.
static void expand_rank(const std::string &kind, int e, const std::vector<int> &pairs, int n,
                        std::vector<BlockRef> &out)
{
    if (kind == "Simp" || kind == "Herm") {
        for (int p = 0; p < e; ++p) out.push_back({pairs[2 * p], pairs[2 * p + 1], (size_t)p, false});
        if (kind == "Herm")  // :380-386: second pass with row/col swapped and the potential conjugated
            for (int p = 0; p < e; ++p) out.push_back({pairs[2 * p + 1], pairs[2 * p], (size_t)p, true});
    } else if (kind == "Diag") {
        for (int l = 0; l < n; ++l) out.push_back({l, l, (size_t)l, false});
    } else if (kind == "Ident") {
        for (int l = 0; l < n; ++l) out.push_back({l, l, 0, false});
    } else if (kind == "Dense") {  // :1268-1275: index row * n + col
        for (int r = 0; r < n; ++r)
            for (int c = 0; c < n; ++c) out.push_back({r, c, (size_t)r * n + c, false});
    } else if (kind == "Band") {
        // :507-552: stored (row, col >= row) at row * bc + (col - row); mirrored (col, row) conjugated
        const int bc = e / n;
        for (int r = 0; r < n; ++r)
            for (int c = r; c < std::min(n, r + bc); ++c) out.push_back({r, c, (size_t)r * bc + (c - r), false});
        for (int r = 0; r < n; ++r)
            for (int c = r + 1; c < std::min(n, r + bc); ++c) out.push_back({c, r, (size_t)r * bc + (c - r), true});
    } else {  // BandNH, :662-694: element (row, col) at col * bc + (sub + row - col)
        const int bc = e / n, sub = (bc - 1) / 2;
        for (int c = 0; c < n; ++c)
            for (int r = std::max(0, c - sub); r <= std::min(n - 1, c + sub); ++r)
                out.push_back({r, c, (size_t)c * bc + (sub + r - c), false});
    }
}

// All non-fibre ranks of a term: rank r's loop nests inside rank r-1's (the generator's
// nesting), rows and columns flatten C-order, potential indices flatten over the extents,
// and conjugate flags of nested ranks combine (each mirrored pass toggles the flag).
static void expand_outer(const HostTerm &t, const std::vector<int> &shape, std::vector<BlockRef> &out)
{
    out.assign(1, BlockRef{0, 0, 0, false});
    std::vector<BlockRef> rank_blocks, next;
    for (size_t r = 0; r + 1 < t.kinds.size(); ++r) {
        rank_blocks.clear();
        expand_rank(t.kinds[r], t.ext[r], t.pairs[r], shape[r], rank_blocks);
        next.clear();
        next.reserve(out.size() * rank_blocks.size());
        for (const BlockRef &a : out)
            for (const BlockRef &q : rank_blocks)
                next.push_back({a.row * shape[r] + q.row, a.col * shape[r] + q.col, a.i0 * (size_t)t.ext[r] + q.i0,
                                a.conj != q.conj});
        out.swap(next);
    }
}

static int autotune(pg_op *op);

// Row-major copy of the bands, [band][ld][2kb+1] (transposed on the device from [band][2kb+1][ld]),
// for the variant that loads each tile's band block as one contiguous bulk copy.
template <typename R>
__global__ void bands_rowmajor_kernel(const cx<R> *__restrict__ dm, cx<R> *__restrict__ rm, int B, int ld, long long n)
{
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const long long band = e / ((long long)B * ld);
        const long long rem = e - band * B * ld;
        const int i = (int)(rem / B), d = (int)(rem - (long long)i * B);
        rm[e] = dm[(band * B + d) * ld + i];
    }
}

static int make_rowmajor_bands(pg_op *op)
{
    if (op->d_bands_rm || op->nbands == 0) return PG_OK;
    const size_t esz = op->precision == PG_FP64 ? sizeof(cxd) : sizeof(cxf);
    const long long n = (long long)op->nbands * op->b * op->ld;
    if (cudaMalloc(&op->d_bands_rm, esz * n) != cudaSuccess) {  // no room: the variant is not offered
        cudaGetLastError();
        op->d_bands_rm = nullptr;
        return PG_OK;
    }
    const int nb = (int)std::min<long long>((n + 255) / 256, 4096);
    if (op->precision == PG_FP64)
        bands_rowmajor_kernel<double><<<nb, 256, 0, op->ctx->stream>>>((const cxd *)op->d_bands, (cxd *)op->d_bands_rm,
                                                                      op->b, op->ld, n);
    else
        bands_rowmajor_kernel<float><<<nb, 256, 0, op->ctx->stream>>>((const cxf *)op->d_bands, (cxf *)op->d_bands_rm,
                                                                     op->b, op->ld, n);
    return pg_check_launch(op->ctx);
}

// Tensor map of the band array [nbands][2kb+1][ld] (complex64 as 8-byte elements, complex128
// as pairs of doubles) with a box of one band's 2kb+1 diagonals x 64 rows, for the TMA variant
// of the bulk matvec. Without the driver entry point the variant is simply not offered.
static void make_band_tensor_map(pg_op *op)
{
    typedef CUresult (*EncodeTiled)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                    const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                    CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    op->has_tmap = false;
    if (op->kb != 6 || op->nbands == 0 || !op->d_bands) return;
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
        return;
    const int per = op->precision == PG_FP64 ? 2 : 1;  // 8-byte elements per complex
    const cuuint64_t dims[3] = {(cuuint64_t)op->ld * per, (cuuint64_t)op->b, (cuuint64_t)op->nbands};
    const cuuint64_t strides[2] = {(cuuint64_t)op->ld * per * 8, (cuuint64_t)op->ld * per * 8 * op->b};
    const cuuint32_t box[3] = {(cuuint32_t)(64 * per), (cuuint32_t)op->b, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = ((EncodeTiled)fn)(&op->tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, op->d_bands, dims, strides, box, estr,
                                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    op->has_tmap = (r == CUDA_SUCCESS);
}

extern "C" int pg_op_finalize(pg_op *op)
{
    if (!op) return PG_ERR_ARG;
    if (op->finalized) return PG_ERR_STATE;
    const int N = op->N, b = op->b, kb = op->kb, nrows = op->nrows;
    typedef std::complex<double> zc;
    struct Ent { int row, col, band, slot; };
    std::vector<Ent> ents, dents;
    std::vector<zc> bands, dense;
    // fibre block -> general band [d][i] (d = j - i + kb); false when it is all zero
    auto radial_band = [&](const HostTerm &t, const double *pot, bool conj, std::vector<zc> &B) {
        const std::string &inner = t.kinds.back();
        B.assign((size_t)b * N, zc(0.0, 0.0));
        auto val = [&](size_t s) { return zc(pot[2 * s], pot[2 * s + 1]); };
        if (inner == "Simp") {  // (i, j) pair list, all within the band (checked by the caller)
            const std::vector<int> &pr = t.pairs.back();
            for (int p = 0; p < t.ext.back(); ++p) {
                const int i = pr[2 * p], j = pr[2 * p + 1];
                const zc v = conj ? std::conj(val(p)) : val(p);
                B[(size_t)(j - i + kb) * N + i] += v;
            }
        } else {
            for (int d = 0; d < b; ++d)
                for (int i = 0; i < N; ++i) {
                    const int j = i + d - kb;
                    if (j < 0 || j >= N) continue;
                    zc v(0.0, 0.0);
                    if (inner == "BandNH") {
                        v = val((size_t)j * b + (kb + i - j));  // zgbmv band layout, :700-723
                        if (conj) v = std::conj(v);
                    } else if (inner == "Band") {
                        // zhbmv('L') (:585-600): lower triangle column-major with lda = kb + 1,
                        // upper = conjugate, imaginary part of the diagonal ignored. The reference
                        // calls zhbmv whatever the conjugate flag, and so does this expansion.
                        const int kl = kb + 1;
                        if (i > j) v = val((size_t)j * kl + (i - j));
                        else if (i < j) v = std::conj(val((size_t)i * kl + (j - i)));
                        else v = zc(val((size_t)j * kl).real(), 0.0);
                    } else if (inner == "Diag") {
                        if (i == j) v = conj ? std::conj(val(i)) : val(i);
                    } else {  // Ident: one value for the whole diagonal
                        if (i == j) v = conj ? std::conj(val(0)) : val(0);
                    }
                    B[(size_t)d * N + i] = v;
                }
        }
        for (const zc &v : B)
            if (v != zc(0.0, 0.0)) return true;
        return false;
    };
    // fibre block -> dense [j][i] (transposed); false when it is all zero
    auto radial_dense = [&](const HostTerm &t, const double *pot, bool conj, std::vector<zc> &D) {
        const std::string &inner = t.kinds.back();
        D.assign((size_t)N * N, zc(0.0, 0.0));
        auto val = [&](size_t s) { return zc(pot[2 * s], pot[2 * s + 1]); };
        if (inner == "Dense") {  // :1268-1275, index row * N + col
            for (int i = 0; i < N; ++i)
                for (int j = 0; j < N; ++j) D[(size_t)j * N + i] = conj ? std::conj(val((size_t)i * N + j)) : val((size_t)i * N + j);
        } else {  // Simp pairs reaching outside the band
            const std::vector<int> &pr = t.pairs.back();
            for (int p = 0; p < t.ext.back(); ++p)
                D[(size_t)pr[2 * p + 1] * N + pr[2 * p]] += conj ? std::conj(val(p)) : val(p);
        }
        for (const zc &v : D)
            if (v != zc(0.0, 0.0)) return true;
        return false;
    };
    std::vector<BlockRef> blocks;
    std::vector<zc> B;
    for (const HostTerm &t : op->terms) {
        expand_outer(t, op->shape, blocks);
        const size_t stride = (size_t)t.ext.back();
        const std::string &inner = t.kinds.back();
        bool as_dense = inner == "Dense";
        if (inner == "Simp") {
            const std::vector<int> &pr = t.pairs.back();
            for (int p = 0; p < t.ext.back() && !as_dense; ++p) as_dense = std::abs(pr[2 * p] - pr[2 * p + 1]) > kb;
        }
        // blocks that read the same potential entry (Ident ranks, both Herm halves of a
        // real block, ...) share one device copy; -1 marks an all-zero block
        std::map<std::pair<size_t, bool>, int> made;
        for (const BlockRef &br : blocks) {
            const auto key = std::make_pair(br.i0, br.conj);
            auto it = made.find(key);
            int id;
            if (it != made.end()) {
                id = it->second;
            } else {
                const double *pot = t.pot.data() + 2 * stride * br.i0;
                id = -1;
                if (as_dense) {
                    if (radial_dense(t, pot, br.conj, B)) {
                        id = (int)(dense.size() / ((size_t)N * N));
                        dense.insert(dense.end(), B.begin(), B.end());
                    }
                } else if (radial_band(t, pot, br.conj, B)) {
                    id = (int)(bands.size() / ((size_t)b * N));
                    bands.insert(bands.end(), B.begin(), B.end());
                }
                made[key] = id;
            }
            if (id < 0) continue;  // an all-zero block adds nothing
            (as_dense ? dents : ents).push_back({br.row, br.col, id, t.slot});
        }
    }
    auto build_csr = [&](std::vector<Ent> &e, std::vector<int> &row_ptr) {
        std::stable_sort(e.begin(), e.end(), [](const Ent &a, const Ent &c) { return a.row < c.row; });
        row_ptr.assign(nrows + 1, 0);
        for (const Ent &x : e) row_ptr[x.row + 1]++;
        for (int r = 0; r < nrows; ++r) row_ptr[r + 1] += row_ptr[r];
    };
    build_csr(ents, op->h_row_ptr);
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
    if (!dents.empty()) {
        std::vector<int> drow;
        build_csr(dents, drow);
        std::vector<int> dcol, dmat, dslot;
        for (const Ent &e : dents) { dcol.push_back(e.col); dmat.push_back(e.band); dslot.push_back(e.slot); }
        op->ndense = (int)(dense.size() / ((size_t)N * N));
        op->ndense_entries = (long long)dents.size();
        PG_CUDA_TRY(cudaMalloc(&op->d_drow_ptr, (nrows + 1) * sizeof(int)));
        PG_CUDA_TRY(cudaMalloc(&op->d_dent_col, dents.size() * sizeof(int)));
        PG_CUDA_TRY(cudaMalloc(&op->d_dent_mat, dents.size() * sizeof(int)));
        PG_CUDA_TRY(cudaMalloc(&op->d_dent_slot, dents.size() * sizeof(int)));
        PG_CUDA_TRY(cudaMemcpy(op->d_drow_ptr, drow.data(), (nrows + 1) * sizeof(int), cudaMemcpyHostToDevice));
        PG_CUDA_TRY(cudaMemcpy(op->d_dent_col, dcol.data(), dcol.size() * sizeof(int), cudaMemcpyHostToDevice));
        PG_CUDA_TRY(cudaMemcpy(op->d_dent_mat, dmat.data(), dmat.size() * sizeof(int), cudaMemcpyHostToDevice));
        PG_CUDA_TRY(cudaMemcpy(op->d_dent_slot, dslot.data(), dslot.size() * sizeof(int), cudaMemcpyHostToDevice));
        const size_t cnt = dense.size();
        if (op->precision == PG_FP64) {
            std::vector<cxd> tmp(cnt);
            for (size_t q = 0; q < cnt; ++q) tmp[q] = mk<double>(dense[q].real(), dense[q].imag());
            PG_CUDA_TRY(cudaMalloc(&op->d_dense, cnt * sizeof(cxd)));
            PG_CUDA_TRY(cudaMemcpy(op->d_dense, tmp.data(), cnt * sizeof(cxd), cudaMemcpyHostToDevice));
        } else {
            std::vector<cxf> tmp(cnt);
            for (size_t q = 0; q < cnt; ++q) tmp[q] = mk<float>((float)dense[q].real(), (float)dense[q].imag());
            PG_CUDA_TRY(cudaMalloc(&op->d_dense, cnt * sizeof(cxf)));
            PG_CUDA_TRY(cudaMemcpy(op->d_dense, tmp.data(), cnt * sizeof(cxf), cudaMemcpyHostToDevice));
        }
    }
    PG_TRY(pg_factored_finalize(op));
    op->finalized = true;
    make_band_tensor_map(op);
    op->tuning = true;
    st = autotune(op);
    op->tuning = false;
    return st;
}

// The matvec kernel variant for this operator, by measurement: each candidate runs 2 untimed
// and 5 timed launches (CUDA events on the context's stream) on zero vectors of the
// operator's shape; the fastest is kept. All variants compute the same sums in the same order.
static int autotune(pg_op *op)
{
    op->variant = 1;
    if (op->kb != 6 || !op->use_bulk) return PG_OK;  // only the bulk kernels have variants
    cudaStream_t s = op->ctx->stream;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    PG_CUDA_TRY(cudaStreamIsCapturing(s, &cs));
    if (cs != cudaStreamCaptureStatusNone) return PG_OK;  // no timing inside a capture
    const size_t esz = op->precision == PG_FP64 ? sizeof(cxd) : sizeof(cxf);
    const size_t n = (size_t)op->nrows * op->N;
    void *x = nullptr, *y = nullptr;
    PG_CUDA_TRY(cudaMalloc(&x, esz * n));
    PG_CUDA_TRY(cudaMalloc(&y, esz * n));
    PG_CUDA_TRY(cudaMemsetAsync(x, 0, esz * n, s));
    cudaEvent_t a, b;
    PG_CUDA_TRY(cudaEventCreate(&a));
    PG_CUDA_TRY(cudaEventCreate(&b));
    pg_scales sc;
    memset(&sc, 0, sizeof(sc));
    const long long launches = op->ctx->launches;
    int code = PG_OK;
    float best = 1e30f;
    int best_v = 1;
    code = make_rowmajor_bands(op);
    for (int v = 1; v <= 8 && code == PG_OK; ++v) {
        if ((v == 4 || v == 5 || v >= 7) && !op->has_tmap) continue;
        if (v == 6 && !op->d_bands_rm) continue;
        op->variant = v;
        for (int k = 0; k < 2 && code == PG_OK; ++k) code = pg_op_matvec_dev(op, sc, nullptr, x, y, 0, nullptr, nullptr);
        if (code != PG_OK) break;
        cudaEventRecord(a, s);
        for (int k = 0; k < 5 && code == PG_OK; ++k) code = pg_op_matvec_dev(op, sc, nullptr, x, y, 0, nullptr, nullptr);
        cudaEventRecord(b, s);
        if (cudaEventSynchronize(b) != cudaSuccess) code = PG_ERR_CUDA;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        op->variant_us[v] = 1e3f * ms / 5.f;
        if (op->variant_us[v] < best) {
            best = op->variant_us[v];
            best_v = v;
        }
    }
    op->ctx->launches = launches;  // tuning launches are not the caller's work
    op->variant = best_v;
    if (best_v != 6 && op->d_bands_rm) {  // the row-major copy is kept only when it is used
        cudaFree(op->d_bands_rm);
        op->d_bands_rm = nullptr;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(x);
    cudaFree(y);
    return code;
}

// Force (1 bulk 64-row tiles, 2 bulk 128-row, 3 plain loads) or read (variant < 0) the matvec
// kernel variant; times_us (optional, 4 floats) receives the tuning measurements.
extern "C" int pg_op_variant(pg_op *op, int variant, int *current, float *times_us)
{
    if (!op || !op->finalized) return PG_ERR_STATE;
    if ((variant >= 1 && variant <= 3) || ((variant == 4 || variant == 5 || variant == 7 || variant == 8) && op->has_tmap))
        op->variant = variant;
    else if (variant == 6) {
        PG_TRY(make_rowmajor_bands(op));
        if (!op->d_bands_rm) return PG_ERR_ARG;
        op->variant = 6;
    }
    else if (variant >= 0) return PG_ERR_ARG;
    if (current) *current = op->variant;
    if (times_us)
        for (int k = 0; k < 9; ++k) times_us[k] = op->variant_us[k];
    return PG_OK;
}

extern "C" long long pg_op_stored_elements(const pg_op *op)
{
    if (!op) return -1;
    return (long long)op->nbands * op->b * op->N + (long long)op->ndense * op->N * op->N;
}

extern "C" int pg_op_matvec(pg_op *op, const double *scales, int nscales, const void *src, void *dst, int accumulate)
{
    if (!op || !src || !dst) return PG_ERR_ARG;
    if (nscales < 0 || nscales > PG_MAX_SLOTS || (nscales > 0 && !scales)) return PG_ERR_ARG;
    pg_scales sc;
    for (int k = 0; k < PG_MAX_SLOTS; ++k) sc.s[k] = mk<double>(k < nscales ? scales[2 * k] : 0.0, k < nscales ? scales[2 * k + 1] : 0.0);
    return pg_op_matvec_dev(op, sc, nullptr, src, dst, accumulate, nullptr, nullptr);
}
