// Blocked triangular solves of one fibre held in shared memory: the device routine behind the
// block-diagonal preconditioner solve (banded.cu) and the fused Cayley step (cayley_fused.cu).
#pragma once
#include "pg_internal.cuh"

template <typename R> __device__ __forceinline__ cx<R> shfl_cx(cx<R> v, int lane)
{
    v.x = __shfl_sync(0xffffffffu, v.x, lane);
    v.y = __shfl_sync(0xffffffffu, v.y, lane);
    return v;
}

// coefficient multiply-add: acc += c * v (c real or complex)
template <typename R> __device__ __forceinline__ void coef_fma(cx<R> &acc, R c, cx<R> v)
{
    acc.x = fma(c, v.x, acc.x);
    acc.y = fma(c, v.y, acc.y);
}
template <typename R> __device__ __forceinline__ void coef_fma(cx<R> &acc, cx<R> c, cx<R> v) { cfma(acc, c, v); }
template <typename R> __device__ __forceinline__ void coef_fms(cx<R> &acc, R c, cx<R> v)
{
    acc.x = fma(-c, v.x, acc.x);
    acc.y = fma(-c, v.y, acc.y);
}
template <typename R> __device__ __forceinline__ void coef_fms(cx<R> &acc, cx<R> c, cx<R> v) { cfma(acc, mk<R>(-c.x, -c.y), v); }

// factor loads through L2 only: every factor element is read once per solve, so caching it in
// L1 would only evict data that callers reuse
__device__ __forceinline__ float tri_ld(const float *p) { return __ldcg(p); }
__device__ __forceinline__ double tri_ld(const double *p) { return __ldcg(p); }
__device__ __forceinline__ cx<float> tri_ld(const cx<float> *p)
{
    const float2 v = __ldcg((const float2 *)p);
    return mk<float>(v.x, v.y);
}
__device__ __forceinline__ cx<double> tri_ld(const cx<double> *p)
{
    const double2 v = __ldcg((const double2 *)p);
    return mk<double>(v.x, v.y);
}
// factor loads from global memory (through L2) or, with SMEM_TAB, from tables the caller
// staged in shared memory
template <bool SMEM_TAB, typename C> __device__ __forceinline__ C tri_ldt(const C *p)
{
    if constexpr (SMEM_TAB) return *p;
    else return tri_ld(p);
}

// Blocked triangular solves, parallel over the blocks of a fibre. With T_b the 32x32 diagonal
// block of block b and C_b its coupling to the w boundary values s of the neighbouring block
// (lower sweep: the last w values of block b-1; upper sweep: the first w values of block
// b+1), the solution of block b is
//     y_b = z_b - G_b s,   z_b = T_b^-1 f_b,   G_b = T_b^-1 C_b   (G_b: 32 x w, precomputed).
// The boundary values of all blocks solve the block-bidiagonal system
//     s_b + G_b[boundary rows] s_{b-/+1} = z_b[boundary rows],
// whose inverse Rb (nblk*w square, block triangular) depends only on the factor, so it is
// precomputed on the host: s = Rb z[boundary rows]. Every step is then parallel - z_b for all
// blocks, the Rb product, the corrections G_b s - with no sequential recurrence left. Lane t
// of a warp owns row 32b + t of block b; the fibre stays in shared memory for both sweeps.
// C: coefficient type (R or cx<R>). inv: [nmat][nblk][32 s][32 t] = T^-1[t][s],
// g: [nmat][nblk][w c][32 t] = G[t][c], rb: [nmat][nblk*w][nblk*w] row-major.
//
// tri_solve_smem runs both sweeps with the CTA's NW warps on xs ([nblk*32], zero past the
// fibre's end) for factor m; sb ([nblk*w]) and sg ([nblk][w][32], when g_in_smem) are shared
// scratch. Callers synchronise the CTA before the call; it returns after a CTA barrier.
// SMEM_TAB: the factor tables (inv, g, rb) are in shared memory (g_in_smem is then 0).
template <typename R, typename C, int NW, bool SMEM_TAB = false>
__device__ __forceinline__ void tri_solve_smem(int nblk, int w, size_t m, const C *__restrict__ lo_inv,
                                               const C *__restrict__ lo_g, const C *__restrict__ lo_rb,
                                               const C *__restrict__ up_inv, const C *__restrict__ up_g,
                                               const C *__restrict__ up_rb, int do_lower, int do_upper, int g_in_smem,
                                               cx<R> *xs, cx<R> *sb, C *sg)
{
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const size_t gstride = (size_t)w * 32;
    const int nb = nblk * w;

    // z_b = T_b^-1 r for lane's row; G_b staged for the correction
    auto solve_block = [&](int blk, cx<R> r, const C *inv, const C *g) {
        const C *ib = inv + (m * nblk + blk) * 1024;
        cx<R> acc[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) acc[a] = mk<R>((R)0, (R)0);
#pragma unroll 1
        for (int q0 = 0; q0 < 32; q0 += 16) {
#pragma unroll
            for (int q = 0; q < 16; ++q) coef_fma(acc[q & 3], tri_ldt<SMEM_TAB>(ib + (q0 + q) * 32 + lane), shfl_cx(r, q0 + q));
        }
        xs[blk * 32 + lane] = (acc[0] + acc[1]) + (acc[2] + acc[3]);
        if (g_in_smem) {
            const C *gb = g + (m * nblk + blk) * gstride;
            for (int c = 0; c < w; ++c) sg[((size_t)blk * w + c) * 32 + lane] = tri_ldt<SMEM_TAB>(gb + c * 32 + lane);
        }
    };
    // s = Rb z[boundary rows]: each warp takes BRW consecutive output rows at a time, lanes
    // over the columns, two 32-column chunks per round so that 2 BRW Rb loads of a lane are in
    // flight together; the block-triangular zero part is skipped by a per-element predicate
    auto boundary = [&](bool lower, const C *rb) {
        constexpr int BRW = 8;
        const C *Rm = rb + m * (size_t)nb * nb;
        const int r0 = lower ? 32 - w : 0;
        for (int row0 = warp * BRW; row0 < nb; row0 += NW * BRW) {
            cx<R> acc[BRW];
#pragma unroll
            for (int q = 0; q < BRW; ++q) acc[q] = mk<R>((R)0, (R)0);
            const int bo_first = row0 / w, bo_last = min(row0 + BRW - 1, nb - 1) / w;
            const int c_lo = lower ? 0 : bo_first * w, c_hi = lower ? (bo_last + 1) * w : nb;
            for (int col0 = c_lo; col0 < c_hi; col0 += 64) {
                const int ca = col0 + lane, cb = col0 + 32 + lane;
                const int bca = ca / w, bcb = cb / w;
                C va[BRW], vb[BRW];
#pragma unroll
                for (int q = 0; q < BRW; ++q) {
                    const int row = row0 + q, bo = row / w;
                    const bool nza = ca < c_hi && row < nb && (lower ? bca <= bo : bca >= bo);
                    const bool nzb = cb < c_hi && row < nb && (lower ? bcb <= bo : bcb >= bo);
                    va[q] = nza ? tri_ldt<SMEM_TAB>(Rm + (size_t)row * nb + ca) : C();
                    vb[q] = nzb ? tri_ldt<SMEM_TAB>(Rm + (size_t)row * nb + cb) : C();
                }
                const cx<R> za = ca < c_hi ? xs[bca * 32 + r0 + (ca - bca * w)] : mk<R>((R)0, (R)0);
                const cx<R> zb = cb < c_hi ? xs[bcb * 32 + r0 + (cb - bcb * w)] : mk<R>((R)0, (R)0);
#pragma unroll
                for (int q = 0; q < BRW; ++q) {
                    coef_fma(acc[q], va[q], za);
                    coef_fma(acc[q], vb[q], zb);
                }
            }
#pragma unroll
            for (int q = 0; q < BRW; ++q) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    acc[q].x += __shfl_xor_sync(0xffffffffu, acc[q].x, o);
                    acc[q].y += __shfl_xor_sync(0xffffffffu, acc[q].y, o);
                }
                if (lane == 0 && row0 + q < nb) sb[row0 + q] = acc[q];
            }
        }
    };
    // y_b = z_b - G_b s (returns the corrected row)
    auto correct = [&](int blk, const C *g, bool lower) -> cx<R> {
        cx<R> y = xs[blk * 32 + lane];
        const int nbk = lower ? blk - 1 : blk + 1;
        if (nbk >= 0 && nbk < nblk) {
            if (g_in_smem) {
                const C *gb = sg + (size_t)blk * gstride;
                for (int c = 0; c < w; ++c) coef_fms(y, gb[c * 32 + lane], sb[nbk * w + c]);
            } else {
                const C *gb = g + (m * nblk + blk) * gstride;
                for (int c = 0; c < w; ++c) coef_fms(y, tri_ldt<SMEM_TAB>(gb + c * 32 + lane), sb[nbk * w + c]);
            }
        }
        return y;
    };

    if (do_lower) {
        for (int blk = warp; blk < nblk; blk += NW) solve_block(blk, xs[blk * 32 + lane], lo_inv, lo_g);
        __syncthreads();
        boundary(true, lo_rb);
        __syncthreads();
        for (int blk = warp; blk < nblk; blk += NW) {
            const cx<R> y = correct(blk, lo_g, true);
            if (do_upper) solve_block(blk, y, up_inv, up_g);  // same rows, same warp
            else xs[blk * 32 + lane] = y;
        }
        __syncthreads();
    } else if (do_upper) {
        for (int blk = warp; blk < nblk; blk += NW) solve_block(blk, xs[blk * 32 + lane], up_inv, up_g);
        __syncthreads();
    }
    if (do_upper) {
        boundary(false, up_rb);
        __syncthreads();
        for (int blk = warp; blk < nblk; blk += NW) {
            const cx<R> y = correct(blk, up_g, false);
            xs[blk * 32 + lane] = y;
        }
        __syncthreads();
    }
}
