// Factorized rank-3 terms: V = sum_q w_q s_slot(q) A_q (x) R_q.
//
// The two-electron repulsion in coupled spherical harmonics is, per angular pair, a sum over
// multipoles l3 of an angular coefficient times the radial function r<^l3 / r>^(l3+1)
// (examples/tensor/helium_stabilization/coupledspherical.cpp:7-127). The reference
// represents the sum per angular pair on SelectionRule_R12 x banded-packed x
// banded-nonhermitian; here each multipole's radial operator R_q is stored once (a band x
// band block on the two radial ranks, real) and the angular coefficients A_q as a sparse
// matrix, so the term costs one radial block per multipole instead of one per angular pair.
//
// One application, after the banded part of the operator has written dst:
//   mix:    Z[q][p][a'] = w_q s_slot(q) sum_a A_q[a'][a] src[a][p]   (p: point of the N1 x N2 grid)
//   radial: dst[a'][i1][i2] += sum_q sum_{d1,d2} R_q[i1][d1][d2][i2] Z[q][i1+d1-k][i2+d2-k][a']
// The scratch Z keeps the channels innermost, so one radial row of Z for a tile of channels
// is a plain 2-D box for the tensor-memory-access unit.
//
// mix: one warp per output channel a' and 32 (FP32: 64) points; only the nonzero (entry,
// factor) pairs are applied, into per-factor accumulators in shared memory; the 4 warps of a
// CTA (4 consecutive channels) then write each point's 4 channels as one 32-byte segment,
// skipping factors none of the 4 channels has (their scratch stays at the zeros written at
// upload).
// radial: a 169-point stencil (k = 6) with coefficients varying per point and shared by all
// channels. A CTA = two radial rows, a tile of tw points of the last rank and CA channels;
// per stage (factor q, input row j1) one TMA box brings the Z rows [tw + 2k][CA] (used by both
// output rows) and one box per output row its coefficient rows [2k+1][tw] into shared memory
// (double-buffered on two mbarriers, bounded waits); each thread keeps PI consecutive points x
// PC channels of accumulators and a sliding window of PI rows of Z in registers. Bound by FP32
// (or FP64) FMA throughput.
#include "pg_internal.cuh"

#include <algorithm>
#include <cmath>
#include <map>

namespace {

const int CB = 4;   // channels per mix CTA (one warp each)

struct FactArgs {
    int Q, Qp, A, Ap, N1, N2, N2p, nct, tw;
    int df;  // FP64 operator with FP32-pair (double-float) scratch and radial factors
    const int *row_ptr, *col, *slot, *nzq, *perm;
    const void *coef;
    const unsigned char *chunk, *bflag;
    const int *seg_ptr, *seg, *pcol;  // segments of the exact-pair mix (FP64 operators)
    const void *pcoef;
    const unsigned char *seg_gq;
    const cxd *w;
    void *Z;
    int *err;
};

FactArgs args_of(const FactDev &f, int *err)
{
    FactArgs a;
    a.Q = f.Q; a.Qp = f.Qp; a.A = f.A; a.Ap = f.Ap; a.N1 = f.N1; a.N2 = f.N2; a.N2p = f.N2p; a.nct = f.nct;
    a.tw = f.tw;
    a.df = f.df;
    a.row_ptr = f.row_ptr; a.col = f.col; a.slot = f.slot; a.nzq = f.nzq; a.perm = f.perm;
    a.coef = f.coef; a.chunk = f.chunk;
    a.seg_ptr = f.seg_ptr; a.seg = f.seg; a.pcol = f.pcol; a.pcoef = f.pcoef; a.seg_gq = f.seg_gq; a.bflag = f.bflag; a.w = f.w; a.Z = f.Z; a.err = err;
    return a;
}

__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void fbar_init(unsigned long long *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fbar_expect(unsigned long long *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool fbar_try(unsigned long long *bar, unsigned parity)
{
    unsigned ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(ok)
                 : "r"(smem_addr(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}
// bounded wait: gives up after 2^26 polls and reports through *err
__device__ __forceinline__ bool fbar_wait(unsigned long long *bar, unsigned parity, int *err)
{
    for (long long it = 0; it < (1LL << 26); ++it)
        if (fbar_try(bar, parity)) return true;
    if (err) atomicExch(err, 1);
    return false;
}
__device__ __forceinline__ void tma_2d(void *dst, const CUtensorMap *map, int c0, int c1, unsigned long long *bar)
{
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n"
                 ::"r"(smem_addr(dst)), "l"(map), "r"(c0), "r"(c1), "r"(smem_addr(bar))
                 : "memory");
}
__device__ __forceinline__ void tma_3d(void *dst, const CUtensorMap *map, int c0, int c1, int c2,
                                       unsigned long long *bar)
{
    asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n"
                 ::"r"(smem_addr(dst)), "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_addr(bar))
                 : "memory");
}

template <typename R>
__device__ __forceinline__ cx<R> ldg_cx(const cx<R> *p)
{
    if constexpr (sizeof(R) == 4) {
        const float2 v = __ldg(reinterpret_cast<const float2 *>(p));
        return mk<R>(v.x, v.y);
    } else {
        const double2 v = __ldg(reinterpret_cast<const double2 *>(p));
        return mk<R>(v.x, v.y);
    }
}

// Z[q][p][a] = w_q s_slot(q) / inv_scale * sum_e coef_e[q] x[col_e][p]. CTA = CB warps (scratch
// slots a0 .. a0+CB, blockIdx.x) x 32 MPT points (blockIdx.y; MPT consecutive points per lane,
// 16-byte source loads).
// The factors are taken MQC at a time with their sums in registers: each angular entry (a, col)
// whose factor range meets the chunk loads its source points once and applies its MQC
// coefficients (16-byte loads, the same for the whole warp). Factors are ordered so that an
// entry's nonzero factors are contiguous (the repulsion's multipoles by parity), which keeps the
// zero coefficients inside a chunk few. The chunk's sums go through shared memory
// [MQC][MPT][32][CB + 1] so that the CTA writes the CB slots of each point as one contiguous
// segment (lanes = 8 points x 4 slots); chunks that no slot of the group has are skipped (their
// scratch stays at the zeros written at upload).
template <typename R> struct MixTile;
template <> struct MixTile<float> { static const int MPT = 4, MQC = 8; };
template <> struct MixTile<double> { static const int MPT = 2, MQC = 8; };
const int MIX_QC = 8;  // == MixTile<R>::MQC: the padding of the coefficient rows

// M consecutive coefficients from a 16-byte aligned row (M a multiple of 16 bytes / sizeof(R))
template <typename R, int M>
__device__ __forceinline__ void load_coefs_row(const R *p, R (&c)[M])
{
    if constexpr (sizeof(R) == 4) {
#pragma unroll
        for (int h = 0; h < M / 4; ++h) {
            const float4 v = __ldg(reinterpret_cast<const float4 *>(p) + h);
            c[4 * h] = v.x; c[4 * h + 1] = v.y; c[4 * h + 2] = v.z; c[4 * h + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int h = 0; h < M / 2; ++h) {
            const double2 v = __ldg(reinterpret_cast<const double2 *>(p) + h);
            c[2 * h] = v.x;
            c[2 * h + 1] = v.y;
        }
    }
}

template <typename R>
__global__ void __launch_bounds__(32 * CB) fact_mix_kernel(FactArgs f, pg_scales scales,
                                                          const cxd *__restrict__ scales_dev,
                                                          const cx<R> *__restrict__ x,
                                                          const double *__restrict__ inv_scale)
{
    constexpr int MPT = MixTile<R>::MPT, MQC = MixTile<R>::MQC, TP = 32 * MPT;
    static_assert(MIX_QC % MQC == 0, "chunks divide the coefficient padding");
    extern __shared__ __align__(16) unsigned char mix_smem[];
    cx<R> *acc_s = reinterpret_cast<cx<R> *>(mix_smem);  // [MQC][MPT][32][CB + 1]
    cx<R> *ws = acc_s + (size_t)MQC * TP * (CB + 1);      // [Q] factor scales
    const int lane = threadIdx.x & 31, wrp = threadIdx.x >> 5;
    const int Q = f.Q, nch = f.Qp / MQC, nflag = f.Qp / MIX_QC;
    const int a0 = blockIdx.x * CB;                      // first scratch slot of the group
    const int a = a0 + wrp < f.A ? f.perm[a0 + wrp] : -1;  // channel of this warp's slot
    const long long NP = (long long)f.N1 * f.N2;
    const long long pbase = (long long)blockIdx.y * TP;
    const long long p0 = pbase + (long long)lane * MPT;  // this lane's first point
    const bool vec = (NP % 2) == 0;                      // rows start 16-byte aligned
    const double sc = inv_scale ? 1.0 / *inv_scale : 1.0;
    for (int q = threadIdx.x; q < Q; q += 32 * CB) {
        const cxd s = scales_dev ? scales_dev[f.slot[q]] : scales.s[f.slot[q]];
        ws[q] = cvt<R>(sc * (f.w[q] * s));
    }
    const int4 *__restrict__ meta = (const int4 *)f.col;  // col, first and last nonzero factor
    const R *__restrict__ coef = (const R *)f.coef;        // [entry][Qp]
    const unsigned char *gf = f.chunk + (size_t)blockIdx.x * nflag;  // chunks of 8 touched by the group
    cx<R> *__restrict__ Z = (cx<R> *)f.Z;
    const int e_begin = a >= 0 ? f.row_ptr[a] : 0, e_end = a >= 0 ? f.row_ptr[a + 1] : 0;
    auto load_x = [&](int col, cx<R> (&v)[MPT]) {
        const cx<R> *xr = x + (size_t)col * NP + p0;
        if (vec && p0 + MPT <= NP) {
            if constexpr (sizeof(R) == 4) {
#pragma unroll
                for (int h = 0; h < MPT / 2; ++h) {
                    const float4 t = __ldg(reinterpret_cast<const float4 *>(xr) + h);
                    v[2 * h] = mk<R>(t.x, t.y);
                    v[2 * h + 1] = mk<R>(t.z, t.w);
                }
            } else {
#pragma unroll
                for (int h = 0; h < MPT; ++h) {
                    const double2 t = __ldg(reinterpret_cast<const double2 *>(xr) + h);
                    v[h] = mk<R>(t.x, t.y);
                }
            }
        } else {
#pragma unroll
            for (int u = 0; u < MPT; ++u) v[u] = p0 + u < NP ? xr[u] : mk<R>((R)0, (R)0);
        }
    };
    __syncthreads();  // factor scales ready
    for (int k = 0; k < nch; ++k) {
        const int q0 = k * MQC;
        if (!gf[q0 / MIX_QC]) continue;  // CTA-uniform
        cx<R> acc[MQC][MPT];
#pragma unroll
        for (int j = 0; j < MQC; ++j)
#pragma unroll
            for (int u = 0; u < MPT; ++u) acc[j][u] = mk<R>((R)0, (R)0);
        for (int e = e_begin; e < e_end; ++e) {
            const int4 m = meta[e];
            if (m.z < q0 || m.y >= q0 + MQC) continue;
            cx<R> xv[MPT];
            load_x(m.x, xv);
            R c[MQC];
            load_coefs_row<R, MQC>(coef + (size_t)e * f.Qp + q0, c);
#pragma unroll
            for (int j = 0; j < MQC; ++j)
#pragma unroll
                for (int u = 0; u < MPT; ++u) {
                    acc[j][u].x = fma(c[j], xv[u].x, acc[j][u].x);
                    acc[j][u].y = fma(c[j], xv[u].y, acc[j][u].y);
                }
        }
#pragma unroll
        for (int j = 0; j < MQC; ++j)
#pragma unroll
            for (int u = 0; u < MPT; ++u) acc_s[(((size_t)j * MPT + u) * 32 + lane) * (CB + 1) + wrp] = acc[j][u];
        __syncthreads();
        for (int t = threadIdx.x; t < MQC * TP * CB; t += 32 * CB) {
            const int r = t % CB, rest = t / CB;
            const int pl = rest % TP, j = rest / TP;
            const int q = q0 + j;
            const long long pp = pbase + pl;
            if (q >= Q || pp >= NP) continue;
            const int u = pl % MPT, ln = pl / MPT;
            const cx<R> v = ws[q] * acc_s[(((size_t)j * MPT + u) * 32 + ln) * (CB + 1) + r];
            const size_t zi = ((size_t)q * NP + pp) * f.Ap + a0 + r;
            if constexpr (sizeof(R) == 8) {
                if (f.df) {  // the 16 bytes hold (re_hi, re_lo, im_hi, im_lo)
                    const float rh = (float)v.x, ih = (float)v.y;
                    reinterpret_cast<float4 *>(Z)[zi] = make_float4(rh, (float)(v.x - (double)rh), ih, (float)(v.y - (double)ih));
                    continue;
                }
            }
            Z[zi] = v;
        }
        __syncthreads();
    }
}

template <typename R>
size_t mix_smem_bytes(int Q)
{
    return ((size_t)MixTile<R>::MQC * 32 * MixTile<R>::MPT * (CB + 1) + Q) * sizeof(cx<R>);
}

// The mix over the exact nonzero (channel, factor) pairs, for the FP64 operator (whose FMAs are
// the bottleneck there, so the zero coefficients inside the chunks of fact_mix_kernel cost more
// than the repeated source loads): each channel's pairs grouped by factor (segments, in factor
// order), a factor's sum in registers (four independent load chains), the factors through
// shared memory [MQC][MPT][32][CB + 1] MQC at a time, the CB slots of each point written as one
// segment (lanes = 8 points x 4 slots); factors no slot of the group has are skipped.
template <typename R> struct SegTile;
template <> struct SegTile<float> { static const int MPT = 4, MQC = 8; };
template <> struct SegTile<double> { static const int MPT = 2, MQC = 8; };

template <typename R>
__global__ void __launch_bounds__(32 * CB) fact_mix_seg_kernel(FactArgs f, pg_scales scales,
                                                          const cxd *__restrict__ scales_dev,
                                                          const cx<R> *__restrict__ x,
                                                          const double *__restrict__ inv_scale)
{
    constexpr int MPT = SegTile<R>::MPT, MQC = SegTile<R>::MQC, TP = 32 * MPT;
    extern __shared__ __align__(16) unsigned char mix_smem[];
    cx<R> *acc = reinterpret_cast<cx<R> *>(mix_smem);  // [MQC][MPT][32][CB + 1]
    cx<R> *ws = acc + (size_t)MQC * TP * (CB + 1);      // [Q] factor scales
    const int lane = threadIdx.x & 31, wrp = threadIdx.x >> 5;
    const int Q = f.Q;
    const int a0 = blockIdx.x * CB;                      // first scratch slot of the group
    const int a = a0 + wrp < f.A ? f.perm[a0 + wrp] : -1;  // channel of this warp's slot
    const long long NP = (long long)f.N1 * f.N2;
    const long long pbase = (long long)blockIdx.y * TP;
    const long long p0 = pbase + (long long)lane * MPT;  // this lane's first point
    const bool vec = (NP % 2) == 0;                      // rows start 16-byte aligned
    const double sc = inv_scale ? 1.0 / *inv_scale : 1.0;
    for (int q = threadIdx.x; q < Q; q += 32 * CB) {
        const cxd s = scales_dev ? scales_dev[f.slot[q]] : scales.s[f.slot[q]];
        ws[q] = cvt<R>(sc * (f.w[q] * s));
    }
    const int4 *__restrict__ seg = (const int4 *)f.seg;  // factor, first pair, last+1 pair
    const int *__restrict__ pcol = f.pcol;
    const R *__restrict__ pc = (const R *)f.pcoef;
    const unsigned char *gf = f.seg_gq + (size_t)blockIdx.x * Q;  // factors touched by this group
    cx<R> *__restrict__ Z = (cx<R> *)f.Z;
    int g = a >= 0 ? f.seg_ptr[a] : 0;
    const int g_end = a >= 0 ? f.seg_ptr[a + 1] : 0;
    auto load_x = [&](int col, cx<R> (&v)[MPT]) {
        const cx<R> *xr = x + (size_t)col * NP + p0;
        if (vec && p0 + MPT <= NP) {
            if constexpr (sizeof(R) == 4) {
#pragma unroll
                for (int h = 0; h < MPT / 2; ++h) {
                    const float4 t = __ldg(reinterpret_cast<const float4 *>(xr) + h);
                    v[2 * h] = mk<R>(t.x, t.y);
                    v[2 * h + 1] = mk<R>(t.z, t.w);
                }
            } else {
#pragma unroll
                for (int h = 0; h < MPT; ++h) {
                    const double2 t = __ldg(reinterpret_cast<const double2 *>(xr) + h);
                    v[h] = mk<R>(t.x, t.y);
                }
            }
        } else {
#pragma unroll
            for (int u = 0; u < MPT; ++u) v[u] = p0 + u < NP ? xr[u] : mk<R>((R)0, (R)0);
        }
    };
    for (int qc = 0; qc < Q; qc += MQC) {
        bool any = false;
        for (int j = 0; j < MQC && qc + j < Q; ++j) any |= gf[qc + j] != 0;
        if (!any) continue;  // CTA-uniform
        for (int j = 0; j < MQC; ++j)
#pragma unroll
            for (int u = 0; u < MPT; ++u)
                acc[(((size_t)j * MPT + u) * 32 + lane) * (CB + 1) + wrp] = mk<R>((R)0, (R)0);
        for (; g < g_end; ++g) {
            const int4 sg = seg[g];
            if (sg.x >= qc + MQC) break;  // segments are in factor order
            constexpr int CH = 4;  // independent chains: four source loads in flight per lane
            cx<R> sum[CH][MPT];
#pragma unroll
            for (int h = 0; h < CH; ++h)
#pragma unroll
                for (int u = 0; u < MPT; ++u) sum[h][u] = mk<R>((R)0, (R)0);
            int z = sg.y;
            for (; z + CH - 1 < sg.z; z += CH) {
                cx<R> xv[CH][MPT];
#pragma unroll
                for (int h = 0; h < CH; ++h) load_x(pcol[z + h], xv[h]);
#pragma unroll
                for (int h = 0; h < CH; ++h) {
                    const R c = pc[z + h];
#pragma unroll
                    for (int u = 0; u < MPT; ++u) {
                        sum[h][u].x = fma(c, xv[h][u].x, sum[h][u].x);
                        sum[h][u].y = fma(c, xv[h][u].y, sum[h][u].y);
                    }
                }
            }
            for (; z < sg.z; ++z) {
                cx<R> x0[MPT];
                load_x(pcol[z], x0);
                const R c = pc[z];
#pragma unroll
                for (int u = 0; u < MPT; ++u) {
                    sum[0][u].x = fma(c, x0[u].x, sum[0][u].x);
                    sum[0][u].y = fma(c, x0[u].y, sum[0][u].y);
                }
            }
#pragma unroll
            for (int u = 0; u < MPT; ++u)
                acc[(((size_t)(sg.x - qc) * MPT + u) * 32 + lane) * (CB + 1) + wrp] =
                    (sum[0][u] + sum[1][u]) + (sum[2][u] + sum[3][u]);
        }
        __syncthreads();
        for (int t = threadIdx.x; t < MQC * TP * CB; t += 32 * CB) {
            const int r = t % CB, rest = t / CB;
            const int pl = rest % TP, j = rest / TP;
            const int q = qc + j;
            const long long pp = pbase + pl;
            if (q >= Q || !gf[q] || pp >= NP) continue;
            const int u = pl % MPT, ln = pl / MPT;
            const cx<R> v = ws[q] * acc[(((size_t)j * MPT + u) * 32 + ln) * (CB + 1) + r];
            const size_t zi = ((size_t)q * NP + pp) * f.Ap + a0 + r;
            if constexpr (sizeof(R) == 8) {
                if (f.df) {  // the 16 bytes hold (re_hi, re_lo, im_hi, im_lo)
                    const float rh = (float)v.x, ih = (float)v.y;
                    reinterpret_cast<float4 *>(Z)[zi] = make_float4(rh, (float)(v.x - (double)rh), ih, (float)(v.y - (double)ih));
                    continue;
                }
            }
            Z[zi] = v;
        }
        __syncthreads();
    }
}

template <typename R>
size_t seg_smem_bytes(int Q)
{
    return ((size_t)SegTile<R>::MQC * 32 * SegTile<R>::MPT * (CB + 1) + Q) * sizeof(cx<R>);
}


// tile shapes per precision: PI points x NV 16-byte vectors of channels per thread, 8 channel
// lanes, CA = 8 x NV x (complex per vector) channels per CTA
template <typename R> struct RadialTile;
template <> struct RadialTile<float> { static const int PI = 8, NV = 2, PCV = 2, TCN = 8, CA = 32; };
template <> struct RadialTile<double> { static const int PI = 4, NV = 2, PCV = 1, TCN = 8, CA = 16; };

template <typename R>
__host__ __device__ inline size_t rad_round128(size_t b) { return (b + 127) & ~(size_t)127; }

// bytes of one stage's Z box and coefficient box
template <typename R>
__host__ __device__ inline size_t rad_zbytes(int tw, int kb)
{
    return (size_t)(tw + 2 * kb) * RadialTile<R>::CA * sizeof(cx<R>);
}
template <typename R>
__host__ __device__ inline size_t rad_rbytes(int tw, int kb)
{
    return (size_t)(2 * kb + 1) * tw * sizeof(R);
}

// rows of the first radial rank per radial-stencil CTA (they share each staged row of Z)
const int RB = 2;

// One CTA = radial rows i1_0 .. i1_0 + RB (blockIdx.x), tw points of the last rank
// (blockIdx.y), CA channels (blockIdx.z); thread = (row rr, PI consecutive points, NV vectors of
// channels). blockDim = RB x tw / PI x 8. A stage is (factor q, input row j1): one TMA box of Z
// row j1 serves both output rows, each with its own box of coefficients R_q[i1][j1 - i1 + k].
template <typename R, int KB>
__global__ void __launch_bounds__(256, 1) fact_radial_kernel(FactArgs f, cx<R> *__restrict__ y,
                                                             const __grid_constant__ CUtensorMap zmap,
                                                             const __grid_constant__ CUtensorMap rmap)
{
    typedef RadialTile<R> T;
    constexpr int B = 2 * KB + 1;
    constexpr int PI = T::PI, NV = T::NV, PCV = T::PCV, TCN = T::TCN, CA = T::CA, PC = NV * PCV;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned long long *bar = (unsigned long long *)smem_raw;
    const int tw = f.tw;
    const unsigned zbytes = (unsigned)rad_zbytes<R>(tw, KB), rbytes = (unsigned)rad_rbytes<R>(tw, KB);
    const size_t zb = rad_round128<R>(zbytes), rb = rad_round128<R>(rbytes), stage = zb + RB * rb;
    unsigned char *buf = smem_raw + 128;
    const int per_row = (tw / PI) * TCN;
    const int tid = threadIdx.x, rr = tid / per_row, lt = tid - rr * per_row;
    const int tc = lt % TCN, ti = lt / TCN;
    const int i1b = blockIdx.x * RB, t0 = blockIdx.y * tw, ct = blockIdx.z, c0 = ct * CA;
    const int i1 = i1b + rr;
    const int N1 = f.N1, N2 = f.N2;
    if (tid == 0) {
        fbar_init(&bar[0], 1);
        fbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    // stages (q, j1): factors with a nonzero row in this channel tile, input rows of the grid
    // within k of one of the CTA's output rows
    const int jlo = max(0, i1b - KB), jhi = min(N1 - 1, min(N1 - 1, i1b + RB - 1) + KB);
    auto advance = [&](int &q, int &j1) {
        for (;;) {
            if (++j1 > jhi) {
                j1 = jlo;
                ++q;
            }
            if (q >= f.Q) return;
            if (!f.bflag[(size_t)q * f.nct + ct]) {
                j1 = jhi;
                continue;
            }
            return;
        }
    };
    auto issue = [&](int s, int q, int j1) {
        unsigned char *dst = buf + (size_t)s * stage;
        unsigned bytes = zbytes;
        for (int r = 0; r < RB; ++r) {
            const int d1 = j1 - (i1b + r) + KB;
            if (i1b + r < N1 && d1 >= 0 && d1 < B) bytes += rbytes;
        }
        fbar_expect(&bar[s], bytes);
        tma_3d(dst, &zmap, 2 * c0, t0 - KB, q * N1 + j1, &bar[s]);
        for (int r = 0; r < RB; ++r) {
            const int d1 = j1 - (i1b + r) + KB;
            if (i1b + r < N1 && d1 >= 0 && d1 < B)
                tma_2d(dst + zb + r * rb, &rmap, t0, ((q * N1 + i1b + r) * B + d1) * B, &bar[s]);
        }
    };
    cx<R> acc[PI][PC];
#pragma unroll
    for (int p = 0; p < PI; ++p)
#pragma unroll
        for (int c = 0; c < PC; ++c) acc[p][c] = mk<R>((R)0, (R)0);
    int q = 0, j1 = jlo - 1;
    advance(q, j1);
    if (tid == 0 && q < f.Q) issue(0, q, j1);
    for (int k = 0; q < f.Q; ++k) {
        const int s = k & 1;
        int qn = q, jn = j1;
        advance(qn, jn);
        // the other buffer was released by the barrier at the end of the previous stage
        if (tid == 0 && qn < f.Q) issue(s ^ 1, qn, jn);
        const unsigned parity = (unsigned)(k >> 1) & 1u;
        const bool ok = fbar_wait(&bar[s], parity, f.err);
        if (__syncthreads_or(ok ? 0 : 1)) {
            // a wait ran out: let the copies in flight land (bounded), then leave
            if (!ok) fbar_wait(&bar[s], parity, f.err);
            if (tid == 0 && qn < f.Q) fbar_wait(&bar[s ^ 1], (unsigned)((k + 1) >> 1) & 1u, f.err);
            return;
        }
        const int d1 = j1 - i1 + KB;
        if (i1 < N1 && d1 >= 0 && d1 < B) {
            const cx<R> *zs = (const cx<R> *)(buf + (size_t)s * stage);
            const R *rs = (const R *)(buf + (size_t)s * stage + zb + rr * rb);
            cx<R> win[PI + B - 1][PC];
            auto load_row = [&](int j, cx<R> (&out)[PC]) {
#pragma unroll
                for (int h = 0; h < NV; ++h) {
                    const cx<R> *src = zs + (size_t)j * CA + (h * TCN + tc) * PCV;
                    if constexpr (sizeof(R) == 4) {
                        const float4 v = *reinterpret_cast<const float4 *>(src);
                        out[h * PCV] = mk<R>(v.x, v.y);
                        out[h * PCV + 1] = mk<R>(v.z, v.w);
                    } else {
                        out[h * PCV] = src[0];
                    }
                }
            };
#pragma unroll
            for (int r = 0; r < PI - 1; ++r) load_row(ti * PI + r, win[r]);
#pragma unroll
            for (int d2 = 0; d2 < B; ++d2) {
                load_row(ti * PI + d2 + PI - 1, win[d2 + PI - 1]);
                R rv[PI];
                const R *rp = rs + d2 * tw + ti * PI;
                if constexpr (sizeof(R) == 4) {
#pragma unroll
                    for (int h = 0; h < PI / 4; ++h) {
                        const float4 v = reinterpret_cast<const float4 *>(rp)[h];
                        rv[4 * h] = v.x; rv[4 * h + 1] = v.y; rv[4 * h + 2] = v.z; rv[4 * h + 3] = v.w;
                    }
                } else {
#pragma unroll
                    for (int h = 0; h < PI / 2; ++h) {
                        const double2 v = reinterpret_cast<const double2 *>(rp)[h];
                        rv[2 * h] = v.x; rv[2 * h + 1] = v.y;
                    }
                }
#pragma unroll
                for (int p = 0; p < PI; ++p)
#pragma unroll
                    for (int c = 0; c < PC; ++c) {
                        acc[p][c].x = fma(rv[p], win[p + d2][c].x, acc[p][c].x);
                        acc[p][c].y = fma(rv[p], win[p + d2][c].y, acc[p][c].y);
                    }
            }
        }
        __syncthreads();  // buffer s is free for the stage after next
        q = qn;
        j1 = jn;
    }
    if (i1 >= N1) return;
    const long long NP = (long long)N1 * N2;
#pragma unroll
    for (int h = 0; h < NV; ++h)
#pragma unroll
        for (int v = 0; v < PCV; ++v) {
            const int sl = c0 + (h * TCN + tc) * PCV + v;  // scratch slot -> channel
            if (sl >= f.A) continue;
            cx<R> *__restrict__ yr = y + (size_t)f.perm[sl] * NP + (size_t)i1 * N2;
#pragma unroll
            for (int p = 0; p < PI; ++p) {
                const int i2 = t0 + ti * PI + p;
                if (i2 < N2) yr[i2] = yr[i2] + acc[p][h * PCV + v];
            }
        }
}

// Double-float accumulation for the FP64 operator (FP64 arithmetic runs at a small fraction of
// the FP32 rate on this GPU): a value v is held as hi + lo, hi = fp32(v), lo = fp32(v - hi).
// Each product r * z is formed exactly in its leading part (p = rh zh, the rounding error of p
// by one FMA) plus the cross terms rh zl + rl zh; p is added to the running hi with an
// error-free two-sum (Knuth), the errors gather in lo. Relative accuracy about 2^-48 per sum
// instead of 2^-53.
// (the _rn intrinsics keep the compiler from contracting these steps into FMAs, which would
// break the error-free transformations)
__device__ __forceinline__ void df_fma(float &hi, float &lo, float rh, float rl, float zh, float zl)
{
    const float p = __fmul_rn(rh, zh);
    float e = fmaf(rh, zh, -p);
    e = fmaf(rh, zl, e);
    e = fmaf(rl, zh, e);
    const float s = __fadd_rn(hi, p);
    const float bb = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(err, e));
}

// The radial stencil of the FP64 operator in double-float arithmetic: the tiles of the FP64
// kernel (scratch elements and coefficients of 16 and 8 bytes: (re_hi, re_lo, im_hi, im_lo) and
// (hi, lo)), the same TMA boxes and stages.
template <int KB>
__global__ void __launch_bounds__(128, 2) fact_radial_df_kernel(FactArgs f, cxd *__restrict__ y,
                                                                const __grid_constant__ CUtensorMap zmap,
                                                                const __grid_constant__ CUtensorMap rmap)
{
    typedef RadialTile<double> T;
    constexpr int B = 2 * KB + 1;
    constexpr int PI = T::PI, NV = T::NV, TCN = T::TCN, CA = T::CA, PC = NV;  // one complex per 16 bytes
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned long long *bar = (unsigned long long *)smem_raw;
    const int tw = f.tw;
    const unsigned zbytes = (unsigned)rad_zbytes<double>(tw, KB), rbytes = (unsigned)rad_rbytes<double>(tw, KB);
    const size_t zb = rad_round128<double>(zbytes), stage = zb + rad_round128<double>(rbytes);
    unsigned char *buf = smem_raw + 128;
    const int tid = threadIdx.x, tc = tid % TCN, ti = tid / TCN;
    const int i1 = blockIdx.x, t0 = blockIdx.y * tw, ct = blockIdx.z, c0 = ct * CA;
    const int N1 = f.N1, N2 = f.N2;
    if (tid == 0) {
        fbar_init(&bar[0], 1);
        fbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    auto advance = [&](int &q, int &d1) {
        for (;;) {
            if (++d1 == B) {
                d1 = 0;
                ++q;
            }
            if (q >= f.Q) return;
            if (!f.bflag[(size_t)q * f.nct + ct]) {
                d1 = B - 1;
                continue;
            }
            const int j1 = i1 + d1 - KB;
            if (j1 >= 0 && j1 < N1) return;
        }
    };
    auto issue = [&](int s, int q, int d1) {
        unsigned char *dst = buf + (size_t)s * stage;
        fbar_expect(&bar[s], zbytes + rbytes);
        tma_3d(dst, &zmap, 2 * c0, t0 - KB, q * N1 + i1 + d1 - KB, &bar[s]);
        tma_2d(dst + zb, &rmap, t0, ((q * N1 + i1) * B + d1) * B, &bar[s]);
    };
    float ah[PI][PC][2], al[PI][PC][2];  // [point][channel][re, im]
#pragma unroll
    for (int p = 0; p < PI; ++p)
#pragma unroll
        for (int c = 0; c < PC; ++c) ah[p][c][0] = ah[p][c][1] = al[p][c][0] = al[p][c][1] = 0.f;
    int q = 0, d1 = -1;
    advance(q, d1);
    if (tid == 0 && q < f.Q) issue(0, q, d1);
    for (int k = 0; q < f.Q; ++k) {
        const int s = k & 1;
        int qn = q, dn = d1;
        advance(qn, dn);
        if (tid == 0 && qn < f.Q) issue(s ^ 1, qn, dn);
        const unsigned parity = (unsigned)(k >> 1) & 1u;
        const bool ok = fbar_wait(&bar[s], parity, f.err);
        if (__syncthreads_or(ok ? 0 : 1)) {
            if (!ok) fbar_wait(&bar[s], parity, f.err);
            if (tid == 0 && qn < f.Q) fbar_wait(&bar[s ^ 1], (unsigned)((k + 1) >> 1) & 1u, f.err);
            return;
        }
        const float4 *zs = (const float4 *)(buf + (size_t)s * stage);
        const float2 *rs = (const float2 *)(buf + (size_t)s * stage + zb);
        float4 win[PI + B - 1][PC];
#pragma unroll
        for (int r = 0; r < PI - 1; ++r)
#pragma unroll
            for (int h = 0; h < NV; ++h) win[r][h] = zs[(size_t)(ti * PI + r) * CA + h * TCN + tc];
#pragma unroll
        for (int d2 = 0; d2 < B; ++d2) {
#pragma unroll
            for (int h = 0; h < NV; ++h) win[d2 + PI - 1][h] = zs[(size_t)(ti * PI + d2 + PI - 1) * CA + h * TCN + tc];
            float2 rv[PI];
#pragma unroll
            for (int p = 0; p < PI; ++p) rv[p] = rs[d2 * tw + ti * PI + p];
#pragma unroll
            for (int p = 0; p < PI; ++p)
#pragma unroll
                for (int c = 0; c < PC; ++c) {
                    const float4 z = win[p + d2][c];
                    df_fma(ah[p][c][0], al[p][c][0], rv[p].x, rv[p].y, z.x, z.y);
                    df_fma(ah[p][c][1], al[p][c][1], rv[p].x, rv[p].y, z.z, z.w);
                }
        }
        __syncthreads();
        q = qn;
        d1 = dn;
    }
    const long long NP = (long long)N1 * N2;
#pragma unroll
    for (int h = 0; h < NV; ++h) {
        const int sl = c0 + h * TCN + tc;
        if (sl >= f.A) continue;
        cxd *__restrict__ yr = y + (size_t)f.perm[sl] * NP + (size_t)i1 * N2;
#pragma unroll
        for (int p = 0; p < PI; ++p) {
            const int i2 = t0 + ti * PI + p;
            if (i2 < N2)
                yr[i2] = yr[i2] + mk<double>((double)ah[p][h][0] + (double)al[p][h][0],
                                             (double)ah[p][h][1] + (double)al[p][h][1]);
        }
    }
}

template <typename R>
int launch_factored(pg_op *op, const pg_scales &scales, const cxd *scales_dev, const void *src, void *dst,
                    const double *inv_scale)
{
    typedef RadialTile<R> T;
    const FactDev &fd = op->fact;
    const FactArgs fa = args_of(fd, op->ctx->d_err);
    cudaStream_t s = op->ctx->stream;
    const long long NP = (long long)fd.N1 * fd.N2;
    const int TP = 32 * MixTile<R>::MPT;
    // channel groups fastest: the CTAs running together share a point tile of the source (L2)
    dim3 g1((unsigned)((fd.A + CB - 1) / CB), (unsigned)((NP + TP - 1) / TP));
    if constexpr (sizeof(R) == 8) {
        const int TPs = 32 * SegTile<R>::MPT;
        dim3 gs((unsigned)((fd.A + CB - 1) / CB), (unsigned)((NP + TPs - 1) / TPs));
        fact_mix_seg_kernel<R><<<gs, 32 * CB, seg_smem_bytes<R>(fd.Q), s>>>(fa, scales, scales_dev,
                                                                            (const cx<R> *)src, inv_scale);
    } else {
        fact_mix_kernel<R><<<g1, 32 * CB, mix_smem_bytes<R>(fd.Q), s>>>(fa, scales, scales_dev, (const cx<R> *)src,
                                                                         inv_scale);
    }
    op->ctx->launches++;
    PG_TRY(pg_check_launch(op->ctx));
    dim3 g2((unsigned)fd.N1, (unsigned)fd.ntiles, (unsigned)fd.nct);
    const int nt = fd.tw / T::PI * T::TCN;
    dim3 g2r((unsigned)((fd.N1 + RB - 1) / RB), (unsigned)fd.ntiles, (unsigned)fd.nct);
    if (op->kb != 6) return PG_ERR_STORAGE;
    if constexpr (sizeof(R) == 8) {
        if (fd.df) {
            fact_radial_df_kernel<6><<<g2, nt, fd.radial_smem, s>>>(fa, (cxd *)dst, fd.zmap, fd.rmap);
            op->ctx->launches++;
            return pg_check_launch(op->ctx);
        }
    }
    fact_radial_kernel<R, 6><<<g2r, RB * nt, fd.radial_smem, s>>>(fa, (cx<R> *)dst, fd.zmap, fd.rmap);
    op->ctx->launches++;
    return pg_check_launch(op->ctx);
}

}  // namespace

int pg_factored_apply(pg_op *op, const pg_scales &scales, const cxd *scales_dev, const void *src, void *dst,
                      const double *src_inv_scale_dev)
{
    if (op->fact.Q == 0) return PG_OK;
    return op->precision == PG_FP64 ? launch_factored<double>(op, scales, scales_dev, src, dst, src_inv_scale_dev)
                                    : launch_factored<float>(op, scales, scales_dev, src, dst, src_inv_scale_dev);
}

void pg_factored_free(pg_op *op)
{
    FactDev &f = op->fact;
    cudaFree(f.row_ptr); cudaFree(f.col); cudaFree(f.nzq); cudaFree(f.slot); cudaFree(f.perm);
    cudaFree(f.coef); cudaFree(f.seg_ptr); cudaFree(f.seg); cudaFree(f.pcol); cudaFree(f.pcoef); cudaFree(f.seg_gq);
    cudaFree(f.chunk); cudaFree(f.bflag); cudaFree(f.radial); cudaFree(f.w); cudaFree(f.Z);
    f = FactDev();
}

extern "C" int pg_op_add_factored(pg_op *op, int nfactors, const double *radial, const double *weights,
                                  const int *slots, long long nentries, const int *ent_factor, const int *ent_row,
                                  const int *ent_col, const double *ent_coef)
{
    if (!op || nfactors < 0 || nentries < 0) return PG_ERR_ARG;
    if (op->finalized) return PG_ERR_STATE;
    if (op->rank != 3) return PG_ERR_STORAGE;
    if (nfactors == 0) return PG_OK;
    if (!radial || !weights || !slots || (nentries > 0 && (!ent_factor || !ent_row || !ent_col || !ent_coef)))
        return PG_ERR_ARG;
    if (op->kb != 6) return PG_ERR_STORAGE;  // the radial stencil is compiled for 13 diagonals
    const int A = op->shape[0], N1 = op->shape[1], N2 = op->shape[2], b = op->b;
    if (N1 <= 2 * op->kb) return PG_ERR_SHAPE;
    if ((long long)N1 * N2 > 65535LL * 64) return PG_ERR_SHAPE;  // point tiles of the mix kernel in grid y
    if (op->factors.size() + nfactors > (size_t)4096) return PG_ERR_ARG;
    for (int q = 0; q < nfactors; ++q)
        if (slots[q] < 0 || slots[q] >= PG_MAX_SLOTS) return PG_ERR_ARG;
    for (long long e = 0; e < nentries; ++e)
        if (ent_factor[e] < 0 || ent_factor[e] >= nfactors || ent_row[e] < 0 || ent_row[e] >= A || ent_col[e] < 0 ||
            ent_col[e] >= A)
            return PG_ERR_SHAPE;
    const size_t rsz = (size_t)N1 * b * b * N2;
    const size_t first = op->factors.size();
    for (int q = 0; q < nfactors; ++q) {
        HostFactor h;
        h.radial.assign(radial + rsz * q, radial + rsz * (q + 1));
        h.w[0] = weights[2 * q];
        h.w[1] = weights[2 * q + 1];
        h.slot = slots[q];
        op->factors.push_back(std::move(h));
    }
    for (long long e = 0; e < nentries; ++e) {
        HostFactor &h = op->factors[first + ent_factor[e]];
        h.row.push_back(ent_row[e]);
        h.col.push_back(ent_col[e]);
        h.coef.push_back(ent_coef[e]);
    }
    return PG_OK;
}

template <typename R>
static int upload_real(void **dst, const std::vector<double> &src)
{
    std::vector<R> tmp(src.size());
    for (size_t k = 0; k < src.size(); ++k) tmp[k] = (R)src[k];
    PG_CUDA_TRY(cudaMalloc(dst, std::max<size_t>(1, tmp.size()) * sizeof(R)));
    if (!tmp.empty()) PG_CUDA_TRY(cudaMemcpy(*dst, tmp.data(), tmp.size() * sizeof(R), cudaMemcpyHostToDevice));
    return PG_OK;
}

template <typename T>
static int upload_vec(T **dst, const std::vector<T> &src)
{
    PG_CUDA_TRY(cudaMalloc((void **)dst, std::max<size_t>(1, src.size()) * sizeof(T)));
    if (!src.empty()) PG_CUDA_TRY(cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
    return PG_OK;
}

int pg_factored_finalize(pg_op *op)
{
    if (op->factors.empty()) return PG_OK;
    FactDev &f = op->fact;
    const int A = op->shape[0], N1 = op->shape[1], N2 = op->shape[2], b = op->b, kb = op->kb;
    const bool fp64 = op->precision == PG_FP64;
    const int Q = (int)op->factors.size();
    f.A = A; f.N1 = N1; f.N2 = N2; f.Q = Q;
    f.Qp = Q;
    f.N2p = (N2 + 3) & ~3;
    f.Ap = (A + CB - 1) / CB * CB;
    const int CA = fp64 ? RadialTile<double>::CA : RadialTile<float>::CA;
    const int PI = fp64 ? RadialTile<double>::PI : RadialTile<float>::PI;
    f.nct = (A + CA - 1) / CA;
    // point tiles of the last rank: at most 16 point groups (128 threads) per CTA, as even as
    // the multiple of PI allows
    const int tmax = 16 * PI;
    f.ntiles = (N2 + tmax - 1) / tmax;
    f.tw = ((N2 + f.ntiles - 1) / f.ntiles + PI - 1) / PI * PI;
    // angular rows: coefficient vector over the factors per (row, col), padded to chunks of
    // MIX_QC factors; each entry records its first and last nonzero factor
    f.Qp = (Q + MIX_QC - 1) / MIX_QC * MIX_QC;
    const int nch = f.Qp / MIX_QC;
    std::vector<std::map<int, std::vector<double>>> rows(A);
    for (int q = 0; q < Q; ++q) {
        const HostFactor &h = op->factors[q];
        for (size_t e = 0; e < h.row.size(); ++e) {
            std::vector<double> &v = rows[h.row[e]][h.col[e]];
            if (v.empty()) v.assign(f.Qp, 0.0);
            v[q] += h.coef[e];
        }
    }
    std::vector<int> row_ptr(A + 1, 0), col;
    std::vector<double> coef;
    const int ngroups = f.Ap / CB;
    std::vector<unsigned char> bflag((size_t)Q * f.nct, 0);
    std::vector<long long> rows_of_q(Q, 0);
    std::vector<std::vector<unsigned char>> has(A, std::vector<unsigned char>(Q, 0));
    std::vector<std::vector<unsigned char>> row_chunks(A, std::vector<unsigned char>(nch, 0));
    double mix_terms = 0;
    for (int a = 0; a < A; ++a) {
        std::vector<unsigned char> &row_has = has[a];
        for (const auto &kv : rows[a]) {
            int lo = f.Qp, hi = -1;
            for (int q = 0; q < Q; ++q)
                if (kv.second[q] != 0.0) {
                    lo = std::min(lo, q);
                    hi = std::max(hi, q);
                    row_has[q] = 1;
                    mix_terms += 1;
                }
            if (hi < 0) continue;  // all coefficients zero
            col.push_back(kv.first);  // entry metadata: col, first and last nonzero factor, 0
            col.push_back(lo);
            col.push_back(hi);
            col.push_back(0);
            coef.insert(coef.end(), kv.second.begin(), kv.second.end());
            for (int k = lo / MIX_QC; k <= hi / MIX_QC; ++k) row_chunks[a][k] = 1;
        }
        row_ptr[a + 1] = (int)(col.size() / 4);
        for (int q = 0; q < Q; ++q) rows_of_q[q] += row_has[q];
    }
    f.nE = (int)(col.size() / 4);
    std::vector<int> nzq;  // unused by the chunked mix
    std::vector<unsigned char> chunk((size_t)ngroups * nch, 0);
    // scratch slots: channels sorted by the set of factors they have, so that the radial
    // kernel's channel tiles skip more (factor, tile) stages; slot s holds channel perm[s]
    std::vector<int> perm(A);
    for (int a = 0; a < A; ++a) perm[a] = a;
    std::vector<int> cnt(A, 0);
    for (int a = 0; a < A; ++a)
        for (int q = 0; q < Q; ++q) cnt[a] += has[a][q];
    std::stable_sort(perm.begin(), perm.end(), [&](int x, int y) {
        if (cnt[x] != cnt[y]) return cnt[x] < cnt[y];
        return has[x] < has[y];
    });
    for (int sl = 0; sl < A; ++sl) {
        for (int q = 0; q < Q; ++q)
            if (has[perm[sl]][q]) bflag[(size_t)q * f.nct + sl / CA] = 1;
        for (int k = 0; k < nch; ++k)
            if (row_chunks[perm[sl]][k]) chunk[(size_t)(sl / CB) * nch + k] = 1;
    }
    // FP64 operators: the exact nonzero pairs per (channel, factor) segment
    std::vector<int> seg_ptr, seg, pcol;
    std::vector<double> pcoef;
    std::vector<unsigned char> seg_gq;
    if (fp64) {
        seg_ptr.assign(A + 1, 0);
        for (int a = 0; a < A; ++a) {
            for (int q = 0; q < Q; ++q) {
                const int first = (int)pcol.size();
                for (const auto &kv : rows[a])
                    if (kv.second[q] != 0.0) {
                        pcol.push_back(kv.first);
                        pcoef.push_back(kv.second[q]);
                    }
                if ((int)pcol.size() == first) continue;
                seg.push_back(q);
                seg.push_back(first);
                seg.push_back((int)pcol.size());
                seg.push_back(0);
            }
            seg_ptr[a + 1] = (int)(seg.size() / 4);
        }
        seg_gq.assign((size_t)ngroups * Q, 0);
        for (int sl = 0; sl < A; ++sl)
            for (int q = 0; q < Q; ++q)
                if (has[perm[sl]][q]) seg_gq[(size_t)(sl / CB) * Q + q] = 1;
    }

    // radial factors, last rank padded to N2p; points outside the grid are dropped
    std::vector<double> rad((size_t)Q * N1 * b * b * f.N2p, 0.0);
    double pts = 0;  // in-grid stencil points of one factor
    for (int i1 = 0; i1 < N1; ++i1)
        for (int d1 = 0; d1 < b; ++d1) {
            const int j1 = i1 + d1 - kb;
            if (j1 < 0 || j1 >= N1) continue;
            for (int i2 = 0; i2 < N2; ++i2)
                for (int d2 = 0; d2 < b; ++d2) {
                    const int j2 = i2 + d2 - kb;
                    if (j2 >= 0 && j2 < N2) pts += 1;
                }
        }
    double radial_terms = 0;
    for (int q = 0; q < Q; ++q) {
        const std::vector<double> &h = op->factors[q].radial;
        for (int i1 = 0; i1 < N1; ++i1)
            for (int d1 = 0; d1 < b; ++d1)
                for (int d2 = 0; d2 < b; ++d2)
                    for (int i2 = 0; i2 < N2; ++i2) {
                        const int j1 = i1 + d1 - kb, j2 = i2 + d2 - kb;
                        if (j1 < 0 || j1 >= N1 || j2 < 0 || j2 >= N2) continue;
                        rad[(((size_t)q * N1 + i1) * b + d1) * b * f.N2p + (size_t)d2 * f.N2p + i2] =
                            h[(((size_t)i1 * b + d1) * b + d2) * N2 + i2];
                    }
        radial_terms += pts * (double)rows_of_q[q];
    }
    const double NP = (double)N1 * N2;
    f.flops_mix = 4.0 * mix_terms * NP;      // complex x real = 2 FMA per nonzero pair and point
    f.flops_radial = 4.0 * radial_terms;     // per in-grid stencil point and nonzero row
    const size_t esz = fp64 ? sizeof(double) : sizeof(float);
    f.radial_bytes = (double)rad.size() * esz;
    std::vector<double> w(2 * (size_t)Q);
    std::vector<int> slot(Q);
    for (int q = 0; q < Q; ++q) {
        w[2 * q] = op->factors[q].w[0];
        w[2 * q + 1] = op->factors[q].w[1];
        slot[q] = op->factors[q].slot;
    }
    PG_TRY(upload_vec(&f.row_ptr, row_ptr));
    PG_TRY(upload_vec(&f.col, col));
    PG_TRY(upload_vec(&f.slot, slot));
    PG_TRY(upload_vec(&f.nzq, nzq));
    PG_TRY(upload_vec(&f.perm, perm));
    if (fp64) {
        PG_TRY(upload_vec(&f.seg_ptr, seg_ptr));
        PG_TRY(upload_vec(&f.seg, seg));
        PG_TRY(upload_vec(&f.pcol, pcol));
        PG_TRY(upload_vec(&f.seg_gq, seg_gq));
        PG_TRY(upload_real<double>(&f.pcoef, pcoef));
    }
    PG_TRY(upload_vec(&f.chunk, chunk));
    PG_TRY(upload_vec(&f.bflag, bflag));
    PG_CUDA_TRY(cudaMalloc(&f.w, sizeof(cxd) * Q));
    PG_CUDA_TRY(cudaMemcpy(f.w, w.data(), sizeof(cxd) * Q, cudaMemcpyHostToDevice));
    PG_TRY(fp64 ? upload_real<double>(&f.coef, coef) : upload_real<float>(&f.coef, coef));
    f.df = fp64 && op->fp64_emulation;
    if (f.df) {  // (hi, lo) float pairs in the 8 bytes of each coefficient
        std::vector<float> pairs(2 * rad.size());
        for (size_t t = 0; t < rad.size(); ++t) {
            const float hi = (float)rad[t];
            pairs[2 * t] = hi;
            pairs[2 * t + 1] = (float)(rad[t] - (double)hi);
        }
        PG_CUDA_TRY(cudaMalloc(&f.radial, sizeof(float) * pairs.size()));
        PG_CUDA_TRY(cudaMemcpy(f.radial, pairs.data(), sizeof(float) * pairs.size(), cudaMemcpyHostToDevice));
    } else {
        PG_TRY(fp64 ? upload_real<double>(&f.radial, rad) : upload_real<float>(&f.radial, rad));
    }
    const size_t zbytes = (size_t)Q * f.Ap * (size_t)N1 * N2 * 2 * esz;
    PG_CUDA_TRY(cudaMalloc(&f.Z, zbytes));
    PG_CUDA_TRY(cudaMemset(f.Z, 0, zbytes));  // rows without entries are read as zeros
    f.z_bytes = (double)zbytes;
    // shared memory: two barriers, then two stages of (Z box, coefficient box)
    if (fp64)
        f.radial_smem = 128 + 2 * (rad_round128<double>(rad_zbytes<double>(f.tw, kb)) +
                                   RB * rad_round128<double>(rad_rbytes<double>(f.tw, kb)));
    else
        f.radial_smem = 128 + 2 * (rad_round128<float>(rad_zbytes<float>(f.tw, kb)) +
                                   RB * rad_round128<float>(rad_rbytes<float>(f.tw, kb)));
    int dev = 0, optin = 0;
    PG_CUDA_TRY(cudaGetDevice(&dev));
    PG_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    if (f.radial_smem > (size_t)optin) return PG_ERR_SHAPE;
    if (fp64) {
        if (seg_smem_bytes<double>(Q) > (size_t)optin) return PG_ERR_SHAPE;
        PG_CUDA_TRY(cudaFuncSetAttribute(fact_mix_seg_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    } else {
        if (mix_smem_bytes<float>(Q) > (size_t)optin) return PG_ERR_SHAPE;
        PG_CUDA_TRY(cudaFuncSetAttribute(fact_mix_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    }
    if (fp64) {
        PG_CUDA_TRY(cudaFuncSetAttribute(fact_radial_kernel<double, 6>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
        PG_CUDA_TRY(cudaFuncSetAttribute(fact_radial_df_kernel<6>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    }
    else
        PG_CUDA_TRY(cudaFuncSetAttribute(fact_radial_kernel<float, 6>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    // TMA maps. Z as [Q * N1][N2][2 Ap] reals: box = 2 CA reals x (tw + 2k) points x 1 row,
    // the innermost coordinate 2 c0 (c0 a multiple of CA: 256-byte aligned); rows before 0 and
    // past N2 read as zeros. Coefficients as [Q * N1 * b * b][N2p] reals: box = tw x b.
    typedef CUresult (*EncodeTiled)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                    const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                    CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult qr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &qr) != cudaSuccess ||
        qr != cudaDriverEntryPointSuccess || !fn) {
        pg_set_last_error(cudaErrorNotSupported, "cuTensorMapEncodeTiled", __FILE__, __LINE__);
        return PG_ERR_CUDA;
    }
    const CUtensorMapDataType dt = fp64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    const cuuint32_t estr[3] = {1, 1, 1};
    {
        const cuuint64_t dims[3] = {(cuuint64_t)2 * f.Ap, (cuuint64_t)N2, (cuuint64_t)Q * N1};
        const cuuint64_t strides[2] = {(cuuint64_t)2 * f.Ap * esz, (cuuint64_t)2 * f.Ap * esz * N2};
        const cuuint32_t box[3] = {(cuuint32_t)(2 * CA), (cuuint32_t)(f.tw + 2 * kb), 1};
        CUresult r = ((EncodeTiled)fn)(&f.zmap, dt, 3, f.Z, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                       CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                       CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) {
            pg_set_last_error(cudaErrorInvalidValue, "cuTensorMapEncodeTiled(scratch)", __FILE__, __LINE__);
            return PG_ERR_CUDA;
        }
    }
    {
        const cuuint64_t dims[2] = {(cuuint64_t)f.N2p, (cuuint64_t)Q * N1 * b * b};
        const cuuint64_t strides[1] = {(cuuint64_t)f.N2p * esz};
        const cuuint32_t box[2] = {(cuuint32_t)f.tw, (cuuint32_t)b};
        CUresult r = ((EncodeTiled)fn)(&f.rmap, dt, 2, f.radial, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                       CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                       CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) {
            pg_set_last_error(cudaErrorInvalidValue, "cuTensorMapEncodeTiled(radial)", __FILE__, __LINE__);
            return PG_ERR_CUDA;
        }
    }
    return PG_OK;
}

extern "C" int pg_op_factored_info(const pg_op *op, double *info)
{
    if (!op || !info) return PG_ERR_ARG;
    const FactDev &f = op->fact;
    info[0] = f.Q;
    info[1] = f.nE;
    info[2] = f.flops_mix;
    info[3] = f.flops_radial;
    info[4] = f.radial_bytes;
    info[5] = f.z_bytes;
    return PG_OK;
}

extern "C" int pg_op_set_fp64_emulation(pg_op *op, int on)
{
    if (!op) return PG_ERR_ARG;
    if (op->finalized) return PG_ERR_STATE;
    if (op->precision != PG_FP64) return PG_ERR_ARG;
    op->fp64_emulation = on != 0;
    return PG_OK;
}
