// Persistent pAMP ensemble step (declarations and the algorithm in pamp_persistent.cuh).
//
// One CTA runs one member's step from start to end, so every wait is a CTA barrier: no CTA
// waits on another, and a launch needs no co-residency. Per member and Arnoldi step j
// (reference: core/krylov/pamp/pamp/pamp.h:270-351, the operator of
// pyprop/propagator/BasisPropagator.py:116-159 MultiplyHamiltonianBalancedOverlap):
//     w = H(t) t_j                        banded rows: real FP32 bands (or basis bands in shared
//                                         memory) x slot values
//     w <- U^-T w                         banded solve by chunks (pm_solve_cta)
//     h1 = V^H w, g = V^H V[j];  h2 = h1 - G h1;  w -= V (h1 + h2);  beta = ||w||
//                                         CGS2 with its second projection through the Gram matrix
//                                         G of the stored basis (FP32 per thread, FP64 CTA sums)
//     V[j+1] = w / beta;  t_(j+1) = U^-1 V[j+1]
// with t_0 = U^-1 V[0], V[0] = U psi / ||U psi||, and at the end c = ||U psi|| exp(-i dt H_k) e_1
// (pamp_expm_block) and psi = U^-1 V c = sum_j c_j t_j in double-float arithmetic. The
// Hessenberg columns, the coefficients and the statistics land where the graph path puts them,
// so both paths share their readers. The member's basis and scratch are read from L2 or HBM;
// its overlap factor, chunk tables and (where they allow it) basis bands sit in shared memory.
#include "pamp_persistent.cuh"

#include <algorithm>
#include <cmath>
#include <mutex>

namespace {

constexpr int PM_MAXM = 20;     // Krylov basis sizes with per-thread column sums in registers
constexpr int PM_MAXKB = 8;     // band half-width (at most the 8-row chunks of the FP64 solve)
constexpr int PM_RED = 4 * PM_MAXM + 2;  // per-warp partials: two complex columns and one scalar
constexpr int PM_WARPS = 16;    // at most 512 threads per CTA
constexpr int PM_MAXBASIS = 4;  // basis bands of an operator staged in shared memory

struct PmLayout {
    size_t us = 0, uinv = 0, gu = 0, gl = 0, zb = 0, rp = 0, ent = 0, bas = 0, red = 0, h = 0, gram = 0, scal = 0,
           cc = 0, ex = 0;
    size_t bytes = 0;
};

__host__ __device__ inline size_t pm_align16(size_t x) { return (x + 15) / 16 * 16; }

// Nmax, kbmax, mmax: the members' largest radial size, band half-width and basis size; nchmax,
// entmax: their largest channel and operator-entry (or term) counts; basismax: their largest
// number of basis bands (0: every member reads its bands from global memory)
__host__ __device__ inline PmLayout pm_layout(int Nmax, int kbmax, int mmax, int nchmax, int entmax, int basismax)
{
    PmLayout L;
    const size_t nck = (size_t)(Nmax + 31) / 32;
    size_t o = 0;
    L.us = o;   o = pm_align16(o + sizeof(float) * (size_t)Nmax * (kbmax + 1));
    L.uinv = o; o = pm_align16(o + sizeof(float) * (size_t)Nmax);
    L.gu = o;   o = pm_align16(o + sizeof(float) * nck * 32 * kbmax);
    L.gl = o;   o = pm_align16(o + sizeof(float) * nck * 32 * kbmax);
    L.zb = o;   o = pm_align16(o + sizeof(cxf) * (size_t)nchmax * nck * kbmax);
    L.rp = o;   o = pm_align16(o + sizeof(int) * (size_t)(nchmax + 1));
    L.ent = o;  o = pm_align16(o + sizeof(int4) * (size_t)entmax);
    // the basis bands are read in the Arnoldi steps only; the exponential's scratch, used after
    // them, shares their region
    L.bas = o;
    L.ex = o;
    o = pm_align16(o + std::max(sizeof(float) * (size_t)basismax * (2 * kbmax + 1) * Nmax,
                                sizeof(cxd) * 6 * (size_t)mmax * mmax));
    L.red = o;  o = pm_align16(o + sizeof(double) * PM_WARPS * PM_RED);
    L.h = o;    o = pm_align16(o + sizeof(cxd) * 3 * (PM_MAXM + 1));
    L.gram = o; o = pm_align16(o + sizeof(cxd) * PM_MAXM * PM_MAXM);
    L.scal = o; o = pm_align16(o + sizeof(cxf) * PG_MAX_SLOTS);
    L.cc = o;   o = pm_align16(o + sizeof(cxd) * PM_MAXM);
    L.bytes = o;
    return L;
}

// Sums of per-thread FP32 column partials acc1[c] and (when two) acc2[c], c < J: warp sums in
// FP32, CTA sums in FP64, into out1[c] and out2[c] (complex128). Ends after a CTA barrier, so the
// results are visible to every thread.
template <int MAXJ, bool TWO>
__device__ __forceinline__ void pm_reduce(const cxf (&acc1)[MAXJ], const cxf (&acc2)[MAXJ], int J, double *red,
                                          cxd *out1, cxd *out2)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int c = 0; c < MAXJ; ++c) {
        if (c < J) {
            float x = acc1[c].x, y = acc1[c].y, u = 0.f, v = 0.f;
            if (TWO) {
                u = acc2[c].x;
                v = acc2[c].y;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                x += __shfl_xor_sync(0xffffffffu, x, o);
                y += __shfl_xor_sync(0xffffffffu, y, o);
                if (TWO) {
                    u += __shfl_xor_sync(0xffffffffu, u, o);
                    v += __shfl_xor_sync(0xffffffffu, v, o);
                }
            }
            if (lane == 0) {
                red[warp * PM_RED + 2 * c] = x;
                red[warp * PM_RED + 2 * c + 1] = y;
                if (TWO) {
                    red[warp * PM_RED + 2 * MAXJ + 2 * c] = u;
                    red[warp * PM_RED + 2 * MAXJ + 2 * c + 1] = v;
                }
            }
        }
    }
    __syncthreads();
    for (int q = threadIdx.x; q < (TWO ? 4 : 2) * J; q += blockDim.x) {
        const int second = q >= 2 * J, v = second ? q - 2 * J : q;
        double sum = 0.0;
        for (int w = 0; w < nw; ++w) sum += red[w * PM_RED + (second ? 2 * MAXJ : 0) + v];
        reinterpret_cast<double *>(second ? out2 : out1)[v] = sum;
    }
    __syncthreads();
}

// sum of one FP64 scalar over the CTA (every thread gets it)
__device__ __forceinline__ double pm_sum1(double v, double *red, double *slot)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp * PM_RED + PM_RED - 1] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < nw; ++w) s += red[w * PM_RED + PM_RED - 1];
        *slot = s;
    }
    __syncthreads();
    return *slot;
}

// Banded triangular solves of every fibre of a member, parallel over chunks of CH rows: with z_c
// the chunk's solution for zero values outside it and G_c (CH x kb, precomputed) its response to
// the kb values that couple it to the neighbouring chunk (the first kb rows of chunk c+1 for
// U x = b, the last kb rows of chunk c-1 for U^T x = b),
//     x_c = z_c + G_c s,
// and the coupling values s follow from a kb-wide recurrence over the chunks of each fibre.
// Phase 1 (one thread per (fibre, chunk), the chunk in registers) writes z_c to x and its kb
// boundary values to shared memory (sb: [nch][nchunks][kb]); phase 2 (one thread per fibre)
// turns them into the coupling values in place; phase 3 (one thread per (fibre, chunk)) adds
// G_c s to x. A CTA barrier after each phase. (Keeping the chunk in registers from phase 1 to
// phase 3 spills them.) U(i, i+d) at U[i (kb+1) + d]; Uinv holds 1 / U(i, i).
template <int KB, int CH, bool LOWER, typename R>
__device__ void pm_solve_cta(const cx<R> *b, double sc, cx<R> *vout, cx<R> *x, int nch, int N, int kb_rt,
                             const R *__restrict__ U, const R *__restrict__ Uinv, const R *__restrict__ G, cx<R> *sb)
{
    const int kb = KB > 0 ? KB : kb_rt, kw = kb + 1;
    const int nck = (N + CH - 1) / CH, ntask = nch * nck, tid = threadIdx.x, T = blockDim.x;
    const R scr = (R)sc;  // the scale in the vector's precision (FP64 arithmetic is slow here)
    // phase 1: z_c and its boundary values
    for (int task = tid; task < ntask; task += T) {
        cx<R> z[CH];
        const int a = task / nck, c = task - a * nck, r0 = c * CH, len = min(CH, N - r0);
        const cx<R> *bb = b + (size_t)a * N + r0;
        // all loads first: vout may be b itself (in-place normalisation), and a store between
        // two loads would make each load wait for the previous one
#pragma unroll
        for (int r = 0; r < CH; ++r) z[r] = r < len ? bb[r] : mk<R>((R)0, (R)0);
        if (sc != 1.0) {
#pragma unroll
            for (int r = 0; r < CH; ++r) z[r] = mk<R>(z[r].x * scr, z[r].y * scr);
        }
        if (vout) {
            cx<R> *vo = vout + (size_t)a * N + r0;
#pragma unroll
            for (int r = 0; r < CH; ++r)
                if (r < len) vo[r] = z[r];
        }
        if constexpr (LOWER) {
#pragma unroll
            for (int r = 0; r < CH; ++r) {
                if (r < len) {
                    cx<R> acc = z[r];
                    if constexpr (KB > 0) {
#pragma unroll
                        for (int d = KB; d >= 1; --d)
                            if (r - d >= 0) {
                                const R u = U[(size_t)(r0 + r - d) * kw + d];
                                acc.x -= u * z[r - d].x;
                                acc.y -= u * z[r - d].y;
                            }
                    } else {
                        for (int d = min(kb, r); d >= 1; --d) {
                            const R u = U[(size_t)(r0 + r - d) * kw + d];
                            acc.x -= u * z[r - d].x;
                            acc.y -= u * z[r - d].y;
                        }
                    }
                    const R inv = Uinv[r0 + r];
                    z[r] = mk<R>(acc.x * inv, acc.y * inv);
                }
            }
        } else {
#pragma unroll
            for (int r = CH - 1; r >= 0; --r) {
                if (r < len) {
                    cx<R> acc = z[r];
                    if constexpr (KB > 0) {
#pragma unroll
                        for (int d = KB; d >= 1; --d)
                            if (r + d < CH) {  // z past the chunk's (or the fibre's) end is zero
                                const R u = U[(size_t)(r0 + r) * kw + d];
                                acc.x -= u * z[r + d].x;
                                acc.y -= u * z[r + d].y;
                            }
                    } else {
                        for (int d = min(kb, CH - 1 - r); d >= 1; --d) {
                            const R u = U[(size_t)(r0 + r) * kw + d];
                            acc.x -= u * z[r + d].x;
                            acc.y -= u * z[r + d].y;
                        }
                    }
                    const R inv = Uinv[r0 + r];
                    z[r] = mk<R>(acc.x * inv, acc.y * inv);
                }
            }
        }
        cx<R> *zb = sb + ((size_t)a * nck + c) * kb;
        if constexpr (KB > 0) {
#pragma unroll
            for (int q = 0; q < KB; ++q) {
                if (LOWER) {
                    if (c + 1 < nck) zb[q] = z[CH - KB + q];  // chunks before the last are full
                } else {
                    zb[q] = z[q];  // zero past the fibre's end
                }
            }
        } else {
            for (int q = 0; q < kb; ++q) {
                if (LOWER) {
                    if (c + 1 < nck) zb[q] = z[CH - kb + q];
                } else {
                    zb[q] = z[q];
                }
            }
        }
        cx<R> *xx = x + (size_t)a * N + r0;
#pragma unroll
        for (int r = 0; r < CH; ++r)
            if (r < len) xx[r] = z[r];
    }
    __syncthreads();
    // phase 2: the coupling values of every chunk, in chunk order, in place of its boundary values
    for (int a = tid; a < nch; a += T) {
        cx<R> *sa = sb + (size_t)a * nck * kb;
        cx<R> s[KB > 0 ? KB : 16];
        cx<R> sn[KB > 0 ? KB : 16];
        if constexpr (LOWER) {
            for (int c = 0; c + 1 < nck; ++c) {  // s_c = the last kb rows of chunk c
                for (int q = 0; q < kb; ++q) {
                    cx<R> v = sa[(size_t)c * kb + q];
                    if (c > 0) {
                        const R *g = G + ((size_t)c * CH + (CH - kb + q)) * kb;
                        for (int p = 0; p < kb; ++p) {
                            v.x += g[p] * s[p].x;
                            v.y += g[p] * s[p].y;
                        }
                    }
                    sn[q] = v;
                }
                for (int q = 0; q < kb; ++q) {
                    s[q] = sn[q];
                    sa[(size_t)c * kb + q] = sn[q];
                }
            }
        } else {
            for (int c = nck - 1; c >= 1; --c) {  // s_c = the first kb rows of chunk c
                for (int q = 0; q < kb; ++q) {
                    cx<R> v = sa[(size_t)c * kb + q];
                    if (c + 1 < nck) {
                        const R *g = G + ((size_t)c * CH + q) * kb;
                        for (int p = 0; p < kb; ++p) {
                            v.x += g[p] * s[p].x;
                            v.y += g[p] * s[p].y;
                        }
                    }
                    sn[q] = v;
                }
                for (int q = 0; q < kb; ++q) {
                    s[q] = sn[q];
                    sa[(size_t)c * kb + q] = sn[q];
                }
            }
        }
    }
    __syncthreads();
    // phase 3: x_c = z_c + G_c s (the neighbouring chunk's coupling values)
    {
        for (int task = tid; task < ntask; task += T) {
            const int a = task / nck, c = task - a * nck, r0 = c * CH, len = min(CH, N - r0);
            const int cs = LOWER ? c - 1 : c + 1;
            if (cs < 0 || cs >= nck) continue;
            const cx<R> *sv = sb + ((size_t)a * nck + cs) * kb;
            cx<R> s[KB > 0 ? KB : 16];
            for (int q = 0; q < kb; ++q) s[q] = sv[q];
            cx<R> *xx = x + (size_t)a * N + r0;
            const R *g = G + (size_t)c * CH * kb;
            // all loads of the chunk first, then the corrections and the stores
            cx<R> z[CH];
#pragma unroll
            for (int r = 0; r < CH; ++r) z[r] = r < len ? xx[r] : mk<R>((R)0, (R)0);
#pragma unroll
            for (int r = 0; r < CH; ++r) {
                if (r < len) {
                    cx<R> v = z[r];
                    for (int q = 0; q < kb; ++q) {
                        const R gq = g[(size_t)r * kb + q];
                        v.x += gq * s[q].x;
                        v.y += gq * s[q].y;
                    }
                    xx[r] = v;
                }
            }
        }
    }
    __syncthreads();
}

// (h, l) += a (bh + bl) in double-float arithmetic: a bh exactly as ph + pl (FMA), a bl added to
// the low part, the high parts summed by Knuth's two-sum
__device__ __forceinline__ void df_madd(float &h, float &l, float a, float bh, float bl)
{
    const float ph = __fmul_rn(a, bh);  // never contracted into an FMA with the two-sum below
    const float pl = fmaf(a, bh, -ph) + a * bl;
    const float s = h + ph;
    const float bb = s - h;
    const float err = (h - (s - bb)) + (ph - bb);
    h = s;
    l += err + pl;
}

// (U psi)[e] in FP64 for element e = a N + i
__device__ __forceinline__ cxd pm_upsi(const cxd *__restrict__ psi, const double *__restrict__ U, int N, int kb,
                                       long long e)
{
    const int a = (int)(e / N), i = (int)(e - (long long)a * N);
    const cxd *x = psi + (size_t)a * N;
    const double *u = U + (size_t)i * (kb + 1);
    cxd y = mk<double>(0.0, 0.0);
    for (int d = 0; d <= kb && i + d < N; ++d) {
        const double c = __ldg(u + d);
        const cxd v = x[i + d];
        y.x = fma(c, v.x, y.x);
        y.y = fma(c, v.y, y.y);
    }
    return y;
}

template <int KB>
__device__ void pm_member_step(const PmMember &M, double dt, unsigned char *smem, const PmLayout &L)
{
    float *Us = reinterpret_cast<float *>(smem + L.us);
    float *Uinv = reinterpret_cast<float *>(smem + L.uinv);
    float *Gu = reinterpret_cast<float *>(smem + L.gu);
    float *Gl = reinterpret_cast<float *>(smem + L.gl);
    cxf *zb = reinterpret_cast<cxf *>(smem + L.zb);  // the solves' chunk boundary values
    int *rp = reinterpret_cast<int *>(smem + L.rp);
    int4 *ent = reinterpret_cast<int4 *>(smem + L.ent);
    double *red = reinterpret_cast<double *>(smem + L.red);
    cxd *h1 = reinterpret_cast<cxd *>(smem + L.h);
    cxd *h2 = h1 + (PM_MAXM + 1);
    cxd *gcol = h2 + (PM_MAXM + 1);
    cxd *gram = reinterpret_cast<cxd *>(smem + L.gram);
    cxf *scal = reinterpret_cast<cxf *>(smem + L.scal);
    cxd *cc = reinterpret_cast<cxd *>(smem + L.cc);
    const int tid = threadIdx.x, T = blockDim.x;
    const int N = M.N, nch = M.nch, m = M.m, ld = M.ld;
    const int kb = (KB > 0) ? KB : M.kb, kw = kb + 1, bw = 2 * kb + 1;
    const long long n = M.n;
    const size_t cd = 2 * (size_t)(m + 2);
    const int nck = (N + 31) / 32;
    cxf *__restrict__ V = M.V;
    cxf *__restrict__ w = M.w;
    cxf *__restrict__ Tb = M.T;  // t_j = U^-1 V[j], all kept: psi = U^-1 V c = T c

    // the member's overlap factor, chunk tables, operator rows and slot values in shared memory
    for (int q = tid; q < N * kw; q += T) Us[q] = M.U32[q];
    for (int i = tid; i < N; i += T) Uinv[i] = 1.0f / M.U32[(size_t)i * kw];
    for (int q = tid; q < nck * 32 * kb; q += T) {
        Gu[q] = M.G32u[q];
        Gl[q] = M.G32l[q];
    }
    for (int r = tid; r <= nch; r += T) rp[r] = M.row_ptr[r];
    for (int e = tid; e < M.nent; e += T)
        ent[e] = make_int4(M.ent_col[e], M.ent_band[e], M.ent_slot[e], __float_as_int(M.ent_coef ? M.ent_coef[e] : 1.f));
    float *Bs = reinterpret_cast<float *>(smem + L.bas);  // basis bands [k][d][N]
    const int nbasis = M.nbasis;
    for (int q = tid; q < nbasis * bw * N; q += T) Bs[q] = M.basis[q];
    for (int s = tid; s < PG_MAX_SLOTS; s += T) scal[s] = cvt<float>(M.scales[s]);

    // V[0] = U psi / ||U psi|| (FP64 products and sum), ||U psi|| kept for the combination
    double nrm = 0.0;
    for (long long e = tid; e < n; e += T) {
        const cxd y = pm_upsi(M.psi, M.U64, N, kb, e);
        nrm = fma(y.x, y.x, fma(y.y, y.y, nrm));
        V[e] = mk<float>((float)y.x, (float)y.y);
    }
    nrm = pm_sum1(nrm, red, reinterpret_cast<double *>(cc));
    {
        const double b = sqrt(nrm);
        const float s = b > 0.0 ? (float)(1.0 / b) : 0.f;
        if (tid == 0) {
            M.norm[0] = nrm;
            M.norm[1] = b;
        }
        for (long long e = tid; e < n; e += T) {
            const cxf y = V[e];
            V[e] = mk<float>(y.x * s, y.y * s);
        }
    }
    __syncthreads();
    pm_solve_cta<KB, 32, false, float>(V, 1.0, nullptr, Tb, nch, N, kb, Us, Uinv, Gu, zb);

    for (int j = 0; j < m; ++j) {
        const cxf *__restrict__ t = Tb + (size_t)j * n;
        const int J = j + 1;
        double *col0 = M.cols + ((size_t)j * 3 + 0) * cd;
        double *col1 = M.cols + ((size_t)j * 3 + 1) * cd;
        double *col2 = M.cols + ((size_t)j * 3 + 2) * cd;
        // w = H(t) t_j
        for (long long e = tid; e < n; e += T) {
            const int a = (int)(e / N), i = (int)(e - (long long)a * N);
            cxf acc = mk<float>(0.f, 0.f);
            const int e1 = rp[a + 1];
            for (int en = rp[a]; en < e1; ++en) {
                const int4 E = ent[en];
                const cxf *__restrict__ x = t + (size_t)E.x * N;
                cxf tt = mk<float>(0.f, 0.f);
                if constexpr (KB > 0) {
                    float c[2 * KB + 1];
                    if (nbasis) {  // basis band from shared memory
                        const float *B = Bs + (size_t)E.y * bw * N + i;
#pragma unroll
                        for (int d = 0; d < 2 * KB + 1; ++d) c[d] = B[(size_t)d * N];
                    } else {
                        const float *__restrict__ B = M.bands + (size_t)E.y * bw * ld + i;
#pragma unroll
                        for (int d = 0; d < 2 * KB + 1; ++d) c[d] = __ldg(B + (size_t)d * ld);
                    }
#pragma unroll
                    for (int d = 0; d < 2 * KB + 1; ++d) {
                        const int jj = i + d - KB;
                        if (jj >= 0 && jj < N) {
                            const cxf v = x[jj];
                            tt.x = fmaf(c[d], v.x, tt.x);
                            tt.y = fmaf(c[d], v.y, tt.y);
                        }
                    }
                } else {
                    const float *B = nbasis ? Bs + (size_t)E.y * bw * N + i : M.bands + (size_t)E.y * bw * ld + i;
                    const int bld = nbasis ? N : ld;
                    for (int d = 0; d < bw; ++d) {
                        const int jj = i + d - kb;
                        if (jj >= 0 && jj < N) {
                            const float c = B[(size_t)d * bld];
                            const cxf v = x[jj];
                            tt.x = fmaf(c, v.x, tt.x);
                            tt.y = fmaf(c, v.y, tt.y);
                        }
                    }
                }
                const float cf = __int_as_float(E.w);
                const cxf sc = scal[E.z];
                cfma(acc, mk<float>(sc.x * cf, sc.y * cf), tt);
            }
            w[e] = acc;
        }
        __syncthreads();
        pm_solve_cta<KB, 32, true, float>(w, 1.0, nullptr, w, nch, N, kb, Us, Uinv, Gl, zb);
        // Gram-Schmidt, first pass: h1 = V^H w and the new Gram column V^H V[j] (one read of V)
        {
            cxf acc[PM_MAXM], gacc[PM_MAXM];
#pragma unroll
            for (int c = 0; c < PM_MAXM; ++c) {
                acc[c] = mk<float>(0.f, 0.f);
                gacc[c] = mk<float>(0.f, 0.f);
            }
            for (long long e = tid; e < n; e += T) {
                const cxf we = w[e], vj = V[(size_t)j * n + e];
#pragma unroll
                for (int c = 0; c < PM_MAXM; ++c)
                    if (c < J) {
                        const cxf v = V[(size_t)c * n + e];
                        cfma_conj(acc[c], v, we);
                        cfma_conj(gacc[c], v, vj);
                    }
            }
            pm_reduce<PM_MAXM, true>(acc, gacc, J, red, h1, gcol);
        }
        // second pass through the Gram matrix G = V^H V of the stored basis:
        // h2 = V^H (w - V h1) = h1 - G h1, so that w - V (h1 + h2) needs one more read of V
        for (int c = tid; c < J; c += T) {
            gram[c * PM_MAXM + j] = gcol[c];
            gram[j * PM_MAXM + c] = c == j ? mk<double>(gcol[c].x, 0.0) : mk<double>(gcol[c].x, -gcol[c].y);
        }
        __syncthreads();
        cxf *hf = reinterpret_cast<cxf *>(cc);  // h1 + h2 in FP32 for the update
        for (int c = tid; c < J; c += T) {
            cxd g = mk<double>(0.0, 0.0);
            if (M.double_ortho)
                for (int q = 0; q < J; ++q) cfma(g, gram[c * PM_MAXM + q], h1[q]);
            const cxd hc = M.double_ortho ? h1[c] - g : mk<double>(0.0, 0.0);
            h2[c] = hc;
            hf[c] = cvt<float>(h1[c] + hc);
            col0[2 * c] = h1[c].x;
            col0[2 * c + 1] = h1[c].y;
            col1[2 * c] = hc.x;
            col1[2 * c + 1] = hc.y;
        }
        __syncthreads();
        // w - V (h1 + h2) into the slot of V[j+1] (unnormalised) and beta = its norm
        {
            cxf *dst = (J < m) ? V + (size_t)J * n : nullptr;
            // the columns read below (c < J) and the slot written (J) are disjoint: separate
            // pointers let the next element's loads go ahead of this element's store
            const cxf *__restrict__ Vr = V;
            cxf *__restrict__ dstw = dst;
            float nf = 0.f;  // per-thread sum in FP32 (as the graph path's column sums), CTA sum in FP64
            for (long long e = tid; e < n; e += T) {
                cxf x = w[e];
#pragma unroll
                for (int c = 0; c < PM_MAXM; ++c)
                    if (c < J) {
                        const cxf v = Vr[(size_t)c * n + e];
                        const cxf hc = hf[c];
                        x.x = fmaf(-v.x, hc.x, x.x);
                        x.x = fmaf(v.y, hc.y, x.x);
                        x.y = fmaf(-v.x, hc.y, x.y);
                        x.y = fmaf(-v.y, hc.x, x.y);
                    }
                if (dstw) dstw[e] = x;
                nf = fmaf(x.x, x.x, fmaf(x.y, x.y, nf));
            }
            __syncthreads();  // hf (in cc) is read above; pm_sum1 writes its slot there
            double nn = pm_sum1((double)nf, red, reinterpret_cast<double *>(cc));
            const double beta = sqrt(nn);
            if (tid == 0) {
                col2[2 * J] = nn;
                col2[2 * J + 1] = beta;
            }
            // V[j+1] = (w - V h) / beta in place and t_(j+1) = U^-1 V[j+1]
            if (dst) {
                const double s = beta > 0.0 ? 1.0 / beta : 0.0;
                pm_solve_cta<KB, 32, false, float>(dst, s, dst, Tb + (size_t)J * n, nch, N, kb, Us, Uinv, Gu,
                                                   zb);
            }
        }
    }
    __syncthreads();  // the columns written above are read by the exponential's threads
    pamp_expm_block_df(M.ex, dt, smem + L.ex);
    // psi = U^-1 V c = T c (c includes ||U psi||): the combination of the t_j = U^-1 V[j] that the
    // Arnoldi steps computed, so no banded solve of psi is needed
    const int k = (int)M.ex.stats[0];
    for (int c = tid; c < PM_MAXM; c += T) cc[c] = c < k ? mk<double>(M.ex.c[2 * c], M.ex.c[2 * c + 1]) : mk<double>(0.0, 0.0);
    __syncthreads();
    // in double-float arithmetic (FP32 pairs hi + lo: the coefficients split into two FP32 parts,
    // each product made exact by an FMA, the sums by Knuth's two-sum), about 2^-44 relative per
    // sum - below the FP32 rounding of the vectors it combines - at FP32 rates
    float *cq = reinterpret_cast<float *>(smem + L.ex);  // [k][4]: re hi, re lo, im hi, im lo
    for (int c = tid; c < k; c += T) {
        const cxd q = cc[c];
        const float rh = (float)q.x, ih = (float)q.y;
        cq[4 * c] = rh;
        cq[4 * c + 1] = (float)(q.x - (double)rh);
        cq[4 * c + 2] = ih;
        cq[4 * c + 3] = (float)(q.y - (double)ih);
    }
    __syncthreads();
    for (long long e = tid; e < n; e += T) {
        float xh = 0.f, xl = 0.f, yh = 0.f, yl = 0.f;
        for (int c = 0; c < k; ++c) {
            const cxf v = Tb[(size_t)c * n + e];
            const float rh = cq[4 * c], rl = cq[4 * c + 1], ih = cq[4 * c + 2], il = cq[4 * c + 3];
            df_madd(xh, xl, v.x, rh, rl);
            df_madd(xh, xl, -v.y, ih, il);
            df_madd(yh, yl, v.x, ih, il);
            df_madd(yh, yl, v.y, rh, rl);
        }
        M.psi[e] = mk<double>((double)xh + (double)xl, (double)yh + (double)yl);
    }
    __syncthreads();
}

// MAXT: the launch bound (512: 128 registers per thread, some spilled; 256: room for all of
// them, fewer warps per SM) - the autotuner times both
template <int KB, int MAXT>
__global__ void __launch_bounds__(MAXT) pm_step_kernel(const PmMember *__restrict__ members, int nmembers,
                                                       const int *__restrict__ order, unsigned *queue,
                                                       const double *__restrict__ dt_dev, PmLayout L)
{
    extern __shared__ __align__(16) unsigned char pm_smem[];
    __shared__ int s_pick;
    const double dt = *dt_dev;
    for (;;) {
        if (threadIdx.x == 0) s_pick = (int)atomicAdd(queue, 1u);
        __syncthreads();
        const int q = s_pick;
        __syncthreads();  // everyone has read the pick before thread 0 takes the next one
        if (q >= nmembers) break;
        pm_member_step<KB>(members[order[q]], dt, pm_smem, L);
    }
}

const void *pm_kernel(bool kb6, bool wide)
{
    if (kb6) return wide ? (const void *)pm_step_kernel<6, 256> : (const void *)pm_step_kernel<6, 512>;
    return wide ? (const void *)pm_step_kernel<-1, 256> : (const void *)pm_step_kernel<-1, 512>;
}

std::mutex g_pm_attr_mutex;
size_t g_pm_attr[4] = {0, 0, 0, 0};

// the dynamic shared-memory limit of an instance only ever rises
cudaError_t pm_raise_smem(bool kb6, bool wide, size_t bytes)
{
    std::lock_guard<std::mutex> lock(g_pm_attr_mutex);
    size_t &cur = g_pm_attr[(kb6 ? 1 : 0) + (wide ? 2 : 0)];
    if (cur >= bytes) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(pm_kernel(kb6, wide), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) cur = bytes;
    return e;
}

}  // namespace

int pm_real_bands(const pg_op *op, float **dev)
{
    const size_t rows = op->h_bands.size() / (size_t)std::max(1, op->N);
    std::vector<float> out(std::max<size_t>(1, rows * (size_t)op->ld), 0.f);
    for (size_t q = 0; q < rows; ++q)
        for (int i = 0; i < op->N; ++i) {
            const std::complex<double> v = op->h_bands[q * op->N + i];
            if (v.imag() != 0.0) return PG_ERR_STORAGE;
            out[q * op->ld + i] = (float)v.real();
        }
    PG_CUDA_TRY(cudaMalloc((void **)dev, out.size() * sizeof(float)));
    PG_CUDA_TRY(cudaMemcpy(*dev, out.data(), out.size() * sizeof(float), cudaMemcpyHostToDevice));
    return PG_OK;
}

size_t pm_smem_bytes(int Nmax, int kbmax, int mmax, int nchmax, int entmax, int basismax)
{
    return pm_layout(Nmax, kbmax, mmax, nchmax, entmax, basismax).bytes;
}

int pm_max_basis_bands() { return PM_MAXBASIS; }

int pm_member_basis(const pg_op *op, PmMember &M, std::vector<void *> &allocs)
{
    M.nbasis = 0;
    const int N = op->N, bw = 2 * op->kb + 1;
    const size_t Lb = (size_t)bw * N;
    if (N < 1 || op->h_bands.size() % Lb) return PG_OK;
    const int nb = (int)(op->h_bands.size() / Lb);
    std::vector<double> B((size_t)nb * Lb);
    for (size_t x = 0; x < B.size(); ++x) B[x] = op->h_bands[x].real();
    auto band = [&](int q) { return B.data() + (size_t)q * Lb; };
    auto amax = [&](const double *v) {
        double m = 0.0;
        for (size_t x = 0; x < Lb; ++x) m = std::max(m, std::fabs(v[x]));
        return m;
    };
    // bands that are multiples of one another: rep[q], band q = ratio[q] * band rep[q]
    std::vector<int> rep(nb, -1), reps;
    std::vector<double> ratio(nb, 0.0);
    std::vector<size_t> piv(nb, 0);
    for (int q = 0; q < nb; ++q) {
        const double *v = band(q);
        const double mq = amax(v);
        for (size_t x = 0; x < Lb; ++x)
            if (std::fabs(v[x]) == mq) { piv[q] = x; break; }
        if (mq == 0.0) { rep[q] = -2; continue; }  // an all-zero band contributes nothing
        for (int r : reps) {
            const double *u = band(r);
            const double rho = v[piv[r]] / u[piv[r]];
            double dev = 0.0;
            for (size_t x = 0; x < Lb && dev <= 1e-13 * mq; ++x) dev = std::max(dev, std::fabs(v[x] - rho * u[x]));
            if (dev <= 1e-13 * mq) { rep[q] = r; ratio[q] = rho; break; }
        }
        if (rep[q] == -1) { rep[q] = q; ratio[q] = 1.0; reps.push_back(q); }
    }
    // representation of every representative over the basis: up to two (basis band, coefficient)
    std::vector<std::vector<double>> basis;
    std::vector<std::vector<std::pair<int, double>>> repr(nb);
    if ((int)reps.size() <= PM_MAXBASIS) {
        for (int r : reps) {
            repr[r] = {{(int)basis.size(), 1.0}};
            basis.emplace_back(band(r), band(r) + Lb);
        }
    } else {
        // blocks on the diagonal: A + alpha D (a common field-free band plus a multiple of one more);
        // the other blocks: one basis band each
        std::vector<char> on_diag(nb, 0), off_diag(nb, 0);
        for (int r = 0; r < op->nrows; ++r)
            for (int e = op->h_row_ptr[r]; e < op->h_row_ptr[r + 1]; ++e) {
                const int q = op->h_ent_band[e];
                if (rep[q] < 0) continue;
                (op->h_ent_col[e] == r ? on_diag : off_diag)[rep[q]] = 1;
            }
        std::vector<int> dreps, oreps;
        for (int r : reps) {
            if (on_diag[r] && off_diag[r]) return PG_OK;
            (on_diag[r] ? dreps : oreps).push_back(r);
        }
        if (dreps.size() < 2 || (int)oreps.size() > PM_MAXBASIS - 2) return PG_OK;
        const double *A = band(dreps[0]);
        std::vector<double> D(Lb);
        for (size_t x = 0; x < Lb; ++x) D[x] = band(dreps[1])[x] - A[x];
        double dd = 0.0;
        for (size_t x = 0; x < Lb; ++x) dd += D[x] * D[x];
        if (dd == 0.0) return PG_OK;
        basis.emplace_back(A, A + Lb);
        basis.push_back(D);
        repr[dreps[0]] = {{0, 1.0}};
        for (size_t k = 1; k < dreps.size(); ++k) {
            const double *v = band(dreps[k]);
            double num = 0.0;
            for (size_t x = 0; x < Lb; ++x) num += (v[x] - A[x]) * D[x];
            const double alpha = num / dd;
            double dev = 0.0;
            for (size_t x = 0; x < Lb; ++x) dev = std::max(dev, std::fabs(v[x] - A[x] - alpha * D[x]));
            if (dev > 1e-12 * std::max(amax(v), amax(A))) return PG_OK;
            repr[dreps[k]] = {{0, 1.0}, {1, alpha}};
        }
        for (int r : oreps) {
            repr[r] = {{(int)basis.size(), 1.0}};
            basis.emplace_back(band(r), band(r) + Lb);
        }
    }
    // terms per operator row, in the order of its entries
    std::vector<int> rp(op->nrows + 1, 0), tcol, tbas, tslot;
    std::vector<float> tcoef;
    for (int r = 0; r < op->nrows; ++r) {
        for (int e = op->h_row_ptr[r]; e < op->h_row_ptr[r + 1]; ++e) {
            const int q = op->h_ent_band[e];
            if (rep[q] < 0) continue;
            for (const auto &kc : repr[rep[q]]) {
                tcol.push_back(op->h_ent_col[e]);
                tbas.push_back(kc.first);
                tslot.push_back(op->h_ent_slot[e]);
                tcoef.push_back((float)(ratio[q] * kc.second));
            }
        }
        rp[r + 1] = (int)tcol.size();
    }
    std::vector<float> bas(basis.size() * Lb);
    for (size_t k = 0; k < basis.size(); ++k)
        for (size_t x = 0; x < Lb; ++x) bas[k * Lb + x] = (float)basis[k][x];
    auto up = [&](const void *src, size_t bytes, const void **dst) -> int {
        void *p = nullptr;
        PG_CUDA_TRY(cudaMalloc(&p, std::max<size_t>(16, bytes)));
        allocs.push_back(p);
        if (bytes) PG_CUDA_TRY(cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice));
        *dst = p;
        return PG_OK;
    };
    PG_TRY(up(rp.data(), rp.size() * sizeof(int), (const void **)&M.row_ptr));
    PG_TRY(up(tcol.data(), tcol.size() * sizeof(int), (const void **)&M.ent_col));
    PG_TRY(up(tbas.data(), tbas.size() * sizeof(int), (const void **)&M.ent_band));
    PG_TRY(up(tslot.data(), tslot.size() * sizeof(int), (const void **)&M.ent_slot));
    PG_TRY(up(tcoef.data(), tcoef.size() * sizeof(float), (const void **)&M.ent_coef));
    PG_TRY(up(bas.data(), bas.size() * sizeof(float), (const void **)&M.basis));
    M.nent = (int)tcol.size();
    M.nbasis = (int)basis.size();
    return PG_OK;
}

// Responses [nchunks][CH][kb] of CH-row chunks to their coupling values (see pm_solve_cta), in
// FP64 from the FP64 factor: upper, the chunk's solution of U y = 0 with y = e_q on the first kb
// rows after it; lower, of U^T y = 0 with y = e_q on the last kb rows before it.
static std::vector<double> pm_chunk_tables(const std::vector<double> &U, int N, int kb, int CH, bool lower)
{
    const int kw = kb + 1, nck = (N + CH - 1) / CH;
    std::vector<double> G((size_t)nck * CH * kb, 0.0), y(N, 0.0);
    for (int c = 0; c < nck; ++c) {
        const int r0 = c * CH, len = std::min(CH, N - r0);
        if (lower ? c == 0 : c + 1 >= nck) continue;
        for (int q = 0; q < kb; ++q) {
            std::fill(y.begin(), y.end(), 0.0);
            if (!lower) {
                const int bi = r0 + CH + q;
                if (bi >= N) continue;
                y[bi] = 1.0;
                for (int i = r0 + len - 1; i >= r0; --i) {
                    double s = 0.0;
                    for (int d = 1; d <= kb && i + d < N; ++d) s += U[(size_t)i * kw + d] * y[i + d];
                    y[i] = -s / U[(size_t)i * kw];
                }
            } else {
                y[r0 - kb + q] = 1.0;
                for (int i = r0; i < r0 + len; ++i) {
                    double s = 0.0;
                    for (int d = 1; d <= kb && i - d >= 0; ++d) s += U[(size_t)(i - d) * kw + d] * y[i - d];
                    y[i] = -s / U[(size_t)i * kw];
                }
            }
            for (int r = 0; r < len; ++r) G[((size_t)c * CH + r) * kb + q] = y[r0 + r];
        }
    }
    return G;
}

template <typename T>
static int pm_upload(const std::vector<double> &v, const T **dst, std::vector<void *> &allocs)
{
    std::vector<T> t(v.begin(), v.end());
    void *p = nullptr;
    PG_CUDA_TRY(cudaMalloc(&p, std::max<size_t>(1, t.size()) * sizeof(T)));
    allocs.push_back(p);
    PG_CUDA_TRY(cudaMemcpy(p, t.data(), t.size() * sizeof(T), cudaMemcpyHostToDevice));
    *dst = (const T *)p;
    return PG_OK;
}

int pm_member_tables(PmMember &M, std::vector<void *> &allocs)
{
    if (M.kb < 1 || M.kb > PM_MAXKB || M.N < 1) return PG_ERR_SHAPE;
    const int kw = M.kb + 1;
    std::vector<double> U((size_t)M.N * kw);
    PG_CUDA_TRY(cudaMemcpy(U.data(), M.U64, U.size() * sizeof(double), cudaMemcpyDeviceToHost));
    PG_TRY(pm_upload<float>(pm_chunk_tables(U, M.N, M.kb, 32, false), &M.G32u, allocs));
    PG_TRY(pm_upload<float>(pm_chunk_tables(U, M.N, M.kb, 32, true), &M.G32l, allocs));
    void *tb = nullptr;
    PG_CUDA_TRY(cudaMalloc(&tb, sizeof(cxf) * (size_t)M.m * M.n + 16));
    allocs.push_back(tb);
    M.T = (cxf *)tb;
    return PG_OK;
}

int pm_occupancy(int threads, size_t smem, bool kb6, bool wide)
{
    if (threads > (wide ? 256 : 512)) return 0;
    if (pm_raise_smem(kb6, wide, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pm_kernel(kb6, wide), threads, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return per_sm;
}

int pm_launch(const PmMember *d_members, int nmembers, const int *d_order, unsigned *d_queue, const double *d_dt,
              int threads, int grid, size_t smem, bool kb6, bool wide, cudaStream_t s, int Nmax, int kbmax, int mmax,
              int nchmax, int entmax, int basismax)
{
    if (threads < 32 || threads > (wide ? 256 : 32 * PM_WARPS) || threads % 32 || grid < 1 || nmembers < 1)
        return PG_ERR_ARG;
    if (mmax > PM_MAXM || kbmax > PM_MAXKB) return PG_ERR_SHAPE;
    const PmLayout L = pm_layout(Nmax, kbmax, mmax, nchmax, entmax, basismax);
    if (L.bytes > smem) return PG_ERR_ARG;
    PG_CUDA_TRY(pm_raise_smem(kb6, wide, smem));
    PG_CUDA_TRY(cudaMemsetAsync(d_queue, 0, sizeof(unsigned), s));
    if (kb6 && wide)
        pm_step_kernel<6, 256><<<grid, threads, smem, s>>>(d_members, nmembers, d_order, d_queue, d_dt, L);
    else if (kb6)
        pm_step_kernel<6, 512><<<grid, threads, smem, s>>>(d_members, nmembers, d_order, d_queue, d_dt, L);
    else if (wide)
        pm_step_kernel<-1, 256><<<grid, threads, smem, s>>>(d_members, nmembers, d_order, d_queue, d_dt, L);
    else
        pm_step_kernel<-1, 512><<<grid, threads, smem, s>>>(d_members, nmembers, d_order, d_queue, d_dt, L);
    PG_CUDA_TRY(cudaGetLastError());
    return PG_OK;
}

int pm_max_basis() { return PM_MAXM; }
int pm_max_halfwidth() { return PM_MAXKB; }
