// Single-kernel mixed-precision Cayley / Crank-Nicolson step.
//
// The same scheme as the captured multi-kernel mixed step of cayley.cu (the reference's step:
// pyprop/propagator/CayleyPropagator.py:71-150, GMRES core/krylov/gmres/gmres.h:433-505),
// run as ONE cooperative launch that keeps every SM busy: CTA a < Nang owns angular channel a.
//   r = b - A psi = -i dt H psi                      (FP64, rows spread over all CTAs)
//   per refinement pass (at most 4, while ||r|| > tol):
//     d = M_a^-1 r_a                                 (complex64 block LU solve, in shared memory)
//     GMRES on M^-1 A e = d in complex64, Gram-Schmidt sums in FP64 across channels,
//     Givens rotations and back-substitution in FP32 (the multi-kernel step's arithmetic)
//     psi += e, r -= A e                             (FP64, rows spread over all CTAs)
// Everything a GMRES iteration needs is local to the channel except the matvec (the dipole
// couples neighbouring channels) and two reductions: h1 = <V, w>, then h2 = <V, w'> of
// w' = w - V h1 together with ||w'||^2. The norm of w'' = w' - V h2 follows by Pythagoras,
// ||w''||^2 = ||w'||^2 - ||h2||^2 (w' is already orthogonal to V up to rounding, so there is
// no cancellation), and an iteration costs two grid barriers instead of seven kernel launches.
// The Krylov vectors of channel a live in V[.][a] and are written only by CTA a. The next
// matvec's sources are published as w' in a ping-pong buffer (wbuf) before the second barrier;
// a CTA staging a neighbour's fibre forms that neighbour's w'' = w' - V h2 itself (the same
// arithmetic as the owner, from the neighbour's Krylov vectors, already visible) and scales it
// by 1/beta, so the second correction needs no barrier of its own. Every CTA sums the
// partials in the same order and runs the (tiny) Givens and back-substitution recurrences
// itself, so all CTAs take identical decisions without another barrier. The FP64 parts
// (residual rows, the correction e = V y) are spread over all CTAs: FP64 arithmetic is scarce
// on this GPU. Grid barriers are bounded waits: one that runs out sets the context's error
// flag (2) and the CTAs return.
//
// Qualifying steppers (pg_cayley_fused_prepare): rank-2 operators whose bands are all real
// (the complex factors of a Cayley step are the slot scales), at most FZ_MAXU distinct source
// channels per row, the block-diagonal LU preconditioner, basis size <= FZ_MAXM and no more
// channels than resident CTAs. Launch: one CTA of 768 threads per SM (cooperative). Shared
// memory of a channel CTA: the fibre and the block solve's scratch (tri_solve_smem), the
// staged source fibres of the row product, and, when they fit, the channel's Krylov vectors
// (Gram-Schmidt reads them from there), else the channel's FP32 bands (copied once per step
// while the first FP64 rows run).
#include "fused_common.cuh"

#include <cooperative_groups.h>

#include <algorithm>
#include <cstring>
#include <mutex>

namespace cg = cooperative_groups;

struct FzGivens {
    float cs[FZ_MAXM];
    float sn[2 * FZ_MAXM];
    float g[2 * (FZ_MAXM + 1)];
    float R[2 * FZ_MAXM * FZ_MAXM];  // column-major R[col * FZ_MAXM + row]
};

// New Hessenberg column j (h1 + h2 above the diagonal, beta below) through the previous
// rotations, the new rotation, the updated g; returns the residual estimate |g_{j+1}|. FP32
// as the multi-kernel step's Givens kernel.
__device__ float fz_givens(FzGivens &G, int j, const float *h1, const float *h2, float beta)
{
    const int J = j + 1;
    float hx[FZ_MAXM + 1], hy[FZ_MAXM + 1];
    for (int i = 0; i < J; ++i) {
        hx[i] = h1[2 * i] + h2[2 * i];
        hy[i] = h1[2 * i + 1] + h2[2 * i + 1];
    }
    hx[J] = beta;
    hy[J] = 0.f;
    for (int i = 0; i < j; ++i) {
        const float c = G.cs[i], sx = G.sn[2 * i], sy = G.sn[2 * i + 1];
        const float tx = c * hx[i] + (sx * hx[i + 1] - sy * hy[i + 1]);
        const float ty = c * hy[i] + (sx * hy[i + 1] + sy * hx[i + 1]);
        const float ux = -(sx * hx[i] + sy * hy[i]) + c * hx[i + 1];
        const float uy = -(sx * hy[i] - sy * hx[i]) + c * hy[i + 1];
        hx[i] = tx; hy[i] = ty;
        hx[i + 1] = ux; hy[i + 1] = uy;
    }
    const float a = hypotf(hx[j], hy[j]);
    const float bb = hypotf(hx[j + 1], hy[j + 1]);
    const float r = hypotf(a, bb);
    float c, sx, sy;
    if (r == 0.f) { c = 1.f; sx = 0.f; sy = 0.f; }
    else if (a == 0.f) { c = 0.f; sx = hx[j + 1] / bb; sy = -hy[j + 1] / bb; }
    else {
        c = a / r;
        const float px = hx[j] / a, py = hy[j] / a;
        sx = (px * hx[j + 1] + py * hy[j + 1]) / r;
        sy = (py * hx[j + 1] - px * hy[j + 1]) / r;
    }
    const float rjx = c * hx[j] + (sx * hx[j + 1] - sy * hy[j + 1]);
    const float rjy = c * hy[j] + (sx * hy[j + 1] + sy * hx[j + 1]);
    hx[j] = rjx; hy[j] = rjy;
    G.cs[j] = c;
    G.sn[2 * j] = sx;
    G.sn[2 * j + 1] = sy;
    const float gx = G.g[2 * j], gy = G.g[2 * j + 1];
    const float g1x = -(sx * gx + sy * gy), g1y = -(sx * gy - sy * gx);
    G.g[2 * j] = c * gx;
    G.g[2 * j + 1] = c * gy;
    G.g[2 * (j + 1)] = g1x;
    G.g[2 * (j + 1) + 1] = g1y;
    for (int i = 0; i <= j; ++i) {
        G.R[2 * (j * FZ_MAXM + i)] = hx[i];
        G.R[2 * (j * FZ_MAXM + i) + 1] = hy[i];
    }
    return hypotf(g1x, g1y);
}

// y = R^-1 g over k columns (FP32), stored as complex128
__device__ void fz_backsolve(const FzGivens &G, int k, cxd *ys)
{
    float yx[FZ_MAXM], yy[FZ_MAXM];
    for (int i = k - 1; i >= 0; --i) {
        float sx = G.g[2 * i], sy = G.g[2 * i + 1];
        for (int q = i + 1; q < k; ++q) {
            const float rx = G.R[2 * (q * FZ_MAXM + i)], ry = G.R[2 * (q * FZ_MAXM + i) + 1];
            sx -= rx * yx[q] - ry * yy[q];
            sy -= rx * yy[q] + ry * yx[q];
        }
        const float dx = G.R[2 * (i * FZ_MAXM + i)], dy = G.R[2 * (i * FZ_MAXM + i) + 1];
        const float den = dx * dx + dy * dy;
        if (den > 0.f) {
            yx[i] = (sx * dx + sy * dy) / den;
            yy[i] = (sy * dx - sx * dy) / den;
        } else {
            yx[i] = 0.f;
            yy[i] = 0.f;
        }
    }
    for (int i = 0; i < k; ++i) ys[i] = mk<double>((double)yx[i], (double)yy[i]);
}

struct FzCtl {
    int j, cont, k, again, passes, ok;
    double tol_eff;
    float tol_f;  // tol_eff in FP32, for the per-iteration test
    float s;      // 1/beta for the next Krylov vector (formed once: FP64 division is slow here)
};

template <int KB>
__global__ void __launch_bounds__(FZ_THREADS, 1) cay_fused_step_kernel(FzArgs a)
{
    if (fz_bad_launch(a, gridDim.x != (unsigned)a.nctas || gridDim.y != 1 || gridDim.z != 1)) return;
    // the previous launch, which used bar_next, has completed: clear it for the next launch
    if (blockIdx.x == 0 && threadIdx.x == 0) a.bar_next->count = 0;
    extern __shared__ __align__(16) unsigned char fz_smem[];
    __shared__ cxd sc_diff[PG_MAX_SLOTS], sc_negplus[PG_MAX_SLOTS];
    __shared__ cxf sc_plus[PG_MAX_SLOTS];
    __shared__ double red[FZ_NW][2 * FZ_CB];
    __shared__ double hd[1];  // FP64 sums of the pass: ||d||^2, then ||r||^2
    __shared__ float hf[2][FZ_PSTRIDE];  // the Gram-Schmidt sums h1 and h2 of this iteration
    __shared__ cxf hs[FZ_MAXM];
    __shared__ cxd ys[FZ_MAXM];
    __shared__ FzGivens G;
    __shared__ FzCtl ctl;

    const int ch = blockIdx.x;                 // angular channel of this CTA (when < nch)
    const bool owner = ch < a.nch;
    const int tid = threadIdx.x;
    const int N = a.N, nblk = a.nblk, w = a.w, npad = nblk * 32;
    const long long n = (long long)a.nch * N;
    const long long lo = __ldg(a.row_lo + ch), hi = __ldg(a.row_lo + ch + 1);  // FP64 rows of this CTA
    cxf *xs = (cxf *)fz_smem;                  // [nblk*32] the channel's fibre
    cxf *sb = xs + (size_t)npad;               // [nblk*w]
    cxf *sg = sb + (size_t)nblk * w;           // [nblk][w][32] (g_in_smem)
    cxf *xsrc = sg + (a.g_in_smem ? (size_t)nblk * w * 32 : 0);  // [FZ_MAXU][N + 2kb] staged sources
    // [entries][2kb+1][ld] this channel's FP32 bands (16-byte aligned), when they fit
    const size_t mat = (size_t)(owner ? ch / a.fib_per_mat : 0);
    cxf *Vc = a.V + (size_t)(owner ? ch : 0) * N;  // V[q][ch] at Vc + q * n
    unsigned char *extra = fz_smem + ((((size_t)npad + (size_t)nblk * w * (a.g_in_smem ? 33 : 1) +
                                       (size_t)FZ_MAXU * (N + 2 * a.opb.kb)) * sizeof(cxf) + 15) / 16) * 16;
    float *sband = (owner && a.bands_smem) ? (float *)extra : nullptr;
    // [m][N] this channel's Krylov vectors, when they fit (read by the same thread that wrote
    // each row; the global copy serves the correction e = V y of the other CTAs)
    cxf *sV = (owner && a.v_smem) ? (cxf *)extra : nullptr;
    const cxf *Vr = sV ? sV : Vc;
    const long long vld = sV ? (long long)N : n;
    const size_t pstride = (size_t)gridDim.x * FZ_PSTRIDE;
    double *part_me = a.part + (size_t)ch * FZ_PSTRIDE;  // + phase * pstride
    unsigned int expect = 0;   // barrier arrivals expected so far (thread 0)
    unsigned int ordinal = 0;  // barriers met so far (thread 0)
    const bool lead = (ch == 0 && tid == 0);  // keeps the step statistics

    if (tid < PG_MAX_SLOTS) {
        const double hdt = 0.5 * a.params.dt;
        const cxd h = a.params.h[tid];
        cxd plus, diff;
        if (tid == 0) {
            plus = mk<double>(1.0, 0.0);
            diff = mk<double>(0.0, 0.0);
        } else {
            plus = mk<double>(-hdt * h.y, hdt * h.x);
            diff = mk<double>(2.0 * hdt * h.y, -2.0 * hdt * h.x);
        }
        sc_plus[tid] = cvt<float>(plus);
        sc_diff[tid] = diff;
        sc_negplus[tid] = mk<double>(-plus.x, -plus.y);
    }
    if (lead) {
        a.st->stats.iterations = 0;
        a.st->stats.passes = 0;
        a.st->stats.true_resid = -1.0;
        a.st->stats.kernels += 1;
    }
    if (tid == 0) ctl.passes = 0;
    __syncthreads();

    // this channel's FP32 bands to shared memory, in flight during the first FP64 rows
    if (sband) fz_bands_load(a, ch, sband);
    // r = -i dt H psi (FP64); psi is read by all CTAs before the first barrier and only
    // changed after the second
    fz_rows64<KB>(a.op64, a.rb64, lo, hi, sc_diff, a.psi, a.r64, false);
    if (sband) fz_bands_wait();  // before any exit: no copy outlives the CTA
    if (!fz_grid_sync(a.bar, expect, ordinal, a, &ctl.ok)) return;

    for (;;) {
        // d = M^-1 r (complex64), published for the first matvec; ||d||^2
        if (owner) {
            for (int i = tid; i < npad; i += FZ_THREADS) {
                cxf v = mk<float>(0.f, 0.f);
                if (i < N) {
                    const cxd r = fz_ldcg(a.r64 + (size_t)ch * N + i);
                    v = mk<float>((float)r.x, (float)r.y);
                }
                xs[i] = v;
            }
            __syncthreads();
            tri_solve_smem<float, cxf, FZ_NW>(nblk, w, mat, a.lo_inv, a.lo_g, a.lo_rb, a.up_inv, a.up_g, a.up_rb, 1,
                                              1, a.g_in_smem, xs, sb, sg);
            for (int i = tid; i < N; i += FZ_THREADS) a.wbuf[(size_t)ch * N + i] = xs[i];
            fz_channel_sums(Vr, vld, 0, true, xs, N, red, part_me + P_NRM * pstride);
        }
        if (!fz_grid_sync(a.bar, expect, ordinal, a, &ctl.ok)) return;
        fz_reduce(a.part + P_NRM * pstride, a.nch, 1, hd);
        if (tid == 0) {
            const double b = sqrt(fmax(hd[0], 0.0));
            ctl.s = (float)(b > 0.0 ? 1.0 / b : 0.0);
            ctl.tol_eff = fmax(a.tol, 2e-6 * b);
            ctl.tol_f = (float)ctl.tol_eff;
            ctl.j = 0;
            ctl.k = 0;
            ctl.cont = b > 0.0 ? 1 : 0;
            ctl.passes += 1;
            G.g[0] = (float)b;
            G.g[1] = 0.f;
            if (lead) {
                a.st->stats.k = 0;
                a.st->stats.beta0 = b;
                a.st->stats.resid = b;
                a.st->stats.passes = ctl.passes;
                a.st->stats.cum_passes += 1;
            }
        }
        __syncthreads();

        while (ctl.cont) {
            const int j = ctl.j, J = j + 1;
            const float s = ctl.s;
            if (owner) {
                // V_j = w'' / beta (this channel), then xs = M^-1 A V_j (row ch); the staged
                // sources are the channels' w' with the previous iteration's second correction
                // (hs = h2, j vectors) applied while staging
                for (int i = tid; i < N; i += FZ_THREADS) {
                    const cxf v = xs[i];
                    const cxf vs = mk<float>(v.x * s, v.y * s);
                    Vc[(size_t)j * n + i] = vs;
                    if (sV) sV[(size_t)j * N + i] = vs;
                }
                fz_matvec32<KB>(a, ch, sc_plus, a.wbuf + (size_t)(j & 1) * n, s, xs, npad, xsrc, sband, j, hs);
                __syncthreads();
                tri_solve_smem<float, cxf, FZ_NW>(nblk, w, mat, a.lo_inv, a.lo_g, a.lo_rb, a.up_inv, a.up_g, a.up_rb,
                                                  1, 1, a.g_in_smem, xs, sb, sg);
                // classical Gram-Schmidt, twice: h1 = <V, w>, w' = w - V h1, h2 = <V, w'>, w'' = w' - V h2
                fz_channel_sums(Vr, vld, J, false, xs, N, red, part_me + P_H1 * pstride);
            }
            if (!fz_grid_sync(a.bar, expect, ordinal, a, &ctl.ok)) return;
            fz_reduce(a.part + P_H1 * pstride, a.nch, 2 * J, hf[0]);
            if (owner) {
                if (tid < J) hs[tid] = mk<float>(hf[0][2 * tid], hf[0][2 * tid + 1]);
                __syncthreads();
                // w' = w - V h1, published for the next products; then h2 and ||w'||^2
                for (int i = tid; i < N; i += FZ_THREADS) {
                    const cxf acc = fz_gs_update<false>(xs[i], Vr + i, vld, J, hs);
                    xs[i] = acc;
                    a.wbuf[(size_t)((j + 1) & 1) * n + (size_t)ch * N + i] = acc;
                }
                __syncthreads();
                fz_channel_sums(Vr, vld, J, false, xs, N, red, part_me + P_H2 * pstride, true);
            }
            if (!fz_grid_sync(a.bar, expect, ordinal, a, &ctl.ok)) return;
            fz_reduce(a.part + P_H2 * pstride, a.nch, 2 * J, hf[1]);
            fz_reduce(a.part + P_H2 * pstride + 2 * J, a.nch, 1, hd);
            if (owner) {
                if (tid < J) hs[tid] = mk<float>(hf[1][2 * tid], hf[1][2 * tid + 1]);
                __syncthreads();
                // w'' = w' - V h2 (kept for the next iteration; the other CTAs form it themselves)
                for (int i = tid; i < N; i += FZ_THREADS) xs[i] = fz_gs_update<false>(xs[i], Vr + i, vld, J, hs);
            }
            if (tid == 0) {
                // ||w''||^2 = ||w'||^2 - ||h2||^2 (FP64), beta in FP32 (it enters the Hessenberg
                // matrix and the next vector as FP32)
                double b2 = hd[0];
                for (int q = 0; q < J; ++q) b2 -= (double)hf[1][2 * q] * hf[1][2 * q] + (double)hf[1][2 * q + 1] * hf[1][2 * q + 1];
                const float fb = (float)sqrt(fmax(b2, 0.0));
                const float resid = fz_givens(G, j, hf[0], hf[1], fb);
                const bool bad = !(resid == resid);
                const bool conv = bad || resid <= ctl.tol_f || J >= a.m || !(fb > 0.f);
                ctl.k = J;
                ctl.s = fb > 0.f ? 1.f / fb : 0.f;
                ctl.cont = conv ? 0 : 1;
                if (!conv) ctl.j = j + 1;
                if (lead) {
                    a.st->stats.k = J;
                    a.st->stats.resid = resid;
                    a.st->stats.iterations += 1;
                    a.st->stats.cum_iterations += 1;
                }
            }
            __syncthreads();
        }

        // e = V y (FP64, this CTA's rows; V read through L2), psi += e, e published
        if (tid == 0) fz_backsolve(G, ctl.k, ys);
        __syncthreads();
        const int k = ctl.k;
        for (long long o = lo + tid; o < hi; o += FZ_THREADS) {
            double ax = 0.0, ay = 0.0;
            for (int q0 = 0; q0 < k; q0 += FZ_CB) {
                cxf v[FZ_CB];
#pragma unroll
                for (int q = 0; q < FZ_CB; ++q)
                    v[q] = q0 + q < k ? fz_ldcg(a.V + (size_t)(q0 + q) * n + o) : mk<float>(0.f, 0.f);
#pragma unroll
                for (int q = 0; q < FZ_CB; ++q) {
                    if (q0 + q >= k) break;
                    const cxd yq = ys[q0 + q];
                    ax = fma((double)v[q].x, yq.x, ax); ax = fma(-(double)v[q].y, yq.y, ax);
                    ay = fma((double)v[q].x, yq.y, ay); ay = fma((double)v[q].y, yq.x, ay);
                }
            }
            a.e64[o] = mk<double>(ax, ay);
            a.psi[o] = a.psi[o] + mk<double>(ax, ay);
        }
        if (!fz_grid_sync(a.bar, expect, ordinal, a, &ctl.ok)) return;
        // r -= (S + i dt/2 H) e in FP64; ||r|| decides whether another pass runs
        const double rn = fz_rows64<KB>(a.op64, a.rb64, lo, hi, sc_negplus, a.e64, a.r64, true);
        fz_cta_sum64(rn, red, part_me + P_RES * pstride);
        if (!fz_grid_sync(a.bar, expect, ordinal, a, &ctl.ok)) return;
        fz_reduce(a.part + P_RES * pstride, gridDim.x, 1, hd);
        if (tid == 0) {
            const double r = sqrt(fmax(hd[0], 0.0));
            ctl.again = (r > a.tol) && (r == r) && ctl.passes < FZ_MAXPASS;
            if (lead) a.st->stats.true_resid = r;
        }
        __syncthreads();
        if (!ctl.again) break;
    }
    // the step's statistics and the error word to the host (mapped memory): the last action
    if (lead && a.hstats) {
        *a.hstats = a.st->stats;
        *(volatile int *)a.herr = *(volatile int *)a.err;  // read by the host after it synchronises
    }
}

// ------------------------------------------------------------------------------------
// the same step with each channel split over a cluster of three CTAs
// ------------------------------------------------------------------------------------
// CTA rank cr of cluster c < Nang owns the fibre blocks [cr bpc, (cr+1) bpc) of channel c and
// keeps those blocks' solve factors (inverse diagonal blocks, couplings) and its third of the
// rows of the boundary-system inverses in shared memory for the whole step: the factors are
// read from HBM/L2 once per step instead of once per solve. The block solves exchange their
// boundary values through distributed shared memory between cluster barriers; the row
// product, the Gram-Schmidt updates and the channel sums run on each CTA's own rows. The
// FP64 rows, the correction e = V y and every decision are those of the single-CTA kernel.
// Grid barriers: every CTA arrives and polls as in the single-CTA kernel; then the three CTAs
// of a cluster meet once and each reads the three outcomes, so they all take the same
// decision. On a wait that ran out they meet once more and leave together: no CTA leaves
// while a peer could still read its shared memory.
static const int CL_SIZE = 3;

__device__ __forceinline__ bool cl_grid_sync(FzBarrier *bar, unsigned int &target, unsigned int &ordinal,
                                             const FzArgs &a, int *s_ok, int *s_all, cg::cluster_group &cluster)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        target += gridDim.x + (ordinal == a.probe_at ? a.probe_extra : 0u);
        ++ordinal;
        __threadfence();
        atomicAdd(&bar->count, 1u);
        unsigned int polls = 0;
        while (fz_ld_acquire(&bar->count) < target) {
            if (++polls > FZ_POLLS) { ok = 0; break; }
            __nanosleep(32);
        }
        if (!ok) {
            atomicExch(a.err, 2);
            if (a.herr) *(volatile int *)a.herr = 2;
        }
        *s_ok = ok;
    }
    cluster.sync();
    if (threadIdx.x == 0) {
        int all = 1;
        for (unsigned int r = 0; r < (unsigned int)CL_SIZE; ++r) all &= *cluster.map_shared_rank(s_ok, r);
        *s_all = all;
    }
    __syncthreads();
    if (*s_all) return true;
    cluster.sync();  // the peers have read this CTA's outcome
    return false;
}

__device__ __forceinline__ unsigned cl_smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
// 1-D bulk copy (TMA) global -> this CTA's shared memory, completing on the mbarrier
__device__ __forceinline__ void cl_bulk(void *dst, const void *src, unsigned bytes, unsigned long long *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                     cl_smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(cl_smem_u32(bar))
                 : "memory");
}
// bounded wait for phase 0 of the factor mbarrier; false (error word 3) when it runs out
__device__ __forceinline__ bool cl_bar_wait(unsigned long long *bar, int *err)
{
    for (long long it = 0; it < (1LL << 26); ++it) {
        unsigned done;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(done)
                     : "r"(cl_smem_u32(bar)), "r"(0u)
                     : "memory");
        if (done) return true;
    }
    atomicExch(err, 3);
    return false;
}

// 8-byte asynchronous global -> shared copy (cp.async; waited for by fz_bands_wait)
__device__ __forceinline__ void cl_cp8(void *dst, const void *src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
}

struct ClSolve {
    const cxf *inv_lo, *inv_up, *g_lo, *g_up, *rb;  // this CTA's factors (shared memory)
    const int *off_lo, *off_up;                      // packed Rb row offsets (lower, upper)
    cxf *zloc, *zall, *sloc, *sall;
    int nblk, w, nb, bpc, rpc, b0, nown, r_first, nrows;
};

// Both sweeps of the blocked triangular solve (the algorithm of tri_solve_smem) on a fibre
// split over the cluster: xs holds this CTA's blocks (local rows). Per sweep: z_b = T_b^-1 f_b
// for the own blocks; the boundary rows of every block gathered from the peers; this CTA's
// rows of s = Rb z (lower sweep: columns [0, (bo+1) w), upper: [bo w, nb)); s gathered; the
// corrections y_b = z_b - G_b s of the neighbouring block. Returns after a CTA barrier.
__device__ __forceinline__ void cl_tri_solve(const ClSolve &S, cxf *xs, cg::cluster_group &cluster)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int w = S.w, nb = S.nb;
    for (int sweep = 0; sweep < 2; ++sweep) {
        const bool lower = sweep == 0;
        const cxf *inv = lower ? S.inv_lo : S.inv_up;
        const cxf *g = lower ? S.g_lo : S.g_up;
        const int *off = lower ? S.off_lo : S.off_up;
        const int r0 = lower ? 32 - w : 0;
        for (int lb = warp; lb < S.nown; lb += FZ_NW) {
            const cxf *ib = inv + (size_t)lb * 1024;
            const cxf f = xs[lb * 32 + lane];
            cxf acc[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[q] = mk<float>(0.f, 0.f);
#pragma unroll
            for (int q = 0; q < 32; ++q) cfma(acc[q & 3], ib[q * 32 + lane], shfl_cx(f, q));
            const cxf z = (acc[0] + acc[1]) + (acc[2] + acc[3]);
            xs[lb * 32 + lane] = z;
            if (lane >= r0 && lane < r0 + w) S.zloc[(S.b0 + lb) * w + (lane - r0)] = z;
        }
        cluster.sync();
        for (int c = threadIdx.x; c < nb; c += FZ_THREADS)
            S.zall[c] = *cluster.map_shared_rank(S.zloc + c, (unsigned int)((c / w) / S.bpc));
        __syncthreads();
        for (int lr = warp; lr < S.nrows; lr += FZ_NW) {
            const int r = S.r_first + lr, bo = r / w;
            const int c0 = lower ? 0 : bo * w, len = lower ? (bo + 1) * w : nb - bo * w;
            const cxf *row = S.rb + off[lr];
            cxf acc = mk<float>(0.f, 0.f);
            for (int c = lane; c < len; c += 32) cfma(acc, row[c], S.zall[c0 + c]);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
                acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
            }
            if (lane == 0) S.sloc[lr] = acc;
        }
        cluster.sync();
        for (int c = threadIdx.x; c < nb; c += FZ_THREADS) {
            const int rk = c / S.rpc;
            S.sall[c] = *cluster.map_shared_rank(S.sloc + (c - rk * S.rpc), (unsigned int)rk);
        }
        __syncthreads();
        for (int lb = warp; lb < S.nown; lb += FZ_NW) {
            const int blk = S.b0 + lb, nbk = lower ? blk - 1 : blk + 1;
            cxf y = xs[lb * 32 + lane];
            if (nbk >= 0 && nbk < S.nblk) {
                const cxf *gb = g + (size_t)lb * w * 32;
                for (int c = 0; c < w; ++c) coef_fms(y, gb[c * 32 + lane], S.sall[nbk * w + c]);
            }
            xs[lb * 32 + lane] = y;
        }
        __syncthreads();
    }
}

// Row product of fz_matvec32 restricted to the rows [row0, row0 + nloc) of channel a (nlocpad
// local rows written, zero past nloc): sources staged over [row0 - kb, row0 + nloc + kb).
template <int KB>
__device__ __forceinline__ void cl_matvec32(const FzArgs &A, int a, const cxf *sc, const cxf *wsrc, float s, cxf *xs,
                                            int row0, int nloc, int nlocpad, cxf *xsrc, int Jc, const cxf *hs)
{
    const OpDev &op = A.opb;
    const long long nall = (long long)A.nch * A.N;
    const int N = op.N, kb = KB >= 0 ? KB : op.kb, b = 2 * kb + 1, ld = op.ld, W = nloc + 2 * kb;
    const int nu = __ldg(A.nucol + a);
    int cols[FZ_MAXU];
#pragma unroll
    for (int u = 0; u < FZ_MAXU; ++u) cols[u] = u < nu ? __ldg(A.ucol + (size_t)a * FZ_MAXU + u) : 0;
    for (int base = 0; base < nu * W; base += FZ_THREADS * FZ_MAXU) {
        cxf v[FZ_MAXU];
#pragma unroll
        for (int k = 0; k < FZ_MAXU; ++k) {
            const int idx = base + threadIdx.x + k * FZ_THREADS;
            const int u = idx / W, q = idx - u * W, j = row0 + q - kb;
            v[k] = (idx < nu * W && j >= 0 && j < N) ? fz_ldcg(wsrc + (size_t)cols[u < FZ_MAXU ? u : 0] * N + j)
                                                     : mk<float>(0.f, 0.f);
        }
        if (Jc > 0) {
#pragma unroll
            for (int k = 0; k < FZ_MAXU; ++k) {
                const int idx = base + threadIdx.x + k * FZ_THREADS;
                const int u = idx / W, q = idx - u * W, j = row0 + q - kb;
                if (idx < nu * W && j >= 0 && j < N)
                    v[k] = fz_gs_update<true>(v[k], A.V + (size_t)cols[u < FZ_MAXU ? u : 0] * N + j, nall, Jc, hs);
            }
        }
#pragma unroll
        for (int k = 0; k < FZ_MAXU; ++k) {
            const int idx = base + threadIdx.x + k * FZ_THREADS;
            if (idx < nu * W) xsrc[idx] = mk<float>(v[k].x * s, v[k].y * s);
        }
    }
    __syncthreads();
    const int e0 = __ldg(op.row_ptr + a), e1 = __ldg(op.row_ptr + a + 1);
    for (int i = threadIdx.x; i < nlocpad; i += FZ_THREADS) {
        cxf acc = mk<float>(0.f, 0.f);
        if (i < nloc) {
            const int gi = row0 + i;
            for (int e = e0; e < e1; e += 2) {
                const bool two = e + 1 < e1;
                const int e1s = two ? e + 1 : e;
                const float *B0 = A.rb32 + (size_t)__ldg(op.ent_band + e) * b * ld + gi;
                const float *B1 = A.rb32 + (size_t)__ldg(op.ent_band + e1s) * b * ld + gi;
                const cxf *x0 = xsrc + (size_t)__ldg(A.ent_u + e) * W + i;  // x[d] = x_e[gi + d - kb]
                const cxf *x1 = xsrc + (size_t)__ldg(A.ent_u + e1s) * W + i;
                float t0x = 0.f, t0y = 0.f, t1x = 0.f, t1y = 0.f;
                if (KB >= 0) {
                    float c0[2 * (KB > 0 ? KB : 0) + 1], c1[2 * (KB > 0 ? KB : 0) + 1];
#pragma unroll
                    for (int d = 0; d < 2 * KB + 1; ++d) {
                        c0[d] = __ldg(B0 + (size_t)d * ld);
                        c1[d] = __ldg(B1 + (size_t)d * ld);
                    }
#pragma unroll
                    for (int d = 0; d < 2 * KB + 1; ++d) {
                        t0x = fmaf(c0[d], x0[d].x, t0x);
                        t0y = fmaf(c0[d], x0[d].y, t0y);
                        t1x = fmaf(c1[d], x1[d].x, t1x);
                        t1y = fmaf(c1[d], x1[d].y, t1y);
                    }
                } else {
                    for (int d = 0; d < b; ++d) {
                        const float c = __ldg(B0 + (size_t)d * ld), c2 = __ldg(B1 + (size_t)d * ld);
                        t0x = fmaf(c, x0[d].x, t0x);
                        t0y = fmaf(c, x0[d].y, t0y);
                        t1x = fmaf(c2, x1[d].x, t1x);
                        t1y = fmaf(c2, x1[d].y, t1y);
                    }
                }
                cfma(acc, sc[__ldg(op.ent_slot + e)], mk<float>(t0x, t0y));
                if (two) cfma(acc, sc[__ldg(op.ent_slot + e + 1)], mk<float>(t1x, t1y));
            }
        }
        xs[i] = acc;
    }
}

// Shared-memory layout of the cluster kernel (byte offsets; every piece 16-byte aligned)
struct ClLayout {
    size_t inv_lo, inv_up, g_lo, g_up, rb, xs, zloc, zall, sloc, sall, xsrc, off_lo, off_up, bytes;
};
__host__ __device__ inline size_t cl_take(size_t &o, size_t bytes)
{
    const size_t at = o;
    o = (o + bytes + 15) / 16 * 16;
    return at;
}
__host__ __device__ inline ClLayout cl_layout(int bpc, int w, int nb, int rpc, int rbmax, int kb)
{
    ClLayout L;
    size_t o = 0;
    L.inv_lo = cl_take(o, (size_t)bpc * 1024 * sizeof(cxf));
    L.inv_up = cl_take(o, (size_t)bpc * 1024 * sizeof(cxf));
    L.g_lo = cl_take(o, (size_t)bpc * w * 32 * sizeof(cxf));
    L.g_up = cl_take(o, (size_t)bpc * w * 32 * sizeof(cxf));
    L.rb = cl_take(o, (size_t)rbmax * sizeof(cxf));
    L.xs = cl_take(o, (size_t)bpc * 32 * sizeof(cxf));
    L.zloc = cl_take(o, (size_t)nb * sizeof(cxf));
    L.zall = cl_take(o, (size_t)nb * sizeof(cxf));
    L.sloc = cl_take(o, (size_t)rpc * sizeof(cxf));
    L.sall = cl_take(o, (size_t)nb * sizeof(cxf));
    L.xsrc = cl_take(o, (size_t)FZ_MAXU * (bpc * 32 + 2 * kb) * sizeof(cxf));
    L.off_lo = cl_take(o, (size_t)(rpc + 1) * sizeof(int));
    L.off_up = cl_take(o, (size_t)(rpc + 1) * sizeof(int));
    L.bytes = o;
    return L;
}

template <int KB>
__global__ void __launch_bounds__(FZ_THREADS, 1) cay_cluster_step_kernel(FzArgs a)
{
    extern __shared__ __align__(16) unsigned char fz_smem[];
    __shared__ cxd sc_diff[PG_MAX_SLOTS], sc_negplus[PG_MAX_SLOTS];
    __shared__ cxf sc_plus[PG_MAX_SLOTS];
    __shared__ double red[FZ_NW][2 * FZ_CB];
    __shared__ double hd[1];
    __shared__ float hf[2][FZ_PSTRIDE];
    __shared__ cxf hs[FZ_MAXM];
    __shared__ cxd ys[FZ_MAXM];
    __shared__ FzGivens G;
    __shared__ FzCtl ctl;
    __shared__ int s_ok, s_all;
    __shared__ __align__(8) unsigned long long fbar;  // the factor copies' mbarrier

    cg::cluster_group cluster = cg::this_cluster();
    if (fz_bad_launch(a, cluster.num_blocks() != CL_SIZE || gridDim.x != (unsigned)a.nctas || gridDim.y != 1 ||
                             gridDim.z != 1))
        return;
    if (blockIdx.x == 0 && threadIdx.x == 0) a.bar_next->count = 0;  // as in cay_fused_step_kernel
    const int cl = blockIdx.x / CL_SIZE;            // cluster: angular channel (when < nch)
    const int cr = (int)cluster.block_rank();       // this CTA's part of the channel
    const bool owner = cl < a.nch;
    const int ch = owner ? cl : 0;
    const int tid = threadIdx.x;
    const int N = a.N, nblk = a.nblk, w = a.w, nb = nblk * w, bpc = a.cl_bpc, rpc = a.cl_rpc;
    const long long n = (long long)a.nch * N;
    const long long lo = __ldg(a.row_lo + blockIdx.x), hi = __ldg(a.row_lo + blockIdx.x + 1);
    const int b0 = min(nblk, cr * bpc), nown = min(nblk, b0 + bpc) - b0;
    const int row0 = b0 * 32, nloc = max(0, min(N, row0 + nown * 32) - row0), nlocpad = nown * 32;
    const int r_first = min(nb, cr * rpc), nrows = min(nb, r_first + rpc) - r_first;
    const ClLayout L = cl_layout(bpc, w, nb, rpc, a.cl_rbmax, a.opb.kb);
    cxf *xs = (cxf *)(fz_smem + L.xs);
    cxf *xsrc = (cxf *)(fz_smem + L.xsrc);
    int *off_lo = (int *)(fz_smem + L.off_lo);
    int *off_up = (int *)(fz_smem + L.off_up);
    ClSolve S;
    S.inv_lo = (const cxf *)(fz_smem + L.inv_lo);
    S.inv_up = (const cxf *)(fz_smem + L.inv_up);
    S.g_lo = (const cxf *)(fz_smem + L.g_lo);
    S.g_up = (const cxf *)(fz_smem + L.g_up);
    S.rb = (const cxf *)(fz_smem + L.rb);
    S.off_lo = off_lo;
    S.off_up = off_up;
    S.zloc = (cxf *)(fz_smem + L.zloc);
    S.zall = (cxf *)(fz_smem + L.zall);
    S.sloc = (cxf *)(fz_smem + L.sloc);
    S.sall = (cxf *)(fz_smem + L.sall);
    S.nblk = nblk; S.w = w; S.nb = nb; S.bpc = bpc; S.rpc = rpc; S.b0 = b0; S.nown = nown;
    S.r_first = r_first; S.nrows = nrows;
    const size_t mat = (size_t)(owner ? ch / a.fib_per_mat : 0);
    cxf *Vc = a.V + (size_t)ch * N + row0;  // this CTA's rows of V[q][ch] at Vc + q * n
    const size_t pstride = (size_t)gridDim.x * FZ_PSTRIDE;
    double *part_me = a.part + (size_t)blockIdx.x * FZ_PSTRIDE;
    const int nown_ctas = a.nch * CL_SIZE;  // the channel phases' partial sums come from these CTAs
    unsigned int expect = 0, ordinal = 0;
    const bool lead = (blockIdx.x == 0 && tid == 0);

    if (tid < PG_MAX_SLOTS) {
        const double hdt = 0.5 * a.params.dt;
        const cxd h = a.params.h[tid];
        cxd plus, diff;
        if (tid == 0) {
            plus = mk<double>(1.0, 0.0);
            diff = mk<double>(0.0, 0.0);
        } else {
            plus = mk<double>(-hdt * h.y, hdt * h.x);
            diff = mk<double>(2.0 * hdt * h.y, -2.0 * hdt * h.x);
        }
        sc_plus[tid] = cvt<float>(plus);
        sc_diff[tid] = diff;
        sc_negplus[tid] = mk<double>(-plus.x, -plus.y);
    }
    if (lead) {
        a.st->stats.iterations = 0;
        a.st->stats.passes = 0;
        a.st->stats.true_resid = -1.0;
        a.st->stats.kernels += 1;
    }
    if (tid == 0) ctl.passes = 0;
    __syncthreads();  // the slot scales
    const bool bulk = (w % 2) == 0;  // every factor piece 16-byte aligned and sized: bulk copies
    if (owner) {
        // packed Rb row offsets, then the factors of this CTA's blocks and Rb rows, in flight
        // while the first FP64 rows run. Bulk copies: warp 0 issues them (lane 0 registers the
        // byte count on the mbarrier first) and the other warps start the rows at once.
        if (tid < 32) {
            if (tid == 0) {
                int ol = 0;
                for (int lr = 0; lr < nrows; ++lr) {
                    off_lo[lr] = ol;
                    ol += ((r_first + lr) / w + 1) * w;
                }
                off_lo[nrows] = ol;
                int ou = ol;
                for (int lr = 0; lr < nrows; ++lr) {
                    off_up[lr] = ou;
                    ou += nb - ((r_first + lr) / w) * w;
                }
                off_up[nrows] = ou;
            }
            __syncwarp();
        }
        const size_t fb = mat * nblk + b0;
        const cxf *RbL = a.lo_rb + mat * (size_t)nb * nb, *RbU = a.up_rb + mat * (size_t)nb * nb;
        if (bulk) {
            if (tid < 32) {
                const unsigned inv_bytes = (unsigned)(nown * 1024 * sizeof(cxf));
                const unsigned g_bytes = (unsigned)(nown * w * 32 * sizeof(cxf));
                if (tid == 0) {
                    const unsigned total = 2 * inv_bytes + 2 * g_bytes + (unsigned)(off_up[nrows] * sizeof(cxf));
                    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(cl_smem_u32(&fbar)), "r"(1u)
                                 : "memory");
                    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(cl_smem_u32(&fbar)),
                                 "r"(total)
                                 : "memory");
                }
                __syncwarp();
                // pieces: 4 blocks of factors (when this CTA owns blocks), then 2 per Rb row
                const int npieces = (inv_bytes ? 4 : 0) + 2 * nrows;
                for (int q = tid; q < npieces; q += 32) {
                    const int qq = inv_bytes ? q : q + 4;
                    if (qq == 0) cl_bulk(fz_smem + L.inv_lo, a.lo_inv + fb * 1024, inv_bytes, &fbar);
                    else if (qq == 1) cl_bulk(fz_smem + L.inv_up, a.up_inv + fb * 1024, inv_bytes, &fbar);
                    else if (qq == 2) cl_bulk(fz_smem + L.g_lo, a.lo_g + fb * w * 32, g_bytes, &fbar);
                    else if (qq == 3) cl_bulk(fz_smem + L.g_up, a.up_g + fb * w * 32, g_bytes, &fbar);
                    else {
                        const int lr = (qq - 4) >> 1, r = r_first + lr, bo = r / w;
                        if (((qq - 4) & 1) == 0)
                            cl_bulk((cxf *)(fz_smem + L.rb) + off_lo[lr], RbL + (size_t)r * nb,
                                    (unsigned)((bo + 1) * w * sizeof(cxf)), &fbar);
                        else
                            cl_bulk((cxf *)(fz_smem + L.rb) + off_up[lr], RbU + (size_t)r * nb + bo * w,
                                    (unsigned)((nb - bo * w) * sizeof(cxf)), &fbar);
                    }
                }
            }
        } else {
            __syncthreads();  // the offsets
            for (int q = tid; q < nown * 1024; q += FZ_THREADS) {
                cl_cp8((cxf *)(fz_smem + L.inv_lo) + q, a.lo_inv + fb * 1024 + q);
                cl_cp8((cxf *)(fz_smem + L.inv_up) + q, a.up_inv + fb * 1024 + q);
            }
            for (int q = tid; q < nown * w * 32; q += FZ_THREADS) {
                cl_cp8((cxf *)(fz_smem + L.g_lo) + q, a.lo_g + fb * w * 32 + q);
                cl_cp8((cxf *)(fz_smem + L.g_up) + q, a.up_g + fb * w * 32 + q);
            }
            for (int lr = 0; lr < nrows; ++lr) {
                const int r = r_first + lr, bo = r / w;
                const int nl = (bo + 1) * w, nu = nb - bo * w;
                for (int c = tid; c < nl + nu; c += FZ_THREADS) {
                    if (c < nl) cl_cp8((cxf *)(fz_smem + L.rb) + off_lo[lr] + c, RbL + (size_t)r * nb + c);
                    else
                        cl_cp8((cxf *)(fz_smem + L.rb) + off_up[lr] + (c - nl),
                               RbU + (size_t)r * nb + bo * w + (c - nl));
                }
            }
            asm volatile("cp.async.commit_group;" ::: "memory");
        }
    }

    // r = -i dt H psi (FP64, rows spread over all CTAs)
    fz_rows64<KB>(a.op64, a.rb64, lo, hi, sc_diff, a.psi, a.r64, false);
    if (owner) {
        // the factors are in shared memory (and no copy outlives the CTA)
        if (bulk) {
            if (tid == 0 && !cl_bar_wait(&fbar, a.err)) cl_bar_wait(&fbar, a.err);
            __syncthreads();
        } else {
            fz_bands_wait();
        }
    }
    if (!cl_grid_sync(a.bar, expect, ordinal, a, &s_ok, &s_all, cluster)) return;

    for (;;) {
        // d = M^-1 r (complex64) on the own rows, published for the first product; ||d||^2
        if (owner) {
            for (int i = tid; i < nlocpad; i += FZ_THREADS) {
                cxf v = mk<float>(0.f, 0.f);
                if (i < nloc) {
                    const cxd r = fz_ldcg(a.r64 + (size_t)ch * N + row0 + i);
                    v = mk<float>((float)r.x, (float)r.y);
                }
                xs[i] = v;
            }
            __syncthreads();
            cl_tri_solve(S, xs, cluster);
            for (int i = tid; i < nloc; i += FZ_THREADS) a.wbuf[(size_t)ch * N + row0 + i] = xs[i];
            fz_channel_sums(Vc, n, 0, true, xs, nloc, red, part_me + P_NRM * pstride);
        }
        if (!cl_grid_sync(a.bar, expect, ordinal, a, &s_ok, &s_all, cluster)) return;
        fz_reduce(a.part + P_NRM * pstride, nown_ctas, 1, hd);
        if (tid == 0) {
            const double b = sqrt(fmax(hd[0], 0.0));
            ctl.s = (float)(b > 0.0 ? 1.0 / b : 0.0);
            ctl.tol_eff = fmax(a.tol, 2e-6 * b);
            ctl.tol_f = (float)ctl.tol_eff;
            ctl.j = 0;
            ctl.k = 0;
            ctl.cont = b > 0.0 ? 1 : 0;
            ctl.passes += 1;
            G.g[0] = (float)b;
            G.g[1] = 0.f;
            if (lead) {
                a.st->stats.k = 0;
                a.st->stats.beta0 = b;
                a.st->stats.resid = b;
                a.st->stats.passes = ctl.passes;
                a.st->stats.cum_passes += 1;
            }
        }
        __syncthreads();

        while (ctl.cont) {
            const int j = ctl.j, J = j + 1;
            const float s = ctl.s;
            if (owner) {
                for (int i = tid; i < nloc; i += FZ_THREADS) {
                    const cxf v = xs[i];
                    Vc[(size_t)j * n + i] = mk<float>(v.x * s, v.y * s);
                }
                cl_matvec32<KB>(a, ch, sc_plus, a.wbuf + (size_t)(j & 1) * n, s, xs, row0, nloc, nlocpad, xsrc, j, hs);
                __syncthreads();
                cl_tri_solve(S, xs, cluster);
                fz_channel_sums(Vc, n, J, false, xs, nloc, red, part_me + P_H1 * pstride);
            }
            if (!cl_grid_sync(a.bar, expect, ordinal, a, &s_ok, &s_all, cluster)) return;
            fz_reduce(a.part + P_H1 * pstride, nown_ctas, 2 * J, hf[0]);
            if (owner) {
                if (tid < J) hs[tid] = mk<float>(hf[0][2 * tid], hf[0][2 * tid + 1]);
                __syncthreads();
                for (int i = tid; i < nloc; i += FZ_THREADS) {
                    const cxf acc = fz_gs_update<false>(xs[i], Vc + i, n, J, hs);
                    xs[i] = acc;
                    a.wbuf[(size_t)((j + 1) & 1) * n + (size_t)ch * N + row0 + i] = acc;
                }
                __syncthreads();
                fz_channel_sums(Vc, n, J, false, xs, nloc, red, part_me + P_H2 * pstride, true);
            }
            if (!cl_grid_sync(a.bar, expect, ordinal, a, &s_ok, &s_all, cluster)) return;
            fz_reduce(a.part + P_H2 * pstride, nown_ctas, 2 * J, hf[1]);
            fz_reduce(a.part + P_H2 * pstride + 2 * J, nown_ctas, 1, hd);
            if (owner) {
                if (tid < J) hs[tid] = mk<float>(hf[1][2 * tid], hf[1][2 * tid + 1]);
                __syncthreads();
                for (int i = tid; i < nloc; i += FZ_THREADS) xs[i] = fz_gs_update<false>(xs[i], Vc + i, n, J, hs);
            }
            if (tid == 0) {
                double b2 = hd[0];
                for (int q = 0; q < J; ++q) b2 -= (double)hf[1][2 * q] * hf[1][2 * q] + (double)hf[1][2 * q + 1] * hf[1][2 * q + 1];
                const float fb = (float)sqrt(fmax(b2, 0.0));
                const float resid = fz_givens(G, j, hf[0], hf[1], fb);
                const bool bad = !(resid == resid);
                const bool conv = bad || resid <= ctl.tol_f || J >= a.m || !(fb > 0.f);
                ctl.k = J;
                ctl.s = fb > 0.f ? 1.f / fb : 0.f;
                ctl.cont = conv ? 0 : 1;
                if (!conv) ctl.j = j + 1;
                if (lead) {
                    a.st->stats.k = J;
                    a.st->stats.resid = resid;
                    a.st->stats.iterations += 1;
                    a.st->stats.cum_iterations += 1;
                }
            }
            __syncthreads();
        }

        // e = V y (FP64, this CTA's spread rows; V read through L2), psi += e, e published
        if (tid == 0) fz_backsolve(G, ctl.k, ys);
        __syncthreads();
        const int k = ctl.k;
        for (long long o = lo + tid; o < hi; o += FZ_THREADS) {
            double ax = 0.0, ay = 0.0;
            for (int q0 = 0; q0 < k; q0 += FZ_CB) {
                cxf v[FZ_CB];
#pragma unroll
                for (int q = 0; q < FZ_CB; ++q)
                    v[q] = q0 + q < k ? fz_ldcg(a.V + (size_t)(q0 + q) * n + o) : mk<float>(0.f, 0.f);
#pragma unroll
                for (int q = 0; q < FZ_CB; ++q) {
                    if (q0 + q >= k) break;
                    const cxd yq = ys[q0 + q];
                    ax = fma((double)v[q].x, yq.x, ax); ax = fma(-(double)v[q].y, yq.y, ax);
                    ay = fma((double)v[q].x, yq.y, ay); ay = fma((double)v[q].y, yq.x, ay);
                }
            }
            a.e64[o] = mk<double>(ax, ay);
            a.psi[o] = a.psi[o] + mk<double>(ax, ay);
        }
        if (!cl_grid_sync(a.bar, expect, ordinal, a, &s_ok, &s_all, cluster)) return;
        const double rn = fz_rows64<KB>(a.op64, a.rb64, lo, hi, sc_negplus, a.e64, a.r64, true);
        fz_cta_sum64(rn, red, part_me + P_RES * pstride);
        if (!cl_grid_sync(a.bar, expect, ordinal, a, &s_ok, &s_all, cluster)) return;
        fz_reduce(a.part + P_RES * pstride, gridDim.x, 1, hd);
        if (tid == 0) {
            const double r = sqrt(fmax(hd[0], 0.0));
            ctl.again = (r > a.tol) && (r == r) && ctl.passes < FZ_MAXPASS;
            if (lead) a.st->stats.true_resid = r;
        }
        __syncthreads();
        if (!ctl.again) break;
    }
    if (lead && a.hstats) {
        *a.hstats = a.st->stats;
        *(volatile int *)a.herr = *(volatile int *)a.err;  // read by the host after it synchronises
    }
    cluster.sync();  // no CTA leaves while a peer could still read its shared memory
}

// ------------------------------------------------------------------------------------
// host
// ------------------------------------------------------------------------------------
struct FusedCayley {
    FzArgs args;
    size_t smem = 0;
    int nctas = 0;
    bool kb6 = false;  // the instance unrolled for 13-diagonal bands (k = 7 B-splines)
    void *bufs[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};  // real bands, tables
    // the cluster variant (three CTAs per channel), when the operator's shape qualifies
    bool cluster_ok = false;
    bool use_cluster = false;
    int parity = 0;     // which of the two arrival counters the next launch uses
    int coop = -1;      // cooperative launch with clusters: -1 untried, 1 works, 0 refused by the driver
    size_t csmem = 0;
    int cnctas = 0;
    FzArgs cargs;
};

static size_t fz_smem_bytes(int N, int nblk, int w, int kb, int g_in_smem, size_t band_bytes)
{
    const size_t base = ((size_t)nblk * 32 + (size_t)nblk * w * (g_in_smem ? 33 : 1) + (size_t)FZ_MAXU * (N + 2 * kb)) *
                        sizeof(cxf);
    return band_bytes ? (base + 15) / 16 * 16 + band_bytes : base;
}

int pg_cayley_fused_prepare(pg_op *op64, pg_op *opb, pg_banded *precb, int m, FusedCayley **out)
{
    if (!out) return PG_ERR_ARG;
    *out = nullptr;
    if (!op64 || !opb || !precb) return PG_ERR_ARG;
    if (m < 2 || m > FZ_MAXM) return PG_ERR_SHAPE;
    if (op64->rank != 2 || opb->rank != 2 || opb->precision != PG_FP32 || op64->precision != PG_FP64)
        return PG_ERR_STORAGE;
    if (!op64->finalized || !opb->finalized) return PG_ERR_STATE;
    if (op64->ndense_entries > 0 || opb->ndense_entries > 0 || op64->fact.Q > 0 || opb->fact.Q > 0)
        return PG_ERR_STORAGE;
    if (op64->nrows != opb->nrows || op64->N != opb->N || op64->kb != opb->kb) return PG_ERR_STORAGE;
    if (precb->kind != 1 || !precb->op || precb->op->precision != PG_FP32 || precb->op->nrows != opb->nrows ||
        precb->N != opb->N || precb->kb < 1 || precb->kb > 32)
        return PG_ERR_STORAGE;
    pg_ctx *ctx = opb->ctx;
    const int N = opb->N, nch = opb->nrows, nblk = (N + 31) / 32, w = precb->kb, kb = opb->kb;
    if (nch < 1 || N < 1) return PG_ERR_SHAPE;
    // real radial bands (the complex factors of a Cayley step are the slot scales)
    std::vector<double> rb64;
    std::vector<float> rb32;
    if (!real_bands<double>(op64, rb64) || !real_bands<float>(opb, rb32)) return PG_ERR_STORAGE;
    // distinct source channels of each row of opb, staged once per matvec
    std::vector<int> ucol, nucol;
    std::vector<unsigned char> ent_u;
    if (!fz_source_tables(opb, ucol, nucol, ent_u)) return PG_ERR_STORAGE;  // wider coupling: multi-kernel step
    const bool kb6 = (kb == 6);
    const void *kern = kb6 ? (const void *)cay_fused_step_kernel<6> : (const void *)cay_fused_step_kernel<-1>;
    const size_t limit = 200 * 1024;
    // a channel's FP32 bands in shared memory when the largest row's fit with the rest
    int max_e = 0;
    for (int r = 0; r < nch; ++r) max_e = std::max(max_e, opb->h_row_ptr[r + 1] - opb->h_row_ptr[r]);
    const size_t band_bytes = (size_t)max_e * (2 * kb + 1) * opb->ld * sizeof(float);
    const size_t v_bytes = (size_t)m * N * sizeof(cxf);
    int g_in_smem = 1, bands_smem = 0, v_smem = 1;
    size_t smem = fz_smem_bytes(N, nblk, w, kb, 1, v_bytes);
    if (smem > limit) {
        v_smem = 0;
        bands_smem = 1;
        smem = fz_smem_bytes(N, nblk, w, kb, 1, band_bytes);
    }
    if (smem > limit) {
        bands_smem = 0;
        smem = fz_smem_bytes(N, nblk, w, kb, 1, 0);
    }
    if (smem > limit) {
        g_in_smem = 0;
        smem = fz_smem_bytes(N, nblk, w, kb, 0, 0);
        if (smem > limit) return PG_ERR_SHAPE;
    }
    PG_CUDA_TRY(raise_smem_limit(kern, smem));
    int per_sm = 0;
    PG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, FZ_THREADS, smem));
    const int resident = per_sm * std::max(1, ctx->num_sms);
    if (per_sm < 1 || nch > resident) return PG_ERR_SHAPE;  // every CTA must be resident at once
    // one CTA per SM: the channels, and the FP64 rows spread over all of them
    const int nctas = std::max(nch, std::min(resident, std::max(1, ctx->num_sms)));

    // the cluster variant: a third of each channel's solve factors per CTA in shared memory
    const int nb = nblk * w;
    const int bpc = (nblk + CL_SIZE - 1) / CL_SIZE, rpc = (nb + CL_SIZE - 1) / CL_SIZE;
    int rbmax = 0;
    for (int cr = 0; cr < CL_SIZE; ++cr) {
        int tot = 0;
        for (int r = std::min(nb, cr * rpc); r < std::min(nb, (cr + 1) * rpc); ++r) tot += (r / w + 1) * w + nb - (r / w) * w;
        rbmax = std::max(rbmax, tot);
    }
    const ClLayout CLL = cl_layout(bpc, w, nb, rpc, rbmax, kb);
    const void *ckern = kb6 ? (const void *)cay_cluster_step_kernel<6> : (const void *)cay_cluster_step_kernel<-1>;
    int cnctas = 0;
    {
        cudaFuncAttributes fa;
        int optin = 0;
        if (cudaFuncGetAttributes(&fa, ckern) == cudaSuccess &&
            cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device) == cudaSuccess &&
            CLL.bytes + fa.sharedSizeBytes + 1024 <= (size_t)optin && w <= 32 &&
            raise_smem_limit(ckern, CLL.bytes) == cudaSuccess) {
            cudaLaunchConfig_t cfg;
            memset(&cfg, 0, sizeof(cfg));
            cfg.gridDim = dim3(CL_SIZE);
            cfg.blockDim = dim3(FZ_THREADS);
            cfg.dynamicSmemBytes = CLL.bytes;
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = CL_SIZE;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            int ncl = 0;
            if (cudaOccupancyMaxActiveClusters(&ncl, ckern, &cfg) == cudaSuccess && ncl >= nch) {
                // every cluster resident at once: the channels, and helpers for the FP64 rows
                const int want = std::max(nch, std::min(ncl, std::max(1, ctx->num_sms / CL_SIZE)));
                cnctas = want * CL_SIZE;
            }
        }
        cudaGetLastError();  // a shape the cluster variant refuses leaves no error behind
    }
    const int maxctas = std::max(nctas, cnctas);

    FusedCayley *f = new FusedCayley();
    FzArgs &a = f->args;
    memset(&a, 0, sizeof(a));
    a.op64 = op64->dev();
    a.opb = opb->dev();
    a.lo_inv = (const cxf *)precb->d_lo_inv;
    a.lo_g = (const cxf *)precb->d_lo_cpl;
    a.lo_rb = (const cxf *)precb->d_lo_rb;
    a.up_inv = (const cxf *)precb->d_up_inv;
    a.up_g = (const cxf *)precb->d_up_cpl;
    a.up_rb = (const cxf *)precb->d_up_rb;
    a.nblk = nblk;
    a.w = w;
    a.fib_per_mat = std::max(1, precb->fib_per_mat);
    a.g_in_smem = g_in_smem;
    a.bands_smem = bands_smem;
    a.v_smem = v_smem;
    a.nch = nch;
    a.N = N;
    a.m = m;
    a.nctas = nctas;
    const size_t n = (size_t)nch * N;
    int code = PG_OK;
    auto alloc = [&](void **p, size_t bytes) {
        if (code == PG_OK && cudaMalloc(p, bytes) != cudaSuccess) code = PG_ERR_CUDA;
    };
    alloc((void **)&a.r64, sizeof(cxd) * n);
    alloc((void **)&a.e64, sizeof(cxd) * n);
    alloc((void **)&a.wbuf, sizeof(cxf) * 2 * n);
    alloc((void **)&a.V, sizeof(cxf) * (size_t)m * n);
    alloc((void **)&a.part, sizeof(double) * P_COUNT * (size_t)maxctas * FZ_PSTRIDE);
    alloc((void **)&a.bar, 2 * sizeof(FzBarrier));
    if (code == PG_OK && cudaMemset(a.bar, 0, 2 * sizeof(FzBarrier)) != cudaSuccess) code = PG_ERR_CUDA;
    if (code == PG_OK) code = upload_vec(rb64, &f->bufs[0]);
    if (code == PG_OK) code = upload_vec(rb32, &f->bufs[1]);
    if (code == PG_OK) code = upload_vec(ucol, &f->bufs[2]);
    if (code == PG_OK) code = upload_vec(nucol, &f->bufs[3]);
    if (code == PG_OK) code = upload_vec(ent_u, &f->bufs[4]);
    // FP64 rows split so that every CTA applies about the same number of band entries
    auto split_rows = [&](int ctas) {
        std::vector<int> row_lo(ctas + 1, 0);
        long long total = 0;
        for (int r = 0; r < nch; ++r) total += (long long)(op64->h_row_ptr[r + 1] - op64->h_row_ptr[r] + 1) * N;
        long long acc = 0;
        int g = 1;
        for (long long o = 0; o < (long long)n && g < ctas; ++o) {
            const int r = (int)(o / N);
            acc += op64->h_row_ptr[r + 1] - op64->h_row_ptr[r] + 1;
            while (g < ctas && acc * ctas >= total * g) row_lo[g++] = (int)(o + 1);
        }
        while (g <= ctas) row_lo[g++] = (int)n;
        return row_lo;
    };
    if (code == PG_OK) code = upload_vec(split_rows(nctas), &f->bufs[5]);
    if (code == PG_OK && cnctas > 0) code = upload_vec(split_rows(cnctas), &f->bufs[6]);
    if (code != PG_OK) {
        pg_cayley_fused_free(f);
        return code;
    }
    a.rb64 = (const double *)f->bufs[0];
    a.rb32 = (const float *)f->bufs[1];
    a.ucol = (const int *)f->bufs[2];
    a.nucol = (const int *)f->bufs[3];
    a.ent_u = (const unsigned char *)f->bufs[4];
    a.row_lo = (const int *)f->bufs[5];
    f->smem = smem;
    f->nctas = nctas;
    f->kb6 = kb6;
    if (cnctas > 0) {
        f->cluster_ok = true;
        f->use_cluster = true;  // the default where it qualifies
        f->csmem = CLL.bytes;
        f->cnctas = cnctas;
        f->cargs = a;
        f->cargs.row_lo = (const int *)f->bufs[6];
        f->cargs.nctas = cnctas;
        f->cargs.cl_bpc = bpc;
        f->cargs.cl_rpc = rpc;
        f->cargs.cl_rbmax = rbmax;
    }
    *out = f;
    return PG_OK;
}

// 0: the cluster variant where it qualifies (default), 1: one CTA per channel, 2: the cluster
// variant (PG_ERR_SHAPE when the operator's shape does not fit it)
int pg_cayley_fused_select(FusedCayley *f, int variant)
{
    if (!f || variant < 0 || variant > 2) return PG_ERR_ARG;
    if (variant == 2 && !f->cluster_ok) return PG_ERR_SHAPE;
    f->use_cluster = f->cluster_ok && variant != 1;
    return PG_OK;
}

int pg_cayley_fused_which(const FusedCayley *f) { return f && f->use_cluster ? 2 : 1; }

int pg_cayley_fused_launch(FusedCayley *f, cudaStream_t s, const StepParams &params, cxd *psi, GmresState *st,
                           double tol, int *err, GmresStats *host_stats, int *host_err)
{
    if (f->use_cluster) {
        FzArgs a = f->cargs;
        a.params = params;
        a.hstats = host_stats;
        a.herr = host_err;
        a.psi = psi;
        a.st = st;
        a.tol = tol;
        a.err = err;
        a.probe_extra = f->args.probe_extra;
        a.probe_at = f->args.probe_at;
        a.bar = f->args.bar + f->parity;
        a.bar_next = f->args.bar + (1 - f->parity);
        f->parity ^= 1;
        cudaLaunchConfig_t cfg;
        memset(&cfg, 0, sizeof(cfg));
        cfg.gridDim = dim3(f->cnctas);
        cfg.blockDim = dim3(FZ_THREADS);
        cfg.dynamicSmemBytes = f->csmem;
        cfg.stream = s;
        cudaLaunchAttribute attr[2];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = CL_SIZE;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        attr[1].id = cudaLaunchAttributeCooperative;
        attr[1].val.cooperative = 1;
        cfg.attrs = attr;
        // every cluster must be resident at once: a cooperative launch guarantees it where the
        // driver accepts one with clusters; otherwise the occupancy check of the set-up does
        cfg.numAttrs = f->coop == 0 ? 1 : 2;
        cudaError_t e = f->kb6 ? cudaLaunchKernelEx(&cfg, cay_cluster_step_kernel<6>, a)
                               : cudaLaunchKernelEx(&cfg, cay_cluster_step_kernel<-1>, a);
        if (e != cudaSuccess && f->coop == -1) {
            cudaGetLastError();
            f->coop = 0;
            cfg.numAttrs = 1;
            e = f->kb6 ? cudaLaunchKernelEx(&cfg, cay_cluster_step_kernel<6>, a)
                       : cudaLaunchKernelEx(&cfg, cay_cluster_step_kernel<-1>, a);
        } else if (e == cudaSuccess && f->coop == -1) {
            f->coop = 1;
        }
        PG_CUDA_TRY(e);
        return PG_OK;
    }
    FzArgs a = f->args;
    a.params = params;
    a.hstats = host_stats;
    a.herr = host_err;
    a.psi = psi;
    a.st = st;
    a.tol = tol;
    a.err = err;
    // launches alternate between two arrival counters, each clearing the other at its start: a
    // counter left half-way by a launch whose wait ran out is cleared before it is used again
    a.bar = f->args.bar + f->parity;
    a.bar_next = f->args.bar + (1 - f->parity);
    f->parity ^= 1;
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.gridDim = dim3(f->nctas);
    cfg.blockDim = dim3(FZ_THREADS);
    cfg.dynamicSmemBytes = f->smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (f->kb6) PG_CUDA_TRY(cudaLaunchKernelEx(&cfg, cay_fused_step_kernel<6>, a));
    else PG_CUDA_TRY(cudaLaunchKernelEx(&cfg, cay_fused_step_kernel<-1>, a));
    return PG_OK;
}

void pg_cayley_fused_set_probe(FusedCayley *f, unsigned int extra_arrivals, unsigned int at_barrier)
{
    if (!f) return;
    f->args.probe_extra = extra_arrivals;
    f->args.probe_at = at_barrier;
}

void pg_cayley_fused_free(FusedCayley *f)
{
    if (!f) return;
    cudaFree(f->args.r64);
    cudaFree(f->args.e64);
    cudaFree(f->args.wbuf);
    cudaFree(f->args.V);
    cudaFree(f->args.part);
    cudaFree(f->args.bar);
    for (void *b : f->bufs) cudaFree(b);
    delete f;
}
