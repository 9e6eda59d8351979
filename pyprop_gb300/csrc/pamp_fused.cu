// Single-kernel mixed-precision pAMP step of one wavefunction.
//
// The step of pg_pamp_step (pAMP, core/krylov/pamp/pamp/pamp.h:613-670, in the balanced-overlap
// form of PamPropagator.AdvanceStep, pyprop/propagator/PamPropagator.py:50-75) as ONE
// cooperative launch in which CTA a owns angular channel a. With S = U^T U, the Arnoldi
// recurrence of A = U^-T H U^-1 on V_j is run on T_j = U^-1 V_j:
//   A V_j - sum_i V_i h_ij = U (S^-1 H T_j - sum_i T_i h_ij),
//   <V_i, A V_j> = T_i^H H T_j,   <V_i, V_k> = T_i^H S T_k,
// so the Krylov vectors are the S-orthonormal T_j, no product with U or U^-1 is left, and
//   psi(t + dt) = U^-1 ||U psi|| V c = ||psi||_S sum_j c_j T_j.
// Per Arnoldi step (the Hessenberg entries are those of the balanced form):
//   y = H T_j (row of channel a, from the neighbour channels' T_j), z = S^-1 y (channel-local
//   blocked solves), h1 = T^H y (= <T, z>_S) ........................... grid barrier
//   z' = z - T h1 (published), u = S z', h2 = T^H u, ||z'||_S^2 = z'^H u . grid barrier
//   z'' = z' - T h2, beta = (||z'||_S^2 - |h2|^2)^(1/2), T_(j+1) = z'' / beta
// (z' is S-orthogonal to T up to rounding, so the norm by Pythagoras has no cancellation). A
// CTA staging a neighbour's T_(j+1) for its row product forms it from that neighbour's z' and
// T_i, visible after the second barrier, with the owner's arithmetic (the device routines of
// the single-kernel Cayley step), so an Arnoldi step costs two grid barriers. Every CTA sums
// the channel partials in the same order and so holds the same Hessenberg matrix; each
// computes c = ||psi||_S exp(-i dt H_k) e_1 itself (the scaled order-6 Pade of
// pamp.h:430-565, double-float arithmetic) and forms its channel of psi in FP64. The basis and
// the products are complex64, the channel sums FP64, ||psi||_S FP64. A happy breakdown
// (beta < tolerance, pamp.h:306-313) truncates the basis. Grid barriers are bounded waits: one
// that runs out sets the context's error word (2) and the CTAs return with psi unchanged.
//
// Qualifying steppers (pg_pamp_fused_prepare): complex64 basis, a rank-2 operator with real
// bands and at most FZ_MAXU distinct source channels per row, basis size <= PF_MAXM, and no
// more channels than resident CTAs of 768 threads.
#include "fused_common.cuh"
#include "pamp_expm.cuh"
#include "pamp_fused.cuh"

#include <cstring>

static const int PF_MAXM = 48;                 // Krylov basis bound of the single-kernel pAMP step
static const int PF_PSTRIDE = 2 * (PF_MAXM + 1);  // doubles per CTA and phase in the partials
static const int PF_PE = 2 * PF_MAXM + 8;
static const int PF_DENSE_MAXN = 176;  // longest fibre whose dense S^-1 is staged in shared memory  // per CTA: c [2m], ||psi||_S^2 and ||psi||_S, statistics [4]

struct PfArgs {
    FzArgs z;                 // channel tables, bands, scratch, barrier, error word, psi
    const float *slo_inv, *slo_g, *slo_rb, *sup_inv, *sup_g, *sup_rb;  // S^-1 = U^-1 U^-T factors
    const float *S32;         // [N][2ks+1] overlap rows
    const double *S64;        // [N][2ks+1]
    int ks;                   // overlap half-bandwidth
    const float *sinv;        // [N][sld] S^-1 in FP32 (dense solve mode)
    int sld;
    const signed char *uslot; // [Nang][FZ_MAXU] cache slot of each source channel of a row (-1: the row's own)
    int ncache, off_cache;    // neighbour Krylov vectors kept in shared memory: slots (0: none), offset
    int off_ys, off_sb, off_sg, off_xsrc, off_band, off_tab, off_T;  // shared-memory layout (bytes)
    double dt;
    double tol;               // beta below it truncates the basis
    cxd h[PG_MAX_SLOTS];      // H(t) slot values
    double *hcols;            // [CTAs][m][3][2(m+2)] each CTA's Hessenberg columns
    double *pe;               // [CTAs][PF_PE] each CTA's coefficients, norms, statistics
    double *ex;               // [0] basis size, [1] error estimate, [2] 0 or -1 (singular), [3] sticky singular flag
};

// (h, l) += (ph, pl): Knuth's two-sum of the high parts, the low parts added
__device__ __forceinline__ void pf_acc(float &h, float &l, float ph, float pl)
{
    const float s = h + ph;
    const float bb = s - h;
    const float err = (h - (s - bb)) + (ph - bb);
    h = s;
    l += err + pl;
}
// (h, l) += a b, the product split exactly by an FMA
__device__ __forceinline__ void pf_madd(float &h, float &l, float a, float b)
{
    const float q = __fmul_rn(a, b);  // never contracted into an FMA with the two-sum
    pf_acc(h, l, q, fmaf(a, b, -q));
}

// out[2q], out[2q+1] = <T_q, y> for q < J (T_q at Tr + q tld) and, with zx, out[2J] =
// Re <zx, y>, each as a double-float pair (high, low) in the 8-byte slot: warp w takes the
// columns w, w + FZ_NW, ...; its lanes stride over the N elements and the 32 lane sums are
// combined by shuffles, all in double-float arithmetic on the complex64 products (the FP64
// pipe of this GPU is too narrow for per-element FP64 sums). No CTA barrier inside (the grid
// barrier that follows has one).
__device__ __forceinline__ void pf_dots(const cxf *Tr, long long tld, int J, const cxf *y, const cxf *zx, int N,
                                        double *outd)
{
    float2 *out = reinterpret_cast<float2 *>(outd);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int ncol = J + (zx ? 1 : 0);
    for (int q = warp; q < ncol; q += FZ_NW) {
        float xh = 0.f, xl = 0.f, yh = 0.f, yl = 0.f;
        const cxf *v = q < J ? Tr + (size_t)q * tld : zx;
        for (int i = lane; i < N; i += 32) {
            const cxf a = v[i], b = y[i];
            pf_madd(xh, xl, a.x, b.x);
            pf_madd(xh, xl, a.y, b.y);
            pf_madd(yh, yl, a.x, b.y);
            pf_madd(yh, yl, -a.y, b.x);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float oxh = __shfl_xor_sync(0xffffffffu, xh, o), oxl = __shfl_xor_sync(0xffffffffu, xl, o);
            const float oyh = __shfl_xor_sync(0xffffffffu, yh, o), oyl = __shfl_xor_sync(0xffffffffu, yl, o);
            pf_acc(xh, xl, oxh, oxl);
            pf_acc(yh, yl, oyh, oyl);
        }
        if (lane == 0) {
            out[2 * q] = make_float2(xh, xl);
            if (q < J) out[2 * q + 1] = make_float2(yh, yl);
        }
    }
}

// out[t] = sum over the channels a < nch of the double-float partials part[a][t], t < nval:
// one warp per value (two values' loads in flight together), the channels over the lanes,
// double-float shuffles in a fixed order (the same in every CTA), one FP64 sum at the end.
// Ends with a CTA barrier.
__device__ __forceinline__ void pf_reduce(const double *part, int nch, int nval, double *out)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int t0 = warp; t0 < nval; t0 += 2 * FZ_NW) {
        float h[2] = {0.f, 0.f}, l[2] = {0.f, 0.f};
        for (int a = lane; a < nch; a += 32) {
            float2 v[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int t = t0 + u * FZ_NW;
                v[u] = t < nval ? __ldcg(reinterpret_cast<const float2 *>(part + (size_t)a * PF_PSTRIDE + t))
                                : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int u = 0; u < 2; ++u) pf_acc(h[u], l[u], v[u].x, v[u].y);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const float oh = __shfl_xor_sync(0xffffffffu, h[u], o), ol = __shfl_xor_sync(0xffffffffu, l[u], o);
                pf_acc(h[u], l[u], oh, ol);
            }
        if (lane == 0)
#pragma unroll
            for (int u = 0; u < 2; ++u)
                if (t0 + u * FZ_NW < nval) out[t0 + u * FZ_NW] = (double)h[u] + (double)l[u];
    }
    __syncthreads();
}

// Stage bytes (a multiple of 4) at src into shared memory at dst with asynchronous copies of
// 16 bytes where both ends allow it, else 4 (waited for by fz_bands_wait).
__device__ __forceinline__ void pf_stage(void *dst, const void *src, size_t bytes)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    const bool v16 = ((bytes | (size_t)src | (size_t)d) & 15) == 0;
    const size_t step = v16 ? 16 : 4;
    for (size_t o = (size_t)threadIdx.x * step; o < bytes; o += (size_t)FZ_THREADS * step) {
        const char *s = (const char *)src + o;
        if (v16) asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d + (unsigned)o), "l"(s) : "memory");
        else asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d + (unsigned)o), "l"(s) : "memory");
    }
}

// Stage the row's source fibres T_j[col] = (z'[col] - sum_q<j T_q[col] h2_q) s into xsrc
// ([nu][N + 2kb], zero halo), with the Gram-Schmidt correction read from shared memory: the
// CTA's own channel from its Krylov vectors sT, each neighbour from the copies of its T_q this
// CTA formed while staging in earlier Arnoldi steps (cache [slot][m][N]); the new T_j of each
// neighbour joins its copies. The same arithmetic as the owner's, so the copies are the
// owner's vectors bit for bit. Only z' is read from global memory (one L2 round trip).
__device__ __forceinline__ void pf_sources(const FzArgs &A, int a, const cxf *wsrc, float s, int j, const cxf *hs,
                                           cxf *xsrc, int kb, const cxf *sT, cxf *cache, const signed char *slot)
{
    const int N = A.N, m = A.m, W = N + 2 * kb, nu = __ldg(A.nucol + a);
    for (int idx = threadIdx.x; idx < nu * W; idx += FZ_THREADS) {
        const int u = idx / W, jj = idx - u * W - kb;
        cxf x = mk<float>(0.f, 0.f);
        if (jj >= 0 && jj < N) {
            const int col = __ldg(A.ucol + (size_t)a * FZ_MAXU + u);
            const int sl = __ldg(slot + u);
            const cxf *Tq = sl < 0 ? sT + jj : cache + (size_t)sl * m * N + jj;
            const cxf v = fz_gs_update<false>(fz_ldcg(wsrc + (size_t)col * N + jj), Tq, N, j, hs);
            x = mk<float>(v.x * s, v.y * s);
            if (sl >= 0) cache[((size_t)sl * m + j) * N + jj] = x;
        }
        xsrc[idx] = x;
    }
    __syncthreads();
}

// The overlap solve z = S^-1 y: SOLVE 0 the blocked triangular solves with factors read through
// L2, 1 the same with the factors staged in shared memory, 2 a product with the dense S^-1 (FP32,
// formed in FP64 on the host) staged in shared memory, for fibres short enough to hold it.
template <int KB, int SOLVE>
__global__ void __launch_bounds__(FZ_THREADS, 1) pamp_fused_step_kernel(PfArgs p)
{
    constexpr bool STAB = SOLVE == 1;
    const FzArgs &a = p.z;
    if (fz_bad_launch(a, gridDim.x != (unsigned)a.nctas || gridDim.y != 1 || gridDim.z != 1)) return;
    // the previous launch, which used bar_next, has completed: clear it for the next launch
    if (blockIdx.x == 0 && threadIdx.x == 0) a.bar_next->count = 0;
    extern __shared__ __align__(16) unsigned char pf_smem[];
    __shared__ cxf sc[PG_MAX_SLOTS];
    __shared__ double red[FZ_NW][2 * FZ_CB];
    __shared__ double h1d[PF_PSTRIDE], h2d[PF_PSTRIDE];
    __shared__ double hd[1];
    __shared__ cxf hs[PF_MAXM];
    __shared__ double cs[2 * PF_MAXM];
    __shared__ int s_ok, s_k, s_cont;
    __shared__ float s_inv;  // 1/beta (first 1/||psi||_S) of the Krylov vector formed next

    const int ch = blockIdx.x, tid = threadIdx.x;
    const int N = a.N, nblk = a.nblk, w = a.w, npad = nblk * 32, m = a.m;
    const long long n = (long long)a.nch * N;
    const int ks = p.ks, sw = 2 * p.ks + 1;
    const size_t cd = 2 * (size_t)(m + 2);
    cxf *xs = (cxf *)pf_smem;                               // [npad] psi, then z, z', z''
    cxf *ys = (cxf *)(pf_smem + p.off_ys);                  // [npad] y = H T_j, then u = S z'
    cxf *sb = (cxf *)(pf_smem + p.off_sb);                  // [nblk*w] block-solve boundary values
    float *sg = (float *)(pf_smem + p.off_sg);              // [nblk][w][32] (g_in_smem)
    cxf *xsrc = (cxf *)(pf_smem + p.off_xsrc);              // [FZ_MAXU][N + 2kb] staged sources
    float *sband = a.bands_smem ? (float *)(pf_smem + p.off_band) : nullptr;
    cxf *sT = a.v_smem ? (cxf *)(pf_smem + p.off_T) : nullptr;  // [m][N] this channel's T_q
    cxf *cache = p.ncache ? (cxf *)(pf_smem + p.off_cache) : nullptr;  // [slots][m][N] neighbours' T_q
    unsigned char *exs = pf_smem + p.off_ys;                // the exponential's scratch, after the loop
    cxf *Tc = a.V + (size_t)ch * N;                         // T_q[ch] at Tc + q n
    const cxf *Tr = sT ? sT : Tc;
    const long long tld = sT ? (long long)N : n;
    const size_t mat = (size_t)(ch / a.fib_per_mat);
    const size_t pstride = (size_t)gridDim.x * PF_PSTRIDE;
    double *part_me = a.part + (size_t)ch * PF_PSTRIDE;
    double *hc = p.hcols + (size_t)ch * m * 3 * cd;
    double *pe = p.pe + (size_t)ch * PF_PE;
    unsigned int expect = 0, ordinal = 0;
    // the overlap solve's factors of this channel's matrix: staged in shared memory for the
    // whole step (STAB) or read through L2 at every solve
    const int nb = nblk * w;
    float *tab = (float *)(pf_smem + p.off_tab);
    const float *lo_inv = STAB ? tab : p.slo_inv;
    const float *up_inv = STAB ? tab + (size_t)nblk * 1024 : p.sup_inv;
    const float *lo_g = STAB ? tab + (size_t)2 * nblk * 1024 : p.slo_g;
    const float *up_g = STAB ? lo_g + (size_t)nb * 32 : p.sup_g;
    const float *lo_rb = STAB ? up_g + (size_t)nb * 32 : p.slo_rb;
    const float *up_rb = STAB ? lo_rb + (size_t)nb * nb : p.sup_rb;
    const size_t tmat = STAB ? 0 : mat;

    if (tid < PG_MAX_SLOTS) sc[tid] = cvt<float>(p.h[tid]);
    // this channel's FP32 bands (and the solve factors) to shared memory, in flight during the norm
    if (SOLVE == 2) {
        pf_stage(tab, p.sinv, sizeof(float) * (size_t)N * p.sld);
        asm volatile("cp.async.commit_group;" ::: "memory");
    }
    if (STAB) {
        pf_stage((void *)lo_inv, p.slo_inv + mat * nblk * 1024, sizeof(float) * nblk * 1024);
        pf_stage((void *)up_inv, p.sup_inv + mat * nblk * 1024, sizeof(float) * nblk * 1024);
        pf_stage((void *)lo_g, p.slo_g + mat * nb * 32, sizeof(float) * nb * 32);
        pf_stage((void *)up_g, p.sup_g + mat * nb * 32, sizeof(float) * nb * 32);
        pf_stage((void *)lo_rb, p.slo_rb + mat * nb * nb, sizeof(float) * nb * nb);
        pf_stage((void *)up_rb, p.sup_rb + mat * nb * nb, sizeof(float) * nb * nb);
        asm volatile("cp.async.commit_group;" ::: "memory");
    }
    if (sband) fz_bands_load(a, ch, sband);
    // ||psi||_S^2 of this channel (FP64); psi in complex64, published for the first products
    {
        const cxd *pc = a.psi + (size_t)ch * N;
        double nrm = 0.0;
        for (int i = tid; i < npad; i += FZ_THREADS) {
            cxf v = mk<float>(0.f, 0.f);
            if (i < N) {
                const cxd x = pc[i];
                double tx = 0.0, ty = 0.0;
                for (int d = 0; d < sw; ++d) {
                    const int q = i + d - ks;
                    if (q >= 0 && q < N) {
                        const double c = __ldg(p.S64 + (size_t)i * sw + d);
                        const cxd y = pc[q];
                        tx = fma(c, y.x, tx);
                        ty = fma(c, y.y, ty);
                    }
                }
                nrm = fma(x.x, tx, nrm);
                nrm = fma(x.y, ty, nrm);
                v = mk<float>((float)x.x, (float)x.y);
                a.wbuf[(size_t)ch * N + i] = v;
            }
            xs[i] = v;
        }
        fz_cta_sum64(nrm, red, part_me + P_NRM * pstride);
    }
    if (sband || SOLVE != 0) fz_bands_wait();  // before any exit: no copy outlives the CTA
    if (!fz_grid_sync(a.bar, expect, ordinal, a, &s_ok)) return;
    if (tid < 32) {  // ||psi||_S^2: the channels' FP64 partials over the lanes, a fixed order
        double v = 0.0;
        for (int c = tid; c < a.nch; c += 32) v += __ldcg(a.part + P_NRM * pstride + (size_t)c * PF_PSTRIDE);
        v = fz_warp_sum(v);
        if (tid == 0) hd[0] = v;
    }
    __syncthreads();
    if (tid == 0) {
        const double nrm = sqrt(fmax(hd[0], 0.0));
        pe[2 * m] = hd[0];
        pe[2 * m + 1] = nrm;
        s_inv = (float)(nrm > 0.0 ? 1.0 / nrm : 0.0);
        s_k = 0;
        s_cont = nrm > 0.0 ? 1 : 0;
    }
    __syncthreads();

    while (s_cont) {
        const int j = s_k, J = j + 1;
        const float s = s_inv;
        // T_j of this channel (z'' of the last step, or psi, scaled)
        for (int i = tid; i < N; i += FZ_THREADS) {
            const cxf v = xs[i];
            const cxf vs = mk<float>(v.x * s, v.y * s);
            Tc[(size_t)j * n + i] = vs;
            if (sT) sT[(size_t)j * N + i] = vs;
        }
        // y = H T_j (row ch); the staged sources are the channels' z' with the last step's
        // second correction (hs = h2, j vectors) applied, scaled by s
        if (cache) {
            pf_sources(a, ch, a.wbuf + (size_t)(j & 1) * n, s, j, hs, xsrc, KB >= 0 ? KB : a.opb.kb, sT, cache,
                       p.uslot + (size_t)ch * FZ_MAXU);
            fz_rowprod32<KB>(a, ch, sc, ys, npad, xsrc, sband);
        } else {
            fz_matvec32<KB>(a, ch, sc, a.wbuf + (size_t)(j & 1) * n, s, ys, npad, xsrc, sband, j, hs);
        }
        __syncthreads();
        if constexpr (SOLVE == 2) {
            // z = S^-1 y: row i by a group of 8 lanes (columns strided by 8), summed by shuffles
            for (int i0 = 0; i0 < npad; i0 += FZ_THREADS / 8) {
                const int i = i0 + (tid >> 3), g = tid & 7;
                float zx = 0.f, zy = 0.f;
                if (i < N) {
                    const float *row = tab + (size_t)i * p.sld;
                    for (int c = g; c < N; c += 8) {
                        const float sv = row[c];
                        const cxf v = ys[c];
                        zx = fmaf(sv, v.x, zx);
                        zy = fmaf(sv, v.y, zy);
                    }
                }
#pragma unroll
                for (int o = 4; o > 0; o >>= 1) {
                    zx += __shfl_xor_sync(0xffffffffu, zx, o);
                    zy += __shfl_xor_sync(0xffffffffu, zy, o);
                }
                if (g == 0 && i < npad) xs[i] = mk<float>(zx, zy);
            }
            __syncthreads();
        } else {
            for (int i = tid; i < npad; i += FZ_THREADS) xs[i] = ys[i];
            __syncthreads();
            // z = S^-1 y = U^-1 U^-T y
            tri_solve_smem<float, float, FZ_NW, STAB>(nblk, w, tmat, lo_inv, lo_g, lo_rb, up_inv, up_g, up_rb, 1, 1,
                                                      STAB ? 0 : a.g_in_smem, xs, sb, sg);
        }
        // h1 = T^H y
        pf_dots(Tr, tld, J, ys, nullptr, N, part_me + P_H1 * pstride);
        if (!fz_grid_sync(a.bar, expect, ordinal, a, &s_ok)) return;
        pf_reduce(a.part + P_H1 * pstride, a.nch, 2 * J, h1d);
        if (tid < J) hs[tid] = mk<float>((float)h1d[2 * tid], (float)h1d[2 * tid + 1]);
        __syncthreads();
        // z' = z - T h1, published for the next products
        for (int i = tid; i < N; i += FZ_THREADS) {
            const cxf acc = fz_gs_update<false>(xs[i], Tr + i, tld, J, hs);
            xs[i] = acc;
            a.wbuf[(size_t)((j + 1) & 1) * n + (size_t)ch * N + i] = acc;
        }
        __syncthreads();
        // u = S z', h2 = T^H u, ||z'||_S^2 = Re z'^H u
        for (int i = tid; i < N; i += FZ_THREADS) {
            float tx = 0.f, ty = 0.f;
            for (int d = 0; d < sw; ++d) {
                const int q = i + d - ks;
                if (q >= 0 && q < N) {
                    const float c = __ldg(p.S32 + (size_t)i * sw + d);
                    const cxf v = xs[q];
                    tx = fmaf(c, v.x, tx);
                    ty = fmaf(c, v.y, ty);
                }
            }
            ys[i] = mk<float>(tx, ty);
        }
        __syncthreads();
        pf_dots(Tr, tld, J, ys, xs, N, part_me + P_H2 * pstride);
        if (!fz_grid_sync(a.bar, expect, ordinal, a, &s_ok)) return;
        pf_reduce(a.part + P_H2 * pstride, a.nch, 2 * J + 1, h2d);
        if (tid < J) hs[tid] = mk<float>((float)h2d[2 * tid], (float)h2d[2 * tid + 1]);
        __syncthreads();
        // z'' = z' - T h2 (the next T_j; the other CTAs form it themselves)
        for (int i = tid; i < N; i += FZ_THREADS) xs[i] = fz_gs_update<false>(xs[i], Tr + i, tld, J, hs);
        if (tid < 32) {
            // Hessenberg column j in the layout the exponential reads (pass 0 h1, pass 1 h2,
            // pass 2 the subdiagonal beta at 2J + 1); beta^2 = ||z'||_S^2 - |h2|^2
            double sq = 0.0;
            for (int q = tid; q < J; q += 32) {
                sq = fma(h2d[2 * q], h2d[2 * q], sq);
                sq = fma(h2d[2 * q + 1], h2d[2 * q + 1], sq);
                hc[((size_t)j * 3 + 0) * cd + 2 * q] = h1d[2 * q];
                hc[((size_t)j * 3 + 0) * cd + 2 * q + 1] = h1d[2 * q + 1];
                hc[((size_t)j * 3 + 1) * cd + 2 * q] = h2d[2 * q];
                hc[((size_t)j * 3 + 1) * cd + 2 * q + 1] = h2d[2 * q + 1];
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
            if (tid == 0) {
                // sqrt from the FP32 reciprocal square root and one Newton step (few FP64 operations)
                const double b2 = fmax(h2d[2 * J] - sq, 0.0);
                const float r = b2 > 0.0 ? rsqrtf((float)b2) : 0.f;
                const double x = (double)((float)b2 * r);
                double beta = x + (b2 - x * x) * (0.5 * (double)r);
                if (!(beta == beta)) beta = 0.0;
                hc[((size_t)j * 3 + 2) * cd + 2 * J + 1] = beta;
                s_k = J;
                s_inv = beta > 0.0 ? 1.0f / (float)beta : 0.f;
                s_cont = (J < m && beta >= p.tol) ? 1 : 0;
            }
        }
        __syncthreads();
    }

    const int k = s_k;
    if (k > 0) {
        // c = ||psi||_S exp(-i dt H_k) e_1 (every CTA, from its own identical copy)
        PampExpArgs ea;
        ea.cols = hc;
        ea.norm = pe + 2 * m;
        ea.c = pe;
        ea.stats = pe + 2 * m + 2;
        ea.m = m;
        ea.double_ortho = 1;
        ea.tol = p.tol;
        pamp_expm_block_df(ea, p.dt, exs);
        for (int q = tid; q < 2 * m; q += FZ_THREADS) cs[q] = pe[q];
        __syncthreads();
        // psi = sum_q c_q T_q (FP64)
        for (int i = tid; i < N; i += FZ_THREADS) {
            double ax = 0.0, ay = 0.0;
            for (int q = 0; q < k; ++q) {
                const cxf v = Tr[(size_t)q * tld + i];
                const double cx_ = cs[2 * q], cy = cs[2 * q + 1];
                ax = fma((double)v.x, cx_, ax);
                ax = fma(-(double)v.y, cy, ax);
                ay = fma((double)v.x, cy, ay);
                ay = fma((double)v.y, cx_, ay);
            }
            a.psi[(size_t)ch * N + i] = mk<double>(ax, ay);
        }
    }
    if (ch == 0 && tid == 0) {
        const double bad = k > 0 ? pe[2 * m + 4] : 0.0;
        p.ex[0] = k;
        p.ex[1] = k > 0 ? pe[2 * m + 3] : 0.0;
        p.ex[2] = bad;
        if (bad != 0.0) p.ex[3] = 1.0;
    }
}

// ------------------------------------------------------------------------------------
// host
// ------------------------------------------------------------------------------------
struct FusedPamp {
    PfArgs args;
    size_t smem = 0;
    int nctas = 0;
    void (*kern)(PfArgs) = nullptr;  // the instance for the band width and solve mode
    int solve = 0;                     // 0 factors through L2, 1 factors in shared memory, 2 dense S^-1
    int parity = 0;
    void *bufs[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};  // bands, source tables, S^-1, slots
};

// S^-1 in FP32 rows of sld floats (zero past N): S from the FP64 overlap rows on the device,
// Cholesky S = L L^T and the inverse column by column in FP64 on the host (set-up only)
static bool dense_inverse(pg_banded *ovl64, int N, int sld, std::vector<float> &out)
{
    const int kb = ovl64->kb, b = 2 * kb + 1;
    std::vector<double> rows((size_t)N * b);
    if (cudaMemcpy(rows.data(), ovl64->d_S, sizeof(double) * rows.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
        return false;
    std::vector<double> L((size_t)N * N, 0.0);
    for (int i = 0; i < N; ++i)
        for (int d = 0; d < b; ++d) {
            const int j = i + d - kb;
            if (j >= 0 && j <= i) L[(size_t)i * N + j] = rows[(size_t)i * b + d];
        }
    for (int j = 0; j < N; ++j) {  // in place: lower triangle of S -> L
        double djj = L[(size_t)j * N + j];
        for (int q = std::max(0, j - 2 * kb); q < j; ++q) djj -= L[(size_t)j * N + q] * L[(size_t)j * N + q];
        if (!(djj > 0.0)) return false;
        djj = std::sqrt(djj);
        L[(size_t)j * N + j] = djj;
        for (int i = j + 1; i < std::min(N, j + kb + 1); ++i) {
            double v = L[(size_t)i * N + j];
            for (int q = std::max(0, i - 2 * kb); q < j; ++q) v -= L[(size_t)i * N + q] * L[(size_t)j * N + q];
            L[(size_t)i * N + j] = v / djj;
        }
    }
    out.assign((size_t)N * sld, 0.f);
    std::vector<double> x(N);
    for (int c = 0; c < N; ++c) {
        for (int i = 0; i < N; ++i) {  // L y = e_c
            double v = i == c ? 1.0 : 0.0;
            for (int q = std::max(0, i - kb); q < i; ++q) v -= L[(size_t)i * N + q] * x[q];
            x[i] = v / L[(size_t)i * N + i];
        }
        for (int i = N - 1; i >= 0; --i) {  // L^T z = y
            double v = x[i];
            for (int q = i + 1; q < std::min(N, i + kb + 1); ++q) v -= L[(size_t)q * N + i] * x[q];
            x[i] = v / L[(size_t)i * N + i];
        }
        for (int i = 0; i < N; ++i) out[(size_t)i * sld + c] = (float)x[i];
    }
    return true;
}

int pg_pamp_fused_prepare(pg_op *opb, pg_banded *ovl64, pg_banded *ovlb, void *T, int m, double tol,
                          FusedPamp **out)
{
    if (!out) return PG_ERR_ARG;
    *out = nullptr;
    if (!opb || !ovl64 || !ovlb || !T) return PG_ERR_ARG;
    if (m < 2 || m > PF_MAXM) return PG_ERR_SHAPE;
    if (opb->rank != 2 || opb->precision != PG_FP32 || !opb->finalized) return PG_ERR_STORAGE;
    if (opb->ndense_entries > 0 || opb->fact.Q > 0) return PG_ERR_STORAGE;
    if (ovlb->kind != 0 || !ovlb->op || ovlb->op->precision != PG_FP32 || ovl64->kind != 0 || !ovl64->op ||
        ovl64->op->precision != PG_FP64)
        return PG_ERR_STORAGE;
    if (ovlb->N != opb->N || ovl64->N != opb->N || ovlb->kb != ovl64->kb || ovlb->kb < 1 || ovlb->kb > 32 ||
        !ovlb->d_S || !ovl64->d_S || !ovlb->d_lo_inv || !ovlb->d_up_inv)
        return PG_ERR_STORAGE;
    pg_ctx *ctx = opb->ctx;
    const int N = opb->N, nch = opb->nrows, nblk = (N + 31) / 32, w = ovlb->kb, kb = opb->kb;
    if (nch < 1 || N < 1) return PG_ERR_SHAPE;
    std::vector<float> rb32;
    if (!real_bands<float>(opb, rb32)) return PG_ERR_STORAGE;
    std::vector<int> ucol, nucol;
    std::vector<unsigned char> ent_u;
    if (!fz_source_tables(opb, ucol, nucol, ent_u)) return PG_ERR_STORAGE;
    const bool kb6 = (kb == 6);
    int max_e = 0;
    for (int r = 0; r < nch; ++r) max_e = std::max(max_e, opb->h_row_ptr[r + 1] - opb->h_row_ptr[r]);
    const size_t band_bytes = (size_t)max_e * (2 * kb + 1) * opb->ld * sizeof(float);
    const size_t npad = (size_t)nblk * 32;
    auto a16 = [](size_t b) { return (b + 15) / 16 * 16; };
    // shared memory: xs | ys sb sg xsrc [bands] [solve factors] (the exponential's scratch over
    // ys...) | [T]
    const size_t nbw = (size_t)nblk * w;
    const size_t fac_bytes = sizeof(float) * (2 * (size_t)nblk * 1024 + 2 * nbw * 32 + 2 * nbw * nbw);
    // the dense inverse's rows padded to 8 banks past a multiple of 32 words: the four rows a
    // warp reads at once fall in distinct banks
    const int sld = ((N + 23) / 32) * 32 + 8;
    const size_t dense_bytes = sizeof(float) * (size_t)N * sld;
    // neighbour channels per row (the cache slots of the staged sources)
    std::vector<signed char> uslot((size_t)nch * FZ_MAXU, -1);
    int ncache = 0;
    for (int r = 0; r < nch; ++r) {
        int c = 0;
        for (int u = 0; u < nucol[r]; ++u)
            if (ucol[(size_t)r * FZ_MAXU + u] != r) uslot[(size_t)r * FZ_MAXU + u] = (signed char)c++;
        ncache = std::max(ncache, c);
    }
    const size_t cache_bytes = (size_t)ncache * m * N * sizeof(cxf);
    struct Lay { size_t ys, sb, sg, xsrc, band, tab, T, cache, total; };
    auto layout = [&](int g_in_smem, int bands_smem, int v_smem, int solve, int cache) {
        Lay L;
        L.ys = npad * sizeof(cxf);
        L.sb = L.ys + npad * sizeof(cxf);
        L.sg = L.sb + (size_t)nblk * w * sizeof(cxf);
        L.xsrc = L.sg + (g_in_smem ? (size_t)nblk * w * 32 * sizeof(float) : 0);
        L.band = a16(L.xsrc + (size_t)FZ_MAXU * (N + 2 * kb) * sizeof(cxf));
        L.tab = a16(L.band + (bands_smem ? band_bytes : 0));
        const size_t work_end = L.tab + (solve == 2 ? dense_bytes : solve == 1 ? fac_bytes : 0);
        const size_t ex_end = L.ys + 6 * sizeof(float4) * (size_t)m * m;
        L.T = a16(std::max(work_end, ex_end));
        L.cache = a16(L.T + (v_smem ? (size_t)m * N * sizeof(cxf) : 0));
        L.total = L.cache + (cache ? cache_bytes : 0);
        return L;
    };
    // the opt-in shared memory of a CTA less room for the kernel's static arrays
    int optin = 0;
    PG_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
    const size_t limit = std::min<size_t>((size_t)std::max(optin, 48 * 1024) - 8 * 1024, 224 * 1024);
    // everything in shared memory where it fits (short fibres: the dense inverse; else the
    // blocked solve's factors); then without the bands, the factors, the Krylov vectors, the
    // couplings
    int g_in_smem = 0, bands_smem = 1, v_smem = 1, solve = N <= PF_DENSE_MAXN ? 2 : 1, use_cache = ncache > 0;
    Lay L = layout(0, 1, 1, solve, use_cache);
    if (L.total > limit && use_cache) { use_cache = 0; L = layout(0, 1, 1, solve, 0); }
    if (L.total > limit) { bands_smem = 0; L = layout(0, 0, 1, solve, 0); }
    if (L.total > limit && solve == 2) { solve = 1; L = layout(0, 0, 1, 1, 0); }
    if (L.total > limit) { solve = 0; g_in_smem = 1; L = layout(1, 0, 1, 0, 0); }
    if (L.total > limit) { v_smem = 0; L = layout(1, 0, 0, 0, 0); }
    if (L.total > limit) { g_in_smem = 0; L = layout(0, 0, 0, 0, 0); }
    if (L.total > limit) return PG_ERR_SHAPE;
    void (*kern)(PfArgs) = kb6 ? (solve == 2 ? pamp_fused_step_kernel<6, 2> : solve == 1 ? pamp_fused_step_kernel<6, 1>
                                                                                        : pamp_fused_step_kernel<6, 0>)
                               : (solve == 2 ? pamp_fused_step_kernel<-1, 2>
                                             : solve == 1 ? pamp_fused_step_kernel<-1, 1> : pamp_fused_step_kernel<-1, 0>);
    std::vector<float> sinv;
    if (solve == 2 && !dense_inverse(ovl64, N, sld, sinv)) return PG_ERR_STORAGE;
    PG_CUDA_TRY(raise_smem_limit((const void *)kern, L.total));
    int per_sm = 0;
    PG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, FZ_THREADS, L.total));
    if (per_sm < 1 || nch > per_sm * std::max(1, ctx->num_sms)) return PG_ERR_SHAPE;  // all CTAs resident

    FusedPamp *f = new FusedPamp();
    PfArgs &p = f->args;
    memset(&p, 0, sizeof(p));
    FzArgs &a = p.z;
    a.opb = opb->dev();
    a.nblk = nblk;
    a.w = w;
    a.fib_per_mat = std::max(1, ovlb->fib_per_mat);
    a.g_in_smem = g_in_smem;
    a.bands_smem = bands_smem;
    a.v_smem = v_smem;
    a.nch = nch;
    a.N = N;
    a.m = m;
    a.nctas = nch;
    a.V = (cxf *)T;
    p.slo_inv = (const float *)ovlb->d_lo_inv;
    p.slo_g = (const float *)ovlb->d_lo_cpl;
    p.slo_rb = (const float *)ovlb->d_lo_rb;
    p.sup_inv = (const float *)ovlb->d_up_inv;
    p.sup_g = (const float *)ovlb->d_up_cpl;
    p.sup_rb = (const float *)ovlb->d_up_rb;
    p.S32 = (const float *)ovlb->d_S;
    p.S64 = (const double *)ovl64->d_S;
    p.ks = ovlb->kb;
    p.off_ys = (int)L.ys;
    p.off_sb = (int)L.sb;
    p.off_sg = (int)L.sg;
    p.off_xsrc = (int)L.xsrc;
    p.off_band = (int)L.band;
    p.off_tab = (int)L.tab;
    p.off_T = (int)L.T;
    p.tol = tol;
    const size_t n = (size_t)nch * N;
    int code = PG_OK;
    auto alloc = [&](void **q, size_t bytes) {
        if (code == PG_OK && cudaMalloc(q, bytes) != cudaSuccess) code = PG_ERR_CUDA;
    };
    alloc((void **)&a.wbuf, sizeof(cxf) * 2 * n);
    alloc((void **)&a.part, sizeof(double) * P_COUNT * (size_t)nch * PF_PSTRIDE);
    alloc((void **)&a.bar, 2 * sizeof(FzBarrier));
    alloc((void **)&p.hcols, sizeof(double) * (size_t)nch * m * 3 * 2 * (m + 2));
    alloc((void **)&p.pe, sizeof(double) * (size_t)nch * PF_PE);
    if (code == PG_OK && cudaMemset(a.bar, 0, 2 * sizeof(FzBarrier)) != cudaSuccess) code = PG_ERR_CUDA;
    if (code == PG_OK && cudaMemset(p.hcols, 0, sizeof(double) * (size_t)nch * m * 3 * 2 * (m + 2)) != cudaSuccess)
        code = PG_ERR_CUDA;
    if (code == PG_OK) code = upload_vec(rb32, &f->bufs[0]);
    if (code == PG_OK) code = upload_vec(ucol, &f->bufs[1]);
    if (code == PG_OK) code = upload_vec(nucol, &f->bufs[2]);
    if (code == PG_OK) code = upload_vec(ent_u, &f->bufs[3]);
    if (code == PG_OK && solve == 2) code = upload_vec(sinv, &f->bufs[4]);
    if (code == PG_OK && use_cache) code = upload_vec(uslot, &f->bufs[5]);
    if (code != PG_OK) {
        pg_pamp_fused_free(f);
        return code;
    }
    a.rb32 = (const float *)f->bufs[0];
    a.ucol = (const int *)f->bufs[1];
    a.nucol = (const int *)f->bufs[2];
    a.ent_u = (const unsigned char *)f->bufs[3];
    p.sinv = (const float *)f->bufs[4];
    p.sld = sld;
    p.uslot = (const signed char *)f->bufs[5];
    p.ncache = use_cache ? ncache : 0;
    p.off_cache = (int)L.cache;
    f->smem = L.total;
    f->nctas = nch;
    f->kern = kern;
    f->solve = solve;
    *out = f;
    return PG_OK;
}

int pg_pamp_fused_launch(FusedPamp *f, cudaStream_t s, cxd *psi, double dt, const cxd *h, double *ex, int *err)
{
    PfArgs p = f->args;
    p.z.psi = psi;
    p.z.err = err;
    p.dt = dt;
    for (int q = 0; q < PG_MAX_SLOTS; ++q) p.h[q] = h[q];
    p.ex = ex;
    // launches alternate between two arrival counters, each clearing the other at its start
    p.z.bar = f->args.z.bar + f->parity;
    p.z.bar_next = f->args.z.bar + (1 - f->parity);
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
    PG_CUDA_TRY(cudaLaunchKernelEx(&cfg, f->kern, p));
    return PG_OK;
}

void pg_pamp_fused_set_probe(FusedPamp *f, unsigned int extra_arrivals, unsigned int at_barrier)
{
    if (!f) return;
    f->args.z.probe_extra = extra_arrivals;
    f->args.z.probe_at = at_barrier;
}

void pg_pamp_fused_free(FusedPamp *f)
{
    if (!f) return;
    cudaFree(f->args.z.wbuf);
    cudaFree(f->args.z.part);
    cudaFree(f->args.z.bar);
    cudaFree(f->args.hcols);
    cudaFree(f->args.pe);
    for (void *b : f->bufs) cudaFree(b);
    delete f;
}
