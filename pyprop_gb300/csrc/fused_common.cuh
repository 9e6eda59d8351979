// Device helpers shared by the single-kernel steps (cayley_fused.cu: Crank-Nicolson GMRES;
// pamp_fused.cu: pAMP): cooperative launch with one CTA per angular channel, bounded grid
// barriers, channel sums reduced in a fixed order (identical in every CTA), the complex64 row
// product of a channel from its staged neighbour fibres.
#pragma once
#include "cayley_state.cuh"
#include "tri_solve.cuh"

#include <algorithm>
#include <complex>
#include <mutex>
#include <vector>

static const int FZ_NW = 24;                 // warps per CTA (the block solve's width for long fibres)
static const int FZ_THREADS = 32 * FZ_NW;
static const int FZ_MAXM = 32;               // Krylov basis bound of the single-kernel step
static const int FZ_CB = 8;                  // columns per register block of the channel sums
static const int FZ_MAXPASS = 4;             // refinement passes (as the multi-kernel step)
static const int FZ_PSTRIDE = 2 * (FZ_MAXM + 1);
static const int FZ_MAXU = 4;                // distinct source channels per operator row (staged)
static const unsigned int FZ_POLLS = 1u << 22;  // barrier polls (each an L2 round trip) before giving up
enum { P_NRM = 0, P_H1 = 1, P_H2 = 2, P_RES = 3, P_COUNT = 4 };

struct FzBarrier {
    unsigned int count;  // arrivals during the current launch
    unsigned int pad;
};

struct FzArgs {
    OpDev op64, opb;             // structure (rows, entries, slots); the bands are the real copies below
    const double *rb64;          // [bands][2kb+1][ld] real FP64 bands of op64
    const float *rb32;           // [bands][2kb+1][ld] real FP32 bands of opb
    const int *ucol;             // [Nang][FZ_MAXU] distinct source channels of each row of opb
    const int *nucol;            // [Nang] how many
    const unsigned char *ent_u;  // [entries of opb] which staged source an entry reads
    const int *row_lo;           // [CTAs + 1] FP64 rows of each CTA (equal numbers of band entries)
    int bands_smem;              // 1: each channel's FP32 bands are copied to shared memory per step
    int v_smem;                  // 1: a channel's Krylov vectors are also kept in shared memory
    unsigned int probe_extra;    // test hook: arrivals barrier number probe_at waits for in addition (0)
    unsigned int probe_at;
    int cl_bpc, cl_rpc, cl_rbmax;  // cluster kernel: blocks and boundary rows per CTA, packed Rb entries
    int nctas;                   // the grid the per-CTA tables are sized for
    const cxf *lo_inv, *lo_g, *lo_rb, *up_inv, *up_g, *up_rb;
    int nblk, w, fib_per_mat, g_in_smem;
    int nch, N, m;
    double tol;
    StepParams params;  // this step's dt and slot values (kernel argument)
    GmresStats *hstats; // mapped host memory: the step's statistics at its end (or null)
    int *herr;          // mapped host memory: the error word at the step's end (or null)
    cxd *psi;
    cxd *r64;        // [nch*N] FP64 residual (rows spread over the CTAs)
    cxd *e64;        // [nch*N] correction of the pass (read across channels by the FP64 rows)
    cxf *wbuf;       // [2][nch*N] unnormalised next Krylov vector (read across channels)
    cxf *V;          // [m][nch*N] Krylov vectors (channel a written by CTA a only)
    double *part;    // [P_COUNT][CTAs][FZ_PSTRIDE] per-CTA partial sums
    FzBarrier *bar;      // this launch's arrival counter (launches alternate between two)
    FzBarrier *bar_next; // the other one, cleared by this launch for the next
    GmresState *st;
    int *err;
};

__device__ __forceinline__ unsigned int fz_ld_acquire(const unsigned int *p)
{
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// All CTAs meet (the launch is cooperative, so all are resident): the arrival count only
// grows during a launch (it is zeroed before each), the k-th barrier completes when it
// reaches k * gridDim.x. Returns false, CTA-uniform, when the wait ran out; the error flag is
// then set. `ordinal` counts the barriers of the launch (thread 0); the test hook makes
// barrier number probe_at wait for probe_extra arrivals that no CTA makes.
__device__ __forceinline__ bool fz_grid_sync(FzBarrier *bar, unsigned int &target, unsigned int &ordinal,
                                             const FzArgs &a, int *s_ok)
{
    int *err = a.err;
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
            atomicExch(err, 2);
            if (a.herr) *(volatile int *)a.herr = 2;
        }
        *s_ok = ok;
    }
    __syncthreads();
    return *s_ok != 0;
}

template <typename R> __device__ __forceinline__ R fz_warp_sum(R v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ cxf fz_ldcg(const cxf *p)
{
    const float2 v = __ldcg((const float2 *)p);
    return mk<float>(v.x, v.y);
}
__device__ __forceinline__ cxd fz_ldcg(const cxd *p)
{
    const double2 v = __ldcg((const double2 *)p);
    return mk<double>(v.x, v.y);
}

// Sum over the channels of the partials of one phase: hs[t] = sum_a part[a][t], t < nval,
// one warp per value, the channels over the lanes, a fixed order (identical in every CTA);
// FP64 sums, stored as T (float for what enters the FP32 Givens recurrence).
template <typename T>
__device__ __forceinline__ void fz_reduce(const double *part, int nch, int nval, T *hs)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int t = warp; t < nval; t += FZ_NW) {
        double s = 0.0;
        for (int a = lane; a < nch; a += 32) s += __ldcg(part + (size_t)a * FZ_PSTRIDE + t);
        s = fz_warp_sum(s);
        if (lane == 0) hs[t] = (T)s;
    }
    __syncthreads();
}

// CTA sum of one FP64 value per thread into out[0] (FP64 throughout)
__device__ __forceinline__ void fz_cta_sum64(double v, double (*red)[2 * FZ_CB], double *out)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = fz_warp_sum(v);
    if (lane == 0) red[warp][0] = v;
    __syncthreads();
    if (warp == 0) {
        double s = lane < FZ_NW ? red[lane][0] : 0.0;
        s = fz_warp_sum(s);
        if (lane == 0) out[0] = s;
    }
    __syncthreads();
}

// Channel sums of the complex64 fibre xs: out[2q], out[2q+1] = <V_q, xs> for q < J (dots),
// out[0] = ||xs||^2 (norm_only); with_norm also out[2J] = ||xs||^2 beside the dots. Element
// sums in FP32 per thread and warp, CTA sums in FP64.
__device__ __forceinline__ void fz_channel_sums(const cxf *Vc, long long ldv, int J, bool norm_only, const cxf *xs,
                                                int N, double (*red)[2 * FZ_CB], double *out, bool with_norm = false)
{
    float n2 = 0.f;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int ncol = norm_only ? 1 : J;
    for (int j0 = 0; j0 < ncol; j0 += FZ_CB) {
        float ax[FZ_CB], ay[FZ_CB];
#pragma unroll
        for (int q = 0; q < FZ_CB; ++q) ax[q] = ay[q] = 0.f;
        for (int i = threadIdx.x; i < N; i += FZ_THREADS) {
            const cxf b = xs[i];
            if (norm_only) {
                ax[0] = fmaf(b.x, b.x, ax[0]);
                ax[0] = fmaf(b.y, b.y, ax[0]);
            } else {
                if (with_norm && j0 == 0) {
                    n2 = fmaf(b.x, b.x, n2);
                    n2 = fmaf(b.y, b.y, n2);
                }
#pragma unroll
                for (int q = 0; q < FZ_CB; ++q)
                    if (j0 + q < J) {
                        const cxf v = Vc[(size_t)(j0 + q) * ldv + i];
                        ax[q] = fmaf(v.x, b.x, ax[q]);
                        ax[q] = fmaf(v.y, b.y, ax[q]);
                        ay[q] = fmaf(v.x, b.y, ay[q]);
                        ay[q] = fmaf(-v.y, b.x, ay[q]);
                    }
            }
        }
#pragma unroll
        for (int q = 0; q < FZ_CB; ++q) {
            if (j0 + q < ncol) {  // CTA-uniform
                const float sx = fz_warp_sum(ax[q]);
                const float sy = fz_warp_sum(ay[q]);
                if (lane == 0) {
                    red[warp][2 * q] = (double)sx;
                    red[warp][2 * q + 1] = (double)sy;
                }
            }
        }
        __syncthreads();
        // warp v sums value v over the warps (lanes), a shuffle tree in FP64
        if (warp < 2 * FZ_CB && j0 + warp / 2 < ncol) {
            double s = lane < FZ_NW ? red[lane][warp] : 0.0;
            s = fz_warp_sum(s);
            if (lane == 0) out[2 * j0 + warp] = s;
        }
        __syncthreads();
    }
    if (with_norm && !norm_only) fz_cta_sum64((double)n2, red, out + 2 * J);
}

// acc -= sum_q V_q h_q over q < J (complex64, FMAs in a fixed order): the classical
// Gram-Schmidt update of one element. The owner of a channel and the CTAs that stage its fibre
// for their products run this same code on the same values, so they form the same vector.
// CG: V is another CTA's global data, read through L2 (L1 may hold lines of an earlier pass).
template <bool CG>
__device__ __forceinline__ cxf fz_gs_update(cxf acc, const cxf *V, long long ldv, int J, const cxf *hs)
{
    for (int q0 = 0; q0 < J; q0 += FZ_CB) {
        cxf v[FZ_CB];  // FZ_CB vectors' loads in flight together
#pragma unroll
        for (int q = 0; q < FZ_CB; ++q)
            v[q] = q0 + q < J ? (CG ? fz_ldcg(V + (size_t)(q0 + q) * ldv) : V[(size_t)(q0 + q) * ldv])
                              : mk<float>(0.f, 0.f);
#pragma unroll
        for (int q = 0; q < FZ_CB; ++q) {
            if (q0 + q >= J) break;
            const cxf hc = hs[q0 + q];
            acc.x = fmaf(-v[q].x, hc.x, acc.x);
            acc.x = fmaf(v[q].y, hc.y, acc.x);
            acc.y = fmaf(-v[q].x, hc.y, acc.y);
            acc.y = fmaf(-v[q].y, hc.x, acc.y);
        }
    }
    return acc;
}

// FP64 rows [lo, hi) of the flattened [Nang][N] operator applied to src (read through L2:
// other CTAs write it): r[o] (+)= sum_e sc[slot_e] sum_d band_e[d][i] src[col_e][i + d - kb],
// o = a N + i, real bands. A row's entries are spread over FZ_RG neighbouring lanes (entry
// e0 + g, e0 + g + FZ_RG, ... on lane g of the group) and summed by shuffles in a fixed order,
// so a CTA's rows (a few hundred) keep all its warps' loads in flight at once. Returns this
// thread's share of ||r||^2 over its rows.
static const int FZ_RG = 4;
template <int KB>
__device__ __forceinline__ double fz_rows64(const OpDev &op, const double *__restrict__ rb, long long lo, long long hi,
                                            const cxd *sc, const cxd *src, cxd *r, bool accumulate)
{
    const int N = op.N, kb = KB >= 0 ? KB : op.kb, b = 2 * kb + 1, ld = op.ld;
    const int g = threadIdx.x & (FZ_RG - 1);
    double nrm = 0.0;
    for (long long base = lo; base < hi; base += FZ_THREADS / FZ_RG) {  // uniform over the CTA
        const long long o = base + threadIdx.x / FZ_RG;
        cxd acc = mk<double>(0.0, 0.0);
        if (o < hi) {
            const int a = (int)(o / N), i = (int)(o - (long long)a * N);
            const int e0 = __ldg(op.row_ptr + a), e1 = __ldg(op.row_ptr + a + 1);
            for (int e = e0 + g; e < e1; e += FZ_RG) {
                const cxd se = sc[__ldg(op.ent_slot + e)];
                if (se.x == 0.0 && se.y == 0.0) continue;  // e.g. the overlap in -i dt H psi
                const double *B = rb + (size_t)__ldg(op.ent_band + e) * b * ld + i;
                const cxd *x = src + (size_t)__ldg(op.ent_col + e) * N + i - kb;
                double tx = 0.0, ty = 0.0;
                if (KB >= 0) {
#pragma unroll
                    for (int d = 0; d < 2 * KB + 1; ++d)
                        if (i + d - kb >= 0 && i + d - kb < N) {
                            const double c = __ldg(B + (size_t)d * ld);
                            const cxd v = fz_ldcg(x + d);
                            tx = fma(c, v.x, tx);
                            ty = fma(c, v.y, ty);
                        }
                } else {
                    for (int d = 0; d < b; ++d)
                        if (i + d - kb >= 0 && i + d - kb < N) {
                            const double c = __ldg(B + (size_t)d * ld);
                            const cxd v = fz_ldcg(x + d);
                            tx = fma(c, v.x, tx);
                            ty = fma(c, v.y, ty);
                        }
                }
                cfma(acc, se, mk<double>(tx, ty));
            }
        }
#pragma unroll
        for (int off = 1; off < FZ_RG; off <<= 1) {
            acc.x += __shfl_xor_sync(0xffffffffu, acc.x, off);
            acc.y += __shfl_xor_sync(0xffffffffu, acc.y, off);
        }
        if (o < hi && g == 0) {
            if (accumulate) acc = acc + fz_ldcg(r + o);
            r[o] = acc;
            nrm = fma(acc.x, acc.x, nrm);
            nrm = fma(acc.y, acc.y, nrm);
        }
    }
    return nrm;
}

// Copy the real FP32 bands of operator row a ([entry][2kb+1][ld] in entry order) to shared
// memory with asynchronous 16-byte copies (cp.async; waited for by fz_bands_wait).
__device__ __forceinline__ void fz_bands_load(const FzArgs &A, int a, float *sband)
{
    const OpDev &op = A.opb;
    const int b = 2 * op.kb + 1, ld = op.ld;  // ld: a multiple of 4, so every row is 16-byte aligned
    const int e0 = __ldg(op.row_ptr + a), e1 = __ldg(op.row_ptr + a + 1);
    const int per = b * ld / 4;  // 16-byte pieces per entry
    for (int q = threadIdx.x; q < (e1 - e0) * per; q += FZ_THREADS) {
        const int e = q / per, r = q - e * per;
        const float *src = A.rb32 + (size_t)__ldg(op.ent_band + e0 + e) * b * ld + 4 * (size_t)r;
        const unsigned dst = (unsigned)__cvta_generic_to_shared(sband + (size_t)e * b * ld + 4 * (size_t)r);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void fz_bands_wait()
{
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncthreads();
}

// complex64 operator row a applied to the normalised vector (wsrc - V hs) * s: the row's
// distinct source fibres are staged (the Gram-Schmidt correction by the first Jc Krylov
// vectors of the source channel applied, scaled, with a zero halo of kb) in xsrc, then thread
// i forms xs[i] = sum_e sc[slot_e] sum_d band_e[d][i] x_e[i + d - kb] from real bands (in
// shared memory when sband is set, else read through L1); zero on the padding up to npad.
template <int KB>
__device__ __forceinline__ void fz_rowprod32(const FzArgs &A, int a, const cxf *sc, cxf *xs, int npad,
                                             const cxf *xsrc, const float *sband);

template <int KB>
__device__ __forceinline__ void fz_matvec32(const FzArgs &A, int a, const cxf *sc, const cxf *wsrc, float s, cxf *xs,
                                            int npad, cxf *xsrc, const float *sband, int Jc, const cxf *hs)
{
    const long long nall = (long long)A.nch * A.N;
    const OpDev &op = A.opb;
    const int N = op.N, kb = KB >= 0 ? KB : op.kb, b = 2 * kb + 1, ld = op.ld, W = N + 2 * kb;
    const int nu = __ldg(A.nucol + a);
    int cols[FZ_MAXU];
#pragma unroll
    for (int u = 0; u < FZ_MAXU; ++u) cols[u] = u < nu ? __ldg(A.ucol + (size_t)a * FZ_MAXU + u) : 0;
    // all staged elements of a thread loaded together (nu W elements over the CTA)
    for (int base = 0; base < nu * W; base += FZ_THREADS * FZ_MAXU) {
        cxf v[FZ_MAXU];
#pragma unroll
        for (int k = 0; k < FZ_MAXU; ++k) {
            const int idx = base + threadIdx.x + k * FZ_THREADS;
            const int u = idx / W, q = idx - u * W, j = q - kb;
            v[k] = (idx < nu * W && j >= 0 && j < N) ? fz_ldcg(wsrc + (size_t)cols[u < FZ_MAXU ? u : 0] * N + j)
                                                     : mk<float>(0.f, 0.f);
        }
        if (Jc > 0) {
#pragma unroll
            for (int k = 0; k < FZ_MAXU; ++k) {
                const int idx = base + threadIdx.x + k * FZ_THREADS;
                const int u = idx / W, q = idx - u * W, j = q - kb;
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
    fz_rowprod32<KB>(A, a, sc, xs, npad, xsrc, sband);
}

// The row product of fz_matvec32 from source fibres already staged in xsrc ([nu][N + 2kb],
// zero halo of kb; callers synchronise the CTA after staging): thread i forms
// xs[i] = sum_e sc[slot_e] sum_d band_e[d][i] x_e[i + d - kb], zero on the padding up to npad.
template <int KB>
__device__ __forceinline__ void fz_rowprod32(const FzArgs &A, int a, const cxf *sc, cxf *xs, int npad,
                                             const cxf *xsrc, const float *sband)
{
    const OpDev &op = A.opb;
    const int N = op.N, kb = KB >= 0 ? KB : op.kb, b = 2 * kb + 1, ld = op.ld, W = N + 2 * kb;
    const int e0 = __ldg(op.row_ptr + a), e1 = __ldg(op.row_ptr + a + 1);
    for (int i = threadIdx.x; i < npad; i += FZ_THREADS) {
        cxf acc = mk<float>(0.f, 0.f);
        if (i < N) {
            for (int e = e0; e < e1; e += 2) {
                // two entries at a time: 2(2kb+1) band loads in flight
                const bool two = e + 1 < e1;
                const int e1s = two ? e + 1 : e;
                const float *B0 = sband ? sband + (size_t)(e - e0) * b * ld + i
                                        : A.rb32 + (size_t)__ldg(op.ent_band + e) * b * ld + i;
                const float *B1 = sband ? sband + (size_t)(e1s - e0) * b * ld + i
                                        : A.rb32 + (size_t)__ldg(op.ent_band + e1s) * b * ld + i;
                const cxf *x0 = xsrc + (size_t)__ldg(A.ent_u + e) * W + i;  // x[d] = x_e[i + d - kb]
                const cxf *x1 = xsrc + (size_t)__ldg(A.ent_u + (two ? e + 1 : e)) * W + i;
                float t0x = 0.f, t0y = 0.f, t1x = 0.f, t1y = 0.f;
                if (KB >= 0) {
                    float c0[2 * (KB > 0 ? KB : 0) + 1], c1[2 * (KB > 0 ? KB : 0) + 1];
#pragma unroll
                    for (int d = 0; d < 2 * KB + 1; ++d) {
                        c0[d] = sband ? B0[(size_t)d * ld] : __ldg(B0 + (size_t)d * ld);
                        c1[d] = sband ? B1[(size_t)d * ld] : __ldg(B1 + (size_t)d * ld);
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
                        const float c = sband ? B0[(size_t)d * ld] : __ldg(B0 + (size_t)d * ld);
                        const float c2 = sband ? B1[(size_t)d * ld] : __ldg(B1 + (size_t)d * ld);
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


// A launch whose shape differs from the one the tables were built for (another grid size, or
// the cluster kernel without its clusters) touches nothing: CTA 0 reports error word 4 in the
// device word and the mapped host copies, and every CTA returns.
__device__ __forceinline__ bool fz_bad_launch(const FzArgs &a, bool bad)
{
    if (!bad) return false;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        atomicExch(a.err, 4);
        if (a.herr) *(volatile int *)a.herr = 4;
        if (a.hstats) *(volatile int *)&a.hstats->passes = 0;
        __threadfence_system();
    }
    return true;
}

// ---- host helpers of the set-ups ------------------------------------------------------------
// The kernels' dynamic shared-memory limit only ever rises (the attribute is per function, not
// per stepper: lowering it for a smaller operator would make a larger stepper's launch fail).
static cudaError_t raise_smem_limit(const void *kern, size_t bytes)
{
    static std::mutex mu;
    std::lock_guard<std::mutex> lock(mu);
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, kern);
    if (e != cudaSuccess) return e;
    if ((size_t)fa.maxDynamicSharedSizeBytes >= bytes) return cudaSuccess;
    return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// real copy of an operator's bands in the device layout [band][2kb+1][ld]; false when a band
// has a non-zero imaginary part
template <typename R>
static bool real_bands(const pg_op *op, std::vector<R> &out)
{
    const size_t rows = op->h_bands.size() / (size_t)op->N;
    out.assign(rows * (size_t)op->ld, (R)0);
    for (size_t q = 0; q < rows; ++q)
        for (int i = 0; i < op->N; ++i) {
            const std::complex<double> v = op->h_bands[q * op->N + i];
            if (v.imag() != 0.0) return false;
            out[q * op->ld + i] = (R)v.real();
        }
    return true;
}

template <typename T>
static int upload_vec(const std::vector<T> &v, void **dst)
{
    PG_CUDA_TRY(cudaMalloc(dst, std::max<size_t>(1, v.size()) * sizeof(T)));
    if (!v.empty()) PG_CUDA_TRY(cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return PG_OK;
}

// Distinct source channels of each row of opb (at most FZ_MAXU; false when a row has more) and,
// per entry, which of them it reads: the row product stages each source fibre once.
static bool fz_source_tables(const pg_op *opb, std::vector<int> &ucol, std::vector<int> &nucol,
                             std::vector<unsigned char> &ent_u)
{
    const int nch = opb->nrows;
    ucol.assign((size_t)nch * FZ_MAXU, 0);
    nucol.assign(nch, 0);
    ent_u.assign(opb->h_ent_col.size(), 0);
    for (int r = 0; r < nch; ++r)
        for (int e = opb->h_row_ptr[r]; e < opb->h_row_ptr[r + 1]; ++e) {
            const int col = opb->h_ent_col[e];
            int u = 0;
            while (u < nucol[r] && ucol[(size_t)r * FZ_MAXU + u] != col) ++u;
            if (u == nucol[r]) {
                if (u == FZ_MAXU) return false;
                ucol[(size_t)r * FZ_MAXU + u] = col;
                nucol[r] = u + 1;
            }
            ent_u[e] = (unsigned char)u;
        }
    return true;
}
