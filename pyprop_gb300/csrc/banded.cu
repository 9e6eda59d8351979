// Banded fibre operators along the B-spline rank.
//
//  * overlap S = U^T U (real, kb super diagonals): U x, U^T x, U^-1 x, U^-T x, S x, S^-1 x
//    - the operations of OverlapMatrix (core/representation/overlapmatrix.cpp:123-149,
//    zpbtrf upper factor :23-37) applied to every fibre psi[a][:];
//  * block-diagonal preconditioner M_a = cS S + cH H_a per angular channel a, factored
//    M_a = L_a U_a without pivoting - the role of BSplineSolver (zgbtrf/zgbtrs,
//    core/transform/bspline/bsplinesolver.h:43-162). M_a has the positive definite
//    Hermitian part Re(cS) S (cS = 1, cH = i dt/2 in the Cayley step), for which
//    elimination without pivoting is stable.
//
// Triangular solves: one warp per fibre, 32-row blocks. Lane t owns row 32*blk + t. The
// coupling to the neighbouring block (at most kb rows) is subtracted with warp shuffles,
// then the precomputed inverse of the 32x32 diagonal block is applied (32 shuffles + FMAs).
// The sequential dependency is one block (not one row) per step.
#include "pg_internal.cuh"

#include <algorithm>
#include <cmath>

typedef std::complex<double> zd;

// ------------------------------------------------------------------------------------
// kernels
// ------------------------------------------------------------------------------------
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

// Asynchronous 16-byte global->shared copies (cp.async, completion by group wait).
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N> __device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

// One CTA of NW warps per fibre. Per 32-row block the inverse diagonal block and the
// coupling rows are copied to shared memory with cp.async TRI_STAGES-1 blocks ahead, so the
// solve reads only shared memory. Lane t of every warp owns row 32*blk + t; warp w forms the
// partial product of the inverse block over columns s in [w*32/NW, (w+1)*32/NW) and warp 0
// sums the partials. NW > 1 spreads FP64 work over the SM's sub-partitions (one warp runs on
// one sub-partition, which has a quarter of the SM's FP64 rate).
// C: coefficient type (R or cx<R>). inv: [nmat][nblk][32 s][32 t], cpl: [nmat][nblk][w][32 t]
static const int TRI_STAGES = 4;

__device__ __forceinline__ void cp_async_wait_dyn(int pending)
{
    // pending groups allowed to remain in flight (0 .. TRI_STAGES-1)
    if (pending >= 3) cp_async_wait<3>();
    else if (pending == 2) cp_async_wait<2>();
    else if (pending == 1) cp_async_wait<1>();
    else cp_async_wait<0>();
}

template <typename R, typename C, bool LOWER, int NW>
__global__ void __launch_bounds__(32 * NW) tri_solve_kernel(int N, int nblk, int w, const C *__restrict__ inv,
                                                            const C *__restrict__ cpl, int per_fibre_matrix,
                                                            cx<R> *__restrict__ x, int nfib)
{
    extern __shared__ __align__(16) unsigned char tri_smem[];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int f = blockIdx.x;
    if (f >= nfib) return;
    const int per_blk = 1024 + w * 32;  // coefficients staged per block
    C *buf = (C *)tri_smem;
    cx<R> *part = (cx<R> *)(buf + (size_t)TRI_STAGES * per_blk);  // [NW][32]
    cx<R> *ybuf = part + NW * 32;                                   // [32] solution of the previous block
    const size_t m = per_fibre_matrix ? (size_t)f : 0;
    cx<R> *xf = x + (size_t)f * N;
    const C *invm = inv + m * (size_t)nblk * 1024;
    const C *cplm = cpl + m * (size_t)nblk * w * 32;
    const int chunks_inv = (int)(1024 * sizeof(C) / 16);
    const int chunks_cpl = (int)(w * 32 * sizeof(C) / 16);
    auto prefetch = [&](int step) {
        const int blk = LOWER ? step : (nblk - 1 - step);
        C *dst = buf + (size_t)(step % TRI_STAGES) * per_blk;
        const unsigned char *gi = (const unsigned char *)(invm + (size_t)blk * 1024);
        const unsigned char *gc = (const unsigned char *)(cplm + (size_t)blk * w * 32);
        unsigned char *si = (unsigned char *)dst;
        unsigned char *sc = (unsigned char *)(dst + 1024);
        for (int c = threadIdx.x; c < chunks_inv; c += 32 * NW) cp_async16(si + 16 * c, gi + 16 * c);
        for (int c = threadIdx.x; c < chunks_cpl; c += 32 * NW) cp_async16(sc + 16 * c, gc + 16 * c);
        cp_async_commit();
    };
    for (int k = 0; k < TRI_STAGES - 1 && k < nblk; ++k) prefetch(k);
    if (threadIdx.x < 32) ybuf[lane] = mk<R>((R)0, (R)0);
    constexpr int SPW = 32 / NW;  // inverse columns per warp
    for (int step = 0; step < nblk; ++step) {
        if (step + TRI_STAGES - 1 < nblk) prefetch(step + TRI_STAGES - 1);
        cp_async_wait_dyn(min(TRI_STAGES - 1, nblk - 1 - step));
        __syncthreads();
        const C *ib = buf + (size_t)(step % TRI_STAGES) * per_blk;
        const C *cb = ib + 1024;
        const int blk = LOWER ? step : (nblk - 1 - step);
        const int row = blk * 32 + lane;
        cx<R> r = (row < N) ? xf[row] : mk<R>((R)0, (R)0);
        if (step > 0) {
            for (int j = 1; j <= w; ++j) {
                // LOWER: row couples to row-j in the previous block when lane < j
                // UPPER: row couples to row+j in the next block when lane >= 32-j
                const int src_lane = LOWER ? (32 - j + lane) & 31 : (lane + j - 32) & 31;
                const bool use = LOWER ? (lane < j) : (lane >= 32 - j);
                if (use) coef_fms(r, cb[(j - 1) * 32 + lane], ybuf[src_lane]);
            }
        }
        cx<R> acc[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) acc[a] = mk<R>((R)0, (R)0);
#pragma unroll
        for (int q = 0; q < SPW; ++q) {
            const int s = warp * SPW + q;
            coef_fma(acc[q & 3], ib[s * 32 + lane], shfl_cx(r, s));
        }
        cx<R> y = (acc[0] + acc[1]) + (acc[2] + acc[3]);
        if (NW > 1) {
            part[warp * 32 + lane] = y;
            __syncthreads();
            if (warp == 0) {
                y = part[lane];
#pragma unroll
                for (int q = 1; q < NW; ++q) y = y + part[q * 32 + lane];
            }
        }
        if (warp == 0) {
            if (row < N) xf[row] = y;
            ybuf[lane] = y;
        }
        __syncthreads();  // ybuf ready; the stage buffer may be refilled
    }
}

// U x (up=1) or U^T x (up=0), U real upper with kb super diagonals, rows [N][kb+1]
template <typename R>
__global__ void tri_mul_kernel(int N, int kb, const R *__restrict__ U, const cx<R> *__restrict__ x,
                               cx<R> *__restrict__ y, int up)
{
    const int f = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const cx<R> *xf = x + (size_t)f * N;
    cx<R> acc = mk<R>((R)0, (R)0);
    if (up) {
        for (int j = 0; j <= kb && i + j < N; ++j) coef_fma(acc, U[(size_t)i * (kb + 1) + j], xf[i + j]);
    } else {
        for (int j = 0; j <= kb && i - j >= 0; ++j) coef_fma(acc, U[(size_t)(i - j) * (kb + 1) + j], xf[i - j]);
    }
    y[(size_t)f * N + i] = acc;
}

// S x with S rows [N][2kb+1]
template <typename R>
__global__ void band_mul_kernel(int N, int kb, const R *__restrict__ S, const cx<R> *__restrict__ x,
                                cx<R> *__restrict__ y)
{
    const int f = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const cx<R> *xf = x + (size_t)f * N;
    cx<R> acc = mk<R>((R)0, (R)0);
    for (int d = 0; d <= 2 * kb; ++d) {
        const int j = i + d - kb;
        if (j >= 0 && j < N) coef_fma(acc, S[(size_t)i * (2 * kb + 1) + d], xf[j]);
    }
    y[(size_t)f * N + i] = acc;
}

// ------------------------------------------------------------------------------------
// host: factorizations and block inverses (complex128 / float64)
// ------------------------------------------------------------------------------------
namespace {

// dense 32x32 triangular block inverse; T given as dense row-major [32][32]
void invert_triangular_32(const zd *T, bool lower, zd *Tinv)
{
    for (int c = 0; c < 32; ++c) {
        zd col[32];
        for (int r = 0; r < 32; ++r) col[r] = (r == c) ? zd(1.0, 0.0) : zd(0.0, 0.0);
        if (lower) {
            for (int r = 0; r < 32; ++r) {
                zd s = col[r];
                for (int q = 0; q < r; ++q) s -= T[r * 32 + q] * col[q];
                col[r] = s / T[r * 32 + r];
            }
        } else {
            for (int r = 31; r >= 0; --r) {
                zd s = col[r];
                for (int q = r + 1; q < 32; ++q) s -= T[r * 32 + q] * col[q];
                col[r] = s / T[r * 32 + r];
            }
        }
        for (int r = 0; r < 32; ++r) Tinv[r * 32 + c] = col[r];
    }
}

// Build block data for a triangular matrix given by accessor A(i, j) (band width w).
// inv[blk][s][t] = Tinv[t][s]; cpl[blk][j-1][t] = A(row, row -/+ j) for the cross-block part.
template <typename Acc>
void build_blocks(int N, int w, bool lower, Acc A, std::vector<zd> &inv, std::vector<zd> &cpl)
{
    const int nblk = (N + 31) / 32;
    inv.assign((size_t)nblk * 1024, zd(0.0, 0.0));
    cpl.assign((size_t)nblk * w * 32, zd(0.0, 0.0));
    std::vector<zd> T(1024), Ti(1024);
    for (int blk = 0; blk < nblk; ++blk) {
        const int r0 = blk * 32;
        for (int t = 0; t < 32; ++t)
            for (int s = 0; s < 32; ++s) {
                const int i = r0 + t, j = r0 + s;
                zd v(0.0, 0.0);
                if (i < N && j < N) {
                    if (std::abs(i - j) <= w && (lower ? j <= i : j >= i)) v = A(i, j);
                } else if (i == j) {
                    v = zd(1.0, 0.0);  // identity padding past N
                }
                T[t * 32 + s] = v;
            }
        invert_triangular_32(T.data(), lower, Ti.data());
        for (int s = 0; s < 32; ++s)
            for (int t = 0; t < 32; ++t) inv[(size_t)blk * 1024 + s * 32 + t] = Ti[t * 32 + s];
        for (int j = 1; j <= w; ++j)
            for (int t = 0; t < 32; ++t) {
                const int i = r0 + t;
                const int col = lower ? i - j : i + j;
                const bool cross = lower ? (t < j) : (t >= 32 - j);
                if (i < N && cross && col >= 0 && col < N) cpl[(size_t)blk * w * 32 + (j - 1) * 32 + t] = A(i, col);
            }
    }
}

// banded Cholesky S = U^T U, S rows [N][2kb+1] (real symmetric positive definite)
bool cholesky_band(int N, int kb, const double *S, std::vector<double> &U)
{
    U.assign((size_t)N * (kb + 1), 0.0);
    auto Sij = [&](int i, int j) { return S[(size_t)i * (2 * kb + 1) + kb + (j - i)]; };
    auto Uij = [&](int i, int j) -> double & { return U[(size_t)i * (kb + 1) + (j - i)]; };
    for (int j = 0; j < N; ++j) {
        for (int i = std::max(0, j - kb); i <= j; ++i) {
            double s = Sij(i, j);
            for (int q = std::max(0, j - kb); q < i; ++q) s -= Uij(q, i) * Uij(q, j);
            if (i == j) {
                if (!(s > 0.0)) return false;
                Uij(j, j) = std::sqrt(s);
            } else {
                Uij(i, j) = s / Uij(i, i);
            }
        }
    }
    return true;
}

// banded LU without pivoting of a complex band matrix A rows [N][2kb+1]: L unit lower, U upper
bool lu_band_nopivot(int N, int kb, std::vector<zd> &A)
{
    const int b = 2 * kb + 1;
    auto a = [&](int i, int j) -> zd & { return A[(size_t)i * b + kb + (j - i)]; };
    for (int k = 0; k < N; ++k) {
        const zd piv = a(k, k);
        if (std::abs(piv) == 0.0) return false;
        for (int i = k + 1; i <= std::min(N - 1, k + kb); ++i) {
            const zd l = a(i, k) / piv;
            a(i, k) = l;
            for (int j = k + 1; j <= std::min(N - 1, k + kb); ++j) a(i, j) -= l * a(k, j);
        }
    }
    return true;
}

template <typename T> struct dev_coef;
template <> struct dev_coef<double> { typedef double real_t; typedef cxd cplx_t; };
template <> struct dev_coef<float> { typedef float real_t; typedef cxf cplx_t; };

template <typename R>
int upload_real(const std::vector<zd> &v, void **dptr)
{
    std::vector<R> t(v.size());
    for (size_t k = 0; k < v.size(); ++k) t[k] = (R)v[k].real();
    PG_CUDA_TRY(cudaMalloc(dptr, std::max<size_t>(1, t.size()) * sizeof(R)));
    PG_CUDA_TRY(cudaMemcpy(*dptr, t.data(), t.size() * sizeof(R), cudaMemcpyHostToDevice));
    return PG_OK;
}
template <typename R>
int upload_real_d(const std::vector<double> &v, void **dptr)
{
    std::vector<R> t(v.begin(), v.end());
    PG_CUDA_TRY(cudaMalloc(dptr, std::max<size_t>(1, t.size()) * sizeof(R)));
    PG_CUDA_TRY(cudaMemcpy(*dptr, t.data(), t.size() * sizeof(R), cudaMemcpyHostToDevice));
    return PG_OK;
}
template <typename R>
int upload_cplx(const std::vector<zd> &v, void **dptr)
{
    std::vector<cx<R>> t(v.size());
    for (size_t k = 0; k < v.size(); ++k) t[k] = mk<R>((R)v[k].real(), (R)v[k].imag());
    PG_CUDA_TRY(cudaMalloc(dptr, std::max<size_t>(1, t.size()) * sizeof(cx<R>)));
    PG_CUDA_TRY(cudaMemcpy(*dptr, t.data(), t.size() * sizeof(cx<R>), cudaMemcpyHostToDevice));
    return PG_OK;
}

}  // namespace

struct pg_banded_ext : pg_banded {
    void *d_scratch = nullptr;
};

extern "C" int pg_overlap_create(pg_op *op, const double *overlap_rows, pg_banded **out)
{
    if (!op || !overlap_rows || !out) return PG_ERR_ARG;
    const int N = op->N, kb = op->kb;
    std::vector<double> U;
    if (!cholesky_band(N, kb, overlap_rows, U)) return PG_ERR_ARG;
    auto Ufun = [&](int i, int j) { return zd(U[(size_t)i * (kb + 1) + (j - i)], 0.0); };
    auto Lfun = [&](int i, int j) { return zd(U[(size_t)j * (kb + 1) + (i - j)], 0.0); };  // L = U^T
    std::vector<zd> up_inv, up_cpl, lo_inv, lo_cpl;
    build_blocks(N, kb, false, Ufun, up_inv, up_cpl);
    build_blocks(N, kb, true, Lfun, lo_inv, lo_cpl);
    pg_banded_ext *b = new pg_banded_ext();
    b->op = op;
    b->kind = 0;
    b->N = N;
    b->kb = kb;
    b->nmat = 1;
    b->complex_coef = 0;
    std::vector<double> Srows(overlap_rows, overlap_rows + (size_t)N * (2 * kb + 1));
    int st;
    if (op->precision == PG_FP64) {
        if ((st = upload_real_d<double>(U, &b->d_U)) != PG_OK) return st;
        if ((st = upload_real_d<double>(Srows, &b->d_S)) != PG_OK) return st;
        if ((st = upload_real<double>(up_inv, &b->d_up_inv)) != PG_OK) return st;
        if ((st = upload_real<double>(up_cpl, &b->d_up_cpl)) != PG_OK) return st;
        if ((st = upload_real<double>(lo_inv, &b->d_lo_inv)) != PG_OK) return st;
        if ((st = upload_real<double>(lo_cpl, &b->d_lo_cpl)) != PG_OK) return st;
    } else {
        if ((st = upload_real_d<float>(U, &b->d_U)) != PG_OK) return st;
        if ((st = upload_real_d<float>(Srows, &b->d_S)) != PG_OK) return st;
        if ((st = upload_real<float>(up_inv, &b->d_up_inv)) != PG_OK) return st;
        if ((st = upload_real<float>(up_cpl, &b->d_up_cpl)) != PG_OK) return st;
        if ((st = upload_real<float>(lo_inv, &b->d_lo_inv)) != PG_OK) return st;
        if ((st = upload_real<float>(lo_cpl, &b->d_lo_cpl)) != PG_OK) return st;
    }
    const size_t esz = op->precision == PG_FP64 ? sizeof(cxd) : sizeof(cxf);
    PG_CUDA_TRY(cudaMalloc(&b->d_scratch, esz * (size_t)op->nrows * N));
    *out = b;
    return PG_OK;
}

extern "C" int pg_prec_blockdiag_create(pg_op *op, const double *overlap_rows, const double *cS, const double *cH,
                                        const int *slots, const double *slot_weights, int nslots, pg_banded **out)
{
    if (!op || !overlap_rows || !cS || !cH || !out || nslots < 0 || (nslots > 0 && (!slots || !slot_weights)))
        return PG_ERR_ARG;
    if (!op->finalized) return PG_ERR_STATE;
    const int N = op->N, kb = op->kb, b = 2 * kb + 1, na = op->nrows;
    const zd zS(cS[0], cS[1]), zH(cH[0], cH[1]);
    std::vector<zd> all_lo_inv, all_lo_cpl, all_up_inv, all_up_cpl;
    for (int a = 0; a < na; ++a) {
        std::vector<zd> M((size_t)N * b, zd(0.0, 0.0));
        for (int i = 0; i < N; ++i)
            for (int d = 0; d < b; ++d) M[(size_t)i * b + d] = zS * overlap_rows[(size_t)i * b + d];
        for (int e = op->h_row_ptr[a]; e < op->h_row_ptr[a + 1]; ++e) {
            if (op->h_ent_col[e] != a) continue;
            zd wgt(0.0, 0.0);
            bool used = false;
            for (int q = 0; q < nslots; ++q)
                if (slots[q] == op->h_ent_slot[e]) {
                    wgt += zd(slot_weights[2 * q], slot_weights[2 * q + 1]);
                    used = true;
                }
            if (!used) continue;
            const zd *B = op->h_bands.data() + (size_t)op->h_ent_band[e] * b * N;
            for (int i = 0; i < N; ++i)
                for (int d = 0; d < b; ++d) M[(size_t)i * b + d] += zH * wgt * B[(size_t)d * N + i];
        }
        if (!lu_band_nopivot(N, kb, M)) return PG_ERR_ARG;
        auto Lf = [&](int i, int j) { return i == j ? zd(1.0, 0.0) : M[(size_t)i * b + kb + (j - i)]; };
        auto Uf = [&](int i, int j) { return M[(size_t)i * b + kb + (j - i)]; };
        std::vector<zd> li, lc, ui, uc;
        build_blocks(N, kb, true, Lf, li, lc);
        build_blocks(N, kb, false, Uf, ui, uc);
        all_lo_inv.insert(all_lo_inv.end(), li.begin(), li.end());
        all_lo_cpl.insert(all_lo_cpl.end(), lc.begin(), lc.end());
        all_up_inv.insert(all_up_inv.end(), ui.begin(), ui.end());
        all_up_cpl.insert(all_up_cpl.end(), uc.begin(), uc.end());
    }
    pg_banded_ext *bd = new pg_banded_ext();
    bd->op = op;
    bd->kind = 1;
    bd->N = N;
    bd->kb = kb;
    bd->nmat = na;
    bd->complex_coef = 1;
    int st;
    if (op->precision == PG_FP64) {
        if ((st = upload_cplx<double>(all_lo_inv, &bd->d_lo_inv)) != PG_OK) return st;
        if ((st = upload_cplx<double>(all_lo_cpl, &bd->d_lo_cpl)) != PG_OK) return st;
        if ((st = upload_cplx<double>(all_up_inv, &bd->d_up_inv)) != PG_OK) return st;
        if ((st = upload_cplx<double>(all_up_cpl, &bd->d_up_cpl)) != PG_OK) return st;
    } else {
        if ((st = upload_cplx<float>(all_lo_inv, &bd->d_lo_inv)) != PG_OK) return st;
        if ((st = upload_cplx<float>(all_lo_cpl, &bd->d_lo_cpl)) != PG_OK) return st;
        if ((st = upload_cplx<float>(all_up_inv, &bd->d_up_inv)) != PG_OK) return st;
        if ((st = upload_cplx<float>(all_up_cpl, &bd->d_up_cpl)) != PG_OK) return st;
    }
    *out = bd;
    return PG_OK;
}

extern "C" int pg_banded_destroy(pg_banded *b)
{
    if (!b) return PG_ERR_ARG;
    pg_banded_ext *e = static_cast<pg_banded_ext *>(b);
    cudaFree(e->d_U);
    cudaFree(e->d_S);
    cudaFree(e->d_lo_inv);
    cudaFree(e->d_lo_cpl);
    cudaFree(e->d_up_inv);
    cudaFree(e->d_up_cpl);
    cudaFree(e->d_scratch);
    delete e;
    return PG_OK;
}

template <typename R, typename C>
static int launch_tri(pg_banded *b, bool lower, void *x)
{
    pg_ctx *ctx = b->op->ctx;
    const int N = b->N, nblk = (N + 31) / 32, w = b->kb;
    const int nfib = b->op->nrows;
    if (w > 32 || (w * 32 * sizeof(C)) % 16 != 0) return PG_ERR_ARG;
    // FP64 spreads each block product over 4 warps, FP32 keeps one warp per fibre
    constexpr int NW = sizeof(R) == 8 ? 4 : 1;
    const size_t smem = (size_t)TRI_STAGES * (1024 + w * 32) * sizeof(C) + (size_t)(NW + 1) * 32 * sizeof(cx<R>);
    static bool configured[2][2] = {{false, false}, {false, false}};
    bool &cfg = configured[lower ? 1 : 0][sizeof(C) == sizeof(R) ? 0 : 1];
    if (!cfg) {
        PG_CUDA_TRY(cudaFuncSetAttribute(tri_solve_kernel<R, C, true, NW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem + 4096));
        PG_CUDA_TRY(cudaFuncSetAttribute(tri_solve_kernel<R, C, false, NW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem + 4096));
        cfg = true;
    }
    if (lower)
        tri_solve_kernel<R, C, true, NW><<<nfib, 32 * NW, smem, ctx->stream>>>(
            N, nblk, w, (const C *)b->d_lo_inv, (const C *)b->d_lo_cpl, b->nmat > 1, (cx<R> *)x, nfib);
    else
        tri_solve_kernel<R, C, false, NW><<<nfib, 32 * NW, smem, ctx->stream>>>(
            N, nblk, w, (const C *)b->d_up_inv, (const C *)b->d_up_cpl, b->nmat > 1, (cx<R> *)x, nfib);
    ctx->launches++;
    return pg_check_launch(ctx);
}

template <typename R>
static int banded_apply_t(pg_banded *bb, int which, void *x)
{
    pg_banded_ext *b = static_cast<pg_banded_ext *>(bb);
    pg_ctx *ctx = b->op->ctx;
    const int N = b->N, kb = b->kb, nfib = b->op->nrows;
    const size_t bytes = sizeof(cx<R>) * (size_t)nfib * N;
    dim3 grid((N + 127) / 128, nfib);
    switch (which) {
    case PG_BAND_MUL_U:
    case PG_BAND_MUL_UT:
        if (b->kind != 0) return PG_ERR_STATE;
        tri_mul_kernel<R><<<grid, 128, 0, ctx->stream>>>(N, kb, (const R *)b->d_U, (const cx<R> *)x,
                                                        (cx<R> *)b->d_scratch, which == PG_BAND_MUL_U);
        ctx->launches++;
        PG_TRY(pg_check_launch(ctx));
        PG_CUDA_TRY(cudaMemcpyAsync(x, b->d_scratch, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
        return PG_OK;
    case PG_BAND_MUL_S:
        if (b->kind != 0) return PG_ERR_STATE;
        band_mul_kernel<R><<<grid, 128, 0, ctx->stream>>>(N, kb, (const R *)b->d_S, (const cx<R> *)x,
                                                         (cx<R> *)b->d_scratch);
        ctx->launches++;
        PG_TRY(pg_check_launch(ctx));
        PG_CUDA_TRY(cudaMemcpyAsync(x, b->d_scratch, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
        return PG_OK;
    case PG_BAND_SOLVE_U:
        if (b->kind != 0) return PG_ERR_STATE;
        return launch_tri<R, R>(b, false, x);
    case PG_BAND_SOLVE_UT:
        if (b->kind != 0) return PG_ERR_STATE;
        return launch_tri<R, R>(b, true, x);
    case PG_BAND_SOLVE_S:
        if (b->kind != 0) return PG_ERR_STATE;
        PG_TRY(launch_tri<R, R>(b, true, x));
        return launch_tri<R, R>(b, false, x);
    case PG_BAND_PREC_SOLVE:
        if (b->kind != 1) return PG_ERR_STATE;
        PG_TRY((launch_tri<R, cx<R>>(b, true, x)));
        return launch_tri<R, cx<R>>(b, false, x);
    default:
        return PG_ERR_ARG;
    }
}

int pg_banded_apply_dev(pg_banded *b, int which, void *x)
{
    if (!b || !x) return PG_ERR_ARG;
    if (b->op->precision == PG_FP64) return banded_apply_t<double>(b, which, x);
    return banded_apply_t<float>(b, which, x);
}

extern "C" int pg_banded_apply(pg_banded *b, int which, void *x) { return pg_banded_apply_dev(b, which, x); }
