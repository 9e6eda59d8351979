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
// Triangular solves: one CTA per fibre, 32-row blocks. The diagonal-block products of all
// blocks run in parallel; the only sequential part is a recurrence on the kb boundary values
// of consecutive blocks (tri_solve_kernel).
#include "pg_internal.cuh"
#include "tri_solve.cuh"

#include <algorithm>
#include <cmath>

typedef std::complex<double> zd;

// ------------------------------------------------------------------------------------
// kernels
// ------------------------------------------------------------------------------------
// One CTA of NW warps per fibre (tri_solve_smem in tri_solve.cuh holds the method): load the
// fibre into shared memory, run both sweeps, store it back.
template <typename R, typename C, int NW>
__global__ void __launch_bounds__(32 * NW, 1)
    tri_solve_kernel(int N, int nblk, int w, const C *__restrict__ lo_inv, const C *__restrict__ lo_g,
                     const C *__restrict__ lo_rb, const C *__restrict__ up_inv, const C *__restrict__ up_g,
                     const C *__restrict__ up_rb, int do_lower, int do_upper, int fib_per_mat, int g_in_smem,
                     cx<R> *__restrict__ x, int nfib)
{
    extern __shared__ __align__(16) unsigned char tri_smem[];
    const int f = blockIdx.x;
    if (f >= nfib) return;
    cx<R> *xs = (cx<R> *)tri_smem;              // [nblk*32] the fibre: f, then z, then y
    cx<R> *sb = xs + (size_t)nblk * 32;          // [nblk*w] boundary values s_b
    C *sg = (C *)(sb + (size_t)nblk * w);        // [nblk][w][32] G_b (when g_in_smem)
    const size_t m = (size_t)(f / fib_per_mat);
    cx<R> *xf = x + (size_t)f * N;
    for (int i = threadIdx.x; i < nblk * 32; i += 32 * NW) xs[i] = (i < N) ? xf[i] : mk<R>((R)0, (R)0);
    __syncthreads();
    tri_solve_smem<R, C, NW>(nblk, w, m, lo_inv, lo_g, lo_rb, up_inv, up_g, up_rb, do_lower, do_upper, g_in_smem, xs,
                             sb, sg);
    for (int i = threadIdx.x; i < N; i += 32 * NW) xf[i] = xs[i];
}

// U x (up=1) or U^T x (up=0), U real upper with kb super diagonals, rows [N][kb+1]
template <typename R>
__global__ void tri_mul_kernel(int nfib, int N, int kb, const R *__restrict__ U, const cx<R> *__restrict__ x,
                               cx<R> *__restrict__ y, int up)
{
    const int f = pg_grid_row();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N || f >= nfib) return;
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
__global__ void band_mul_kernel(int nfib, int N, int kb, const R *__restrict__ S, const cx<R> *__restrict__ x,
                                cx<R> *__restrict__ y)
{
    const int f = pg_grid_row();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N || f >= nfib) return;
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

// Build block data for a triangular matrix given by accessor A(i, j) (band width w):
// inv[blk][s][t] = T^-1[t][s] for the diagonal block T, and g[blk][c][t] = (T^-1 C)[t][c] for
// the coupling C[t][c] = A(32 blk + t, col_c) to the neighbouring block's boundary columns
// col_c = 32 blk - w + c (lower) or 32 (blk + 1) + c (upper), c < w.
template <typename Acc>
void build_blocks(int N, int w, bool lower, Acc A, std::vector<zd> &inv, std::vector<zd> &g, std::vector<zd> &rb)
{
    const int nblk = (N + 31) / 32;
    inv.assign((size_t)nblk * 1024, zd(0.0, 0.0));
    g.assign((size_t)nblk * w * 32, zd(0.0, 0.0));
    std::vector<zd> T(1024), Ti(1024), Cm((size_t)32 * w);
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
        for (int t = 0; t < 32; ++t)
            for (int c = 0; c < w; ++c) {
                const int i = r0 + t;
                const int col = lower ? r0 - w + c : r0 + 32 + c;
                zd v(0.0, 0.0);
                if (i < N && col >= 0 && col < N && std::abs(i - col) <= w) v = A(i, col);
                Cm[(size_t)t * w + c] = v;
            }
        for (int t = 0; t < 32; ++t)
            for (int c = 0; c < w; ++c) {
                zd acc(0.0, 0.0);
                for (int s = 0; s < 32; ++s) acc += Ti[t * 32 + s] * Cm[(size_t)s * w + c];
                g[(size_t)blk * w * 32 + (size_t)c * 32 + t] = acc;
            }
    }
    // Boundary system s_b + T_b s_{b-/+1} = z_b[boundary rows], T_b = G_b[boundary rows]
    // (lower: rows 32-w.., coupling to block b-1; upper: rows 0.., coupling to block b+1).
    // rb = its inverse, [nb][nb] row-major, by substitution on the unit vectors.
    const int nb = nblk * w, r0 = lower ? 32 - w : 0;
    rb.assign((size_t)nb * nb, zd(0.0, 0.0));
    std::vector<zd> sv(nb);
    for (int j = 0; j < nb; ++j) {
        std::fill(sv.begin(), sv.end(), zd(0.0, 0.0));
        sv[j] = zd(1.0, 0.0);
        for (int step = 1; step < nblk; ++step) {
            const int bk = lower ? step : nblk - 1 - step, prev = lower ? bk - 1 : bk + 1;
            for (int r = 0; r < w; ++r) {
                zd acc = sv[bk * w + r];
                for (int c = 0; c < w; ++c) acc -= g[(size_t)bk * w * 32 + (size_t)c * 32 + r0 + r] * sv[prev * w + c];
                sv[bk * w + r] = acc;
            }
        }
        for (int i = 0; i < nb; ++i) rb[(size_t)i * nb + j] = sv[i];
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
    void *d_swap = nullptr;  // two-electron operators: the wavefunction with its radial ranks swapped
};

extern "C" int pg_overlap_create(pg_op *op, const double *overlap_rows, pg_banded **out)
{
    if (!op || !overlap_rows || !out) return PG_ERR_ARG;
    const int N = op->N, kb = op->kb;
    std::vector<double> U;
    if (!cholesky_band(N, kb, overlap_rows, U)) return PG_ERR_ARG;
    auto Ufun = [&](int i, int j) { return zd(U[(size_t)i * (kb + 1) + (j - i)], 0.0); };
    auto Lfun = [&](int i, int j) { return zd(U[(size_t)j * (kb + 1) + (i - j)], 0.0); };  // L = U^T
    std::vector<zd> up_inv, up_cpl, up_rb, lo_inv, lo_cpl, lo_rb;
    build_blocks(N, kb, false, Ufun, up_inv, up_cpl, up_rb);
    build_blocks(N, kb, true, Lfun, lo_inv, lo_cpl, lo_rb);
    pg_banded_ext *b = new pg_banded_ext();
    b->op = op;
    b->kind = 0;
    b->N = N;
    b->kb = kb;
    b->nmat = 1;
    b->fib_per_mat = std::max(1, op->nrows);  // one factor for every fibre
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
        if ((st = upload_real<double>(up_rb, &b->d_up_rb)) != PG_OK) return st;
        if ((st = upload_real<double>(lo_rb, &b->d_lo_rb)) != PG_OK) return st;
    } else {
        if ((st = upload_real_d<float>(U, &b->d_U)) != PG_OK) return st;
        if ((st = upload_real_d<float>(Srows, &b->d_S)) != PG_OK) return st;
        if ((st = upload_real<float>(up_inv, &b->d_up_inv)) != PG_OK) return st;
        if ((st = upload_real<float>(up_cpl, &b->d_up_cpl)) != PG_OK) return st;
        if ((st = upload_real<float>(lo_inv, &b->d_lo_inv)) != PG_OK) return st;
        if ((st = upload_real<float>(lo_cpl, &b->d_lo_cpl)) != PG_OK) return st;
        if ((st = upload_real<float>(up_rb, &b->d_up_rb)) != PG_OK) return st;
        if ((st = upload_real<float>(lo_rb, &b->d_lo_rb)) != PG_OK) return st;
    }
    const size_t esz = op->precision == PG_FP64 ? sizeof(cxd) : sizeof(cxf);
    PG_CUDA_TRY(cudaMalloc(&b->d_scratch, esz * (size_t)op->nrows * N));
    if (op->rank == 3) {
        if (op->shape[1] != N) return PG_ERR_SHAPE;  // both radial ranks share the B-spline basis
        PG_CUDA_TRY(cudaMalloc(&b->d_swap, esz * (size_t)op->nrows * N));
    }
    *out = b;
    return PG_OK;
}

extern "C" int pg_prec_blockdiag_create(pg_op *op, const double *overlap_rows, const double *cS, const double *cH,
                                        const int *slots, const double *slot_weights, int nslots, pg_banded **out)
{
    if (!op || !overlap_rows || !cS || !cH || !out || nslots < 0 || (nslots > 0 && (!slots || !slot_weights)))
        return PG_ERR_ARG;
    if (!op->finalized) return PG_ERR_STATE;
    if (op->rank != 2) return PG_ERR_STORAGE;  // blocks are angular channels of a rank-2 operator
    const int N = op->N, kb = op->kb, b = 2 * kb + 1, na = op->nrows;
    const zd zS(cS[0], cS[1]), zH(cH[0], cH[1]);
    std::vector<zd> all_lo_inv, all_lo_cpl, all_up_inv, all_up_cpl, all_lo_rb, all_up_rb;
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
        std::vector<zd> li, lc, lr, ui, uc, ur;
        build_blocks(N, kb, true, Lf, li, lc, lr);
        build_blocks(N, kb, false, Uf, ui, uc, ur);
        all_lo_rb.insert(all_lo_rb.end(), lr.begin(), lr.end());
        all_up_rb.insert(all_up_rb.end(), ur.begin(), ur.end());
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
        if ((st = upload_cplx<double>(all_lo_rb, &bd->d_lo_rb)) != PG_OK) return st;
        if ((st = upload_cplx<double>(all_up_rb, &bd->d_up_rb)) != PG_OK) return st;
    } else {
        if ((st = upload_cplx<float>(all_lo_inv, &bd->d_lo_inv)) != PG_OK) return st;
        if ((st = upload_cplx<float>(all_lo_cpl, &bd->d_lo_cpl)) != PG_OK) return st;
        if ((st = upload_cplx<float>(all_up_inv, &bd->d_up_inv)) != PG_OK) return st;
        if ((st = upload_cplx<float>(all_up_cpl, &bd->d_up_cpl)) != PG_OK) return st;
        if ((st = upload_cplx<float>(all_lo_rb, &bd->d_lo_rb)) != PG_OK) return st;
        if ((st = upload_cplx<float>(all_up_rb, &bd->d_up_rb)) != PG_OK) return st;
    }
    *out = bd;
    return PG_OK;
}

// Factor one complex band matrix A = cS S + cH h (rows [N][2kb+1]) and append its block data.
static int factor_append(int N, int kb, const double *S, const zd &zS, const zd &zH, const double *h,
                         std::vector<zd> *lo, std::vector<zd> *up)
{
    const int b = 2 * kb + 1;
    std::vector<zd> M((size_t)N * b);
    for (size_t q = 0; q < (size_t)N * b; ++q) M[q] = zS * S[q] + zH * zd(h[2 * q], h[2 * q + 1]);
    if (!lu_band_nopivot(N, kb, M)) return PG_ERR_ARG;
    auto Lf = [&](int i, int j) { return i == j ? zd(1.0, 0.0) : M[(size_t)i * b + kb + (j - i)]; };
    auto Uf = [&](int i, int j) { return M[(size_t)i * b + kb + (j - i)]; };
    std::vector<zd> li, lc, lr, ui, uc, ur;
    build_blocks(N, kb, true, Lf, li, lc, lr);
    build_blocks(N, kb, false, Uf, ui, uc, ur);
    lo[0].insert(lo[0].end(), li.begin(), li.end());
    lo[1].insert(lo[1].end(), lc.begin(), lc.end());
    lo[2].insert(lo[2].end(), lr.begin(), lr.end());
    up[0].insert(up[0].end(), ui.begin(), ui.end());
    up[1].insert(up[1].end(), uc.begin(), uc.end());
    up[2].insert(up[2].end(), ur.begin(), ur.end());
    return PG_OK;
}

template <typename R>
static int upload_sets(pg_banded_ext *bd, std::vector<zd> *lo, std::vector<zd> *up, std::vector<zd> *lo1,
                       std::vector<zd> *up1)
{
    PG_TRY(upload_cplx<R>(lo[0], &bd->d_lo_inv));
    PG_TRY(upload_cplx<R>(lo[1], &bd->d_lo_cpl));
    PG_TRY(upload_cplx<R>(lo[2], &bd->d_lo_rb));
    PG_TRY(upload_cplx<R>(up[0], &bd->d_up_inv));
    PG_TRY(upload_cplx<R>(up[1], &bd->d_up_cpl));
    PG_TRY(upload_cplx<R>(up[2], &bd->d_up_rb));
    PG_TRY(upload_cplx<R>(lo1[0], &bd->d_lo_inv1));
    PG_TRY(upload_cplx<R>(lo1[1], &bd->d_lo_cpl1));
    PG_TRY(upload_cplx<R>(lo1[2], &bd->d_lo_rb1));
    PG_TRY(upload_cplx<R>(up1[0], &bd->d_up_inv1));
    PG_TRY(upload_cplx<R>(up1[1], &bd->d_up_cpl1));
    return upload_cplx<R>(up1[2], &bd->d_up_rb1);
}

// Two-electron radial preconditioner, Kronecker-factorized per angular channel a:
//     M_a = (cS S + cH h1_a) x (cS S + cH h2_a)  ~  cS^2 S x S + cS cH (h1_a x S + S x h2_a),
// h1_a, h2_a the one-electron radial Hamiltonians of the channel's two electrons (host
// complex128 rows [nchan][N][2kb+1]). It stands in for the reference's sparse direct / ILU
// block preconditioners (examples/tensor/helium_stabilization/preconditioner.py:77-244):
// it leaves out the electron-electron repulsion of the block and adds the small
// cH^2 h1 x h2, and its inverse is two banded block solves, one along each radial rank.
extern "C" int pg_prec_kron_create(pg_op *op, const double *overlap_rows, const double *cS, const double *cH,
                                   const double *h1, const double *h2, pg_banded **out)
{
    if (!op || !overlap_rows || !cS || !cH || !h1 || !h2 || !out) return PG_ERR_ARG;
    if (!op->finalized) return PG_ERR_STATE;
    if (op->rank != 3 || op->shape[1] != op->N) return PG_ERR_STORAGE;
    const int N = op->N, kb = op->kb, b = 2 * kb + 1, nchan = op->shape[0];
    const zd zS(cS[0], cS[1]), zH(cH[0], cH[1]);
    std::vector<zd> lo2[3], up2[3], lo1[3], up1[3];
    const size_t per = (size_t)N * b * 2;  // doubles per channel
    for (int a = 0; a < nchan; ++a) {
        PG_TRY(factor_append(N, kb, overlap_rows, zS, zH, h2 + a * per, lo2, up2));
        PG_TRY(factor_append(N, kb, overlap_rows, zS, zH, h1 + a * per, lo1, up1));
    }
    pg_banded_ext *bd = new pg_banded_ext();
    bd->op = op;
    bd->kind = 2;
    bd->N = N;
    bd->kb = kb;
    bd->nmat = nchan;
    bd->complex_coef = 1;
    bd->fib_per_mat = op->shape[1];   // fibres (a, i1): channel a = f / N1
    bd->fib_per_mat1 = op->shape[2];  // swapped fibres (a, i2): channel a = f / N2
    const size_t esz = op->precision == PG_FP64 ? sizeof(cxd) : sizeof(cxf);
    PG_CUDA_TRY(cudaMalloc(&bd->d_swap, esz * (size_t)op->nrows * N));
    if (op->precision == PG_FP64) PG_TRY(upload_sets<double>(bd, lo2, up2, lo1, up1));
    else PG_TRY(upload_sets<float>(bd, lo2, up2, lo1, up1));
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
    cudaFree(e->d_lo_rb);
    cudaFree(e->d_up_rb);
    for (void *p : {e->d_lo_inv1, e->d_lo_cpl1, e->d_lo_rb1, e->d_up_inv1, e->d_up_cpl1, e->d_up_rb1}) cudaFree(p);
    cudaFree(e->d_scratch);
    cudaFree(e->d_swap);
    cudaFree(e->d_fdV);
    cudaFree(e->d_fdD);
    cudaFree(e->d_fdl);
    cudaFree(e->d_fdP0);
    cudaFree(e->d_fdP1);
    delete e;
    return PG_OK;
}

// One CTA of NW warps per fibre; NW covers the blocks of a fibre (one block per warp where
// possible), bounded by the registers of the unrolled block product.
// One factor set of a blocked triangular solve (the device arrays of build_blocks).
struct TriSet {
    const void *lo_inv, *lo_cpl, *lo_rb, *up_inv, *up_cpl, *up_rb;
    int fib_per_mat;
};

static TriSet tri_set(const pg_banded *b, bool first_rank)
{
    if (first_rank) return {b->d_lo_inv1, b->d_lo_cpl1, b->d_lo_rb1, b->d_up_inv1, b->d_up_cpl1, b->d_up_rb1, b->fib_per_mat1};
    return {b->d_lo_inv, b->d_lo_cpl, b->d_lo_rb, b->d_up_inv, b->d_up_cpl, b->d_up_rb, b->fib_per_mat};
}

// One CTA of NW warps per fibre; NW covers the blocks of a fibre (one block per warp where
// possible), bounded by the registers of the unrolled block product.
template <typename R, typename C, int NW>
static int launch_tri_nw(pg_banded *b, const TriSet &ts, bool do_lower, bool do_upper, void *x)
{
    pg_ctx *ctx = b->op->ctx;
    const int N = b->N, nblk = (N + 31) / 32, w = b->kb;
    const int nfib = b->op->nrows;
    const size_t base = (size_t)nblk * 32 * sizeof(cx<R>) + (size_t)nblk * w * sizeof(cx<R>);
    const size_t full = base + (size_t)nblk * w * 32 * sizeof(C);
    const size_t limit = 200 * 1024;
    if (base > limit) return PG_ERR_SHAPE;  // fibre too long for the shared-memory solve
    const bool g_in_smem = full <= limit;
    const size_t smem = g_in_smem ? full : base;
    static size_t configured = 0;
    if (configured < smem) {
        PG_CUDA_TRY(cudaFuncSetAttribute(tri_solve_kernel<R, C, NW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem));
        configured = smem;
    }
    tri_solve_kernel<R, C, NW><<<nfib, 32 * NW, smem, ctx->stream>>>(
        N, nblk, w, (const C *)ts.lo_inv, (const C *)ts.lo_cpl, (const C *)ts.lo_rb, (const C *)ts.up_inv,
        (const C *)ts.up_cpl, (const C *)ts.up_rb, do_lower ? 1 : 0, do_upper ? 1 : 0, std::max(1, ts.fib_per_mat),
        g_in_smem ? 1 : 0, (cx<R> *)x, nfib);
    ctx->launches++;
    return pg_check_launch(ctx);
}

template <typename R, typename C>
static int launch_tri(pg_banded *b, bool do_lower, bool do_upper, void *x, bool first_rank = false)
{
    const int nblk = (b->N + 31) / 32;
    if (b->kb < 1 || b->kb > 32) return PG_ERR_ARG;
    const TriSet ts = tri_set(b, first_rank);
    if (nblk <= 8) return launch_tri_nw<R, C, 8>(b, ts, do_lower, do_upper, x);
    // FP64 stays at 16 warps (register budget of the complex128 block product)
    if constexpr (sizeof(R) == 8) {
        return launch_tri_nw<R, C, 16>(b, ts, do_lower, do_upper, x);
    } else {
        if (nblk <= 16) return launch_tri_nw<R, C, 16>(b, ts, do_lower, do_upper, x);
        return launch_tri_nw<R, C, 24>(b, ts, do_lower, do_upper, x);
    }
}

template <typename R>
static int banded_apply_t(pg_banded *bb, int which, void *x)
{
    pg_banded_ext *b = static_cast<pg_banded_ext *>(bb);
    pg_ctx *ctx = b->op->ctx;
    const int N = b->N, kb = b->kb, nfib = b->op->nrows;
    const size_t bytes = sizeof(cx<R>) * (size_t)nfib * N;
    const dim3 grid = pg_row_grid((N + 127) / 128, nfib);
    switch (which) {
    case PG_BAND_MUL_U:
    case PG_BAND_MUL_UT:
        if (b->kind != 0) return PG_ERR_STATE;
        tri_mul_kernel<R><<<grid, 128, 0, ctx->stream>>>(nfib, N, kb, (const R *)b->d_U, (const cx<R> *)x,
                                                        (cx<R> *)b->d_scratch, which == PG_BAND_MUL_U);
        ctx->launches++;
        PG_TRY(pg_check_launch(ctx));
        PG_CUDA_TRY(cudaMemcpyAsync(x, b->d_scratch, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
        return PG_OK;
    case PG_BAND_MUL_S:
        if (b->kind != 0) return PG_ERR_STATE;
        band_mul_kernel<R><<<grid, 128, 0, ctx->stream>>>(nfib, N, kb, (const R *)b->d_S, (const cx<R> *)x,
                                                         (cx<R> *)b->d_scratch);
        ctx->launches++;
        PG_TRY(pg_check_launch(ctx));
        PG_CUDA_TRY(cudaMemcpyAsync(x, b->d_scratch, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
        return PG_OK;
    case PG_BAND_SOLVE_U:
        if (b->kind != 0) return PG_ERR_STATE;
        return launch_tri<R, R>(b, false, true, x);
    case PG_BAND_SOLVE_UT:
        if (b->kind != 0) return PG_ERR_STATE;
        return launch_tri<R, R>(b, true, false, x);
    case PG_BAND_SOLVE_S:
        if (b->kind != 0) return PG_ERR_STATE;
        return launch_tri<R, R>(b, true, true, x);
    case PG_BAND_PREC_SOLVE:
        if (b->kind == 1) return launch_tri<R, cx<R>>(b, true, true, x);
        if (b->kind == 3) return pg_fd_apply_dev(b, x);
        if (b->kind == 2) {
            // (A1 x A2)^-1 = (A1^-1 x 1)(1 x A2^-1): the second electron's rank as fibres, then
            // the first electron's rank on the swapped copy
            const int n0 = b->op->shape[0], n1 = b->op->shape[1], n2 = b->op->shape[2];
            PG_TRY((launch_tri<R, cx<R>>(b, true, true, x)));
            PG_TRY(pg_swap_last2_dev(ctx, b->op->precision, x, b->d_swap, n0, n1, n2));
            PG_TRY((launch_tri<R, cx<R>>(b, true, true, b->d_swap, true)));
            return pg_swap_last2_dev(ctx, b->op->precision, b->d_swap, x, n0, n2, n1);
        }
        return PG_ERR_STATE;
    default:
        return PG_ERR_ARG;
    }
}

static int banded_apply_fibres(pg_banded *b, int which, void *x)
{
    if (b->op->precision == PG_FP64) return banded_apply_t<double>(b, which, x);
    return banded_apply_t<float>(b, which, x);
}

// Overlap operations act on every B-spline rank: for a two-electron operator [Nang][N][N]
// the last rank as fibres, then the middle rank on the copy with the two radial ranks swapped
// (S x S = (S x 1)(1 x S); the same for the factors U).
int pg_banded_apply_dev(pg_banded *b, int which, void *x)
{
    if (!b || !x) return PG_ERR_ARG;
    PG_TRY(banded_apply_fibres(b, which, x));
    if (b->kind != 0 || b->op->rank != 3) return PG_OK;
    pg_banded_ext *e = static_cast<pg_banded_ext *>(b);
    const int n0 = b->op->shape[0], n1 = b->op->shape[1], n2 = b->op->shape[2];
    PG_TRY(pg_swap_last2_dev(b->op->ctx, b->op->precision, x, e->d_swap, n0, n1, n2));
    PG_TRY(banded_apply_fibres(b, which, e->d_swap));
    return pg_swap_last2_dev(b->op->ctx, b->op->precision, e->d_swap, x, n0, n2, n1);
}

extern "C" int pg_banded_apply(pg_banded *b, int which, void *x) { return pg_banded_apply_dev(b, which, x); }

int pg_banded_solve_kernels(const pg_banded *b) { return b->kind == 2 ? 4 : b->kind == 3 ? pg_fd_kernels(b) : 1; }

// Two-electron preconditioner by fast diagonalization (fdprec.cu): per channel a the exact
// inverse of cS S x S + cH (h_l1 x S + S x h_l2) from the generalized eigenvectors
// V_l (h_l V = S V Lambda, V^T S V = 1) of the one-electron Hamiltonians.
extern "C" int pg_prec_fd_create(pg_op *op, int nl, const double *V, const double *lam, const int *lidx,
                                 const double *cS, const double *cH, pg_banded **out)
{
    if (!op || nl < 1 || !V || !lam || !lidx || !cS || !cH || !out) return PG_ERR_ARG;
    if (!op->finalized) return PG_ERR_STATE;
    if (op->rank != 3 || op->shape[1] != op->shape[2]) return PG_ERR_STORAGE;
    const int A = op->shape[0], N = op->shape[1];
    const int NP0 = (N + 3) & ~3;
    for (int a = 0; a < 2 * A; ++a)
        if (lidx[a] < 0 || lidx[a] >= nl) return PG_ERR_ARG;
    // the shared-memory kernel when the channel block fits, batched GEMMs otherwise
    const bool global = pg_fd_prepare(op->precision, NP0) != PG_OK;
    const int NP = global ? N : NP0;
    const zd zS(cS[0], cS[1]), zH(cH[0], cH[1]);
    std::vector<double> Vp((size_t)nl * NP * NP, 0.0);
    for (int l = 0; l < nl; ++l)
        for (int k = 0; k < N; ++k)
            for (int i = 0; i < N; ++i) Vp[((size_t)l * NP + k) * NP + i] = V[((size_t)l * N + k) * N + i];
    std::vector<zd> D((size_t)A * N * N);
    for (int a = 0; a < A; ++a) {
        const double *L1 = lam + (size_t)lidx[2 * a] * N, *L2 = lam + (size_t)lidx[2 * a + 1] * N;
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j) D[((size_t)a * N + i) * N + j] = 1.0 / (zS + zH * (L1[i] + L2[j]));
    }
    pg_banded_ext *bd = new pg_banded_ext();
    bd->op = op;
    bd->kind = 3;
    bd->N = N;
    bd->kb = op->kb;
    bd->nmat = A;
    bd->complex_coef = 1;
    bd->fdN = N;
    bd->fdNP = NP;
    bd->fdGlobal = global ? 1 : 0;
    if (global) {
        const size_t bytes = (op->precision == PG_FP64 ? sizeof(double) : sizeof(float)) * 2 * (size_t)A * N * N;
        PG_CUDA_TRY(cudaMalloc(&bd->d_fdP0, bytes));
        PG_CUDA_TRY(cudaMalloc(&bd->d_fdP1, bytes));
    }
    PG_CUDA_TRY(cudaMalloc(&bd->d_fdl, sizeof(int) * 2 * A));
    PG_CUDA_TRY(cudaMemcpy(bd->d_fdl, lidx, sizeof(int) * 2 * A, cudaMemcpyHostToDevice));
    if (op->precision == PG_FP64) {
        PG_CUDA_TRY(cudaMalloc(&bd->d_fdV, sizeof(double) * Vp.size()));
        PG_CUDA_TRY(cudaMemcpy(bd->d_fdV, Vp.data(), sizeof(double) * Vp.size(), cudaMemcpyHostToDevice));
        std::vector<cxd> Dd(D.size());
        for (size_t t = 0; t < D.size(); ++t) Dd[t] = mk<double>(D[t].real(), D[t].imag());
        PG_CUDA_TRY(cudaMalloc(&bd->d_fdD, sizeof(cxd) * Dd.size()));
        PG_CUDA_TRY(cudaMemcpy(bd->d_fdD, Dd.data(), sizeof(cxd) * Dd.size(), cudaMemcpyHostToDevice));
    } else {
        std::vector<float> Vf(Vp.begin(), Vp.end());
        PG_CUDA_TRY(cudaMalloc(&bd->d_fdV, sizeof(float) * Vf.size()));
        PG_CUDA_TRY(cudaMemcpy(bd->d_fdV, Vf.data(), sizeof(float) * Vf.size(), cudaMemcpyHostToDevice));
        std::vector<cxf> Df(D.size());
        for (size_t t = 0; t < D.size(); ++t) Df[t] = mk<float>((float)D[t].real(), (float)D[t].imag());
        PG_CUDA_TRY(cudaMalloc(&bd->d_fdD, sizeof(cxf) * Df.size()));
        PG_CUDA_TRY(cudaMemcpy(bd->d_fdD, Df.data(), sizeof(cxf) * Df.size(), cudaMemcpyHostToDevice));
    }
    *out = bd;
    return PG_OK;
}

extern "C" int pg_prec_fd_max_n(int precision) { return pg_fd_max_n(precision); }
