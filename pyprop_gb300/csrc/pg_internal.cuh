// Internal definitions shared by the libpyprop_gpu translation units.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <vector>
#include <complex>
#include <string>

#include "../../include/pyprop_gpu.h"

// ------------------------------------------------------------------------------------
// complex arithmetic on interleaved pairs
// ------------------------------------------------------------------------------------
template <typename R> struct __align__(2 * sizeof(R)) cx {
    R x, y;
};
typedef cx<double> cxd;
typedef cx<float> cxf;

template <typename R> __host__ __device__ __forceinline__ cx<R> mk(R a, R b) { cx<R> c; c.x = a; c.y = b; return c; }
template <typename R> __host__ __device__ __forceinline__ cx<R> operator+(cx<R> a, cx<R> b) { return mk<R>(a.x + b.x, a.y + b.y); }
template <typename R> __host__ __device__ __forceinline__ cx<R> operator-(cx<R> a, cx<R> b) { return mk<R>(a.x - b.x, a.y - b.y); }
template <typename R> __host__ __device__ __forceinline__ cx<R> operator*(cx<R> a, cx<R> b) {
    return mk<R>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename R> __host__ __device__ __forceinline__ cx<R> operator*(R s, cx<R> a) { return mk<R>(s * a.x, s * a.y); }
template <typename R> __host__ __device__ __forceinline__ cx<R> conjx(cx<R> a) { return mk<R>(a.x, -a.y); }
// acc += a * b
template <typename R> __device__ __forceinline__ void cfma(cx<R> &acc, cx<R> a, cx<R> b) {
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(-a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(a.y, b.x, acc.y);
}
// acc += conj(a) * b
template <typename R> __device__ __forceinline__ void cfma_conj(cx<R> &acc, cx<R> a, cx<R> b) {
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(-a.y, b.x, acc.y);
}
template <typename R, typename S> __host__ __device__ __forceinline__ cx<R> cvt(cx<S> a) { return mk<R>((R)a.x, (R)a.y); }

template <typename R> struct prec_of;
template <> struct prec_of<double> { static const int value = PG_FP64; };
template <> struct prec_of<float> { static const int value = PG_FP32; };

// ------------------------------------------------------------------------------------
// context
// ------------------------------------------------------------------------------------
struct pg_ctx {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    long long launches = 0;
    int num_sms = 0;
    // scratch for reductions: per-block partials and an arrival counter
    double *red_partial = nullptr;   // [max_blocks * max_cols] complex -> 2 doubles each
    unsigned int *red_counter = nullptr;
    double *red_out = nullptr;       // [max_cols] complex + extra
    double *h_pinned = nullptr;      // pinned host mirror of red_out
    int red_max_blocks = 0;
    int red_max_cols = 0;
    int *d_err = nullptr;            // set to non-zero by a kernel whose bounded wait ran out
};

#define PG_CUDA_TRY(...)                                                                     \
    do {                                                                                     \
        cudaError_t _e = (__VA_ARGS__);                                                             \
        if (_e != cudaSuccess) {                                                             \
            pg_set_last_error(_e, #__VA_ARGS__, __FILE__, __LINE__);                                \
            return PG_ERR_CUDA;                                                              \
        }                                                                                    \
    } while (0)

#define PG_TRY(...)                                                                          \
    do {                                                                                     \
        int _s = (__VA_ARGS__);                                                                     \
        if (_s != PG_OK) return _s;                                                          \
    } while (0)

void pg_set_last_error(cudaError_t e, const char *what, const char *file, int line);
int pg_check_launch(pg_ctx *ctx);

// reduction scratch sizes
static const int PG_RED_BLOCKS = 304;   // 2 x 152 SMs
static const int PG_RED_COLS = 130;     // up to 128 Krylov vectors + norm + spare
int pg_ctx_ensure_reduction(pg_ctx *ctx);

// ------------------------------------------------------------------------------------
// device operator
// ------------------------------------------------------------------------------------
static const int PG_MAX_SLOTS = 16;

// Row-indexed launches: rows spread over grid y and z (gridDim.y is limited to 65535, a
// two-electron operator has Nang * N rows).
static const int PG_GRID_Y = 65535;
__host__ inline dim3 pg_row_grid(unsigned tiles, long long rows)
{
    const long long y = rows < PG_GRID_Y ? rows : PG_GRID_Y;
    return dim3(tiles, (unsigned)(y > 0 ? y : 1), (unsigned)((rows + PG_GRID_Y - 1) / PG_GRID_Y > 0 ? (rows + PG_GRID_Y - 1) / PG_GRID_Y : 1));
}
__device__ __forceinline__ int pg_grid_row() { return (int)(blockIdx.y + (unsigned)PG_GRID_Y * blockIdx.z); }

struct pg_scales {
    cxd s[PG_MAX_SLOTS];
};

struct OpDev {
    int nrows;        // angular rows (Nang)
    int N;            // radial length
    int ld;           // band row length on the device (N rounded up to a multiple of 4)
    int kb;           // super diagonals
    int b;            // 2kb+1
    const int *row_ptr;
    const int *ent_col;
    const int *ent_band;
    const int *ent_slot;
    const void *bands;  // [nbands][b][N] complex<R>
};

struct HostTerm {
    std::string storage;
    std::vector<std::string> kinds;        // storage id of each rank ("Simp", "BandNH", ...)
    std::vector<int> ext;                  // potential extent of each rank
    std::vector<std::vector<int>> pairs;   // (row, col) lists of the ranks that have one
    std::vector<double> pot;               // complex interleaved, reference layout
    int slot = 0;
};

// one factor of a factorized rank-3 term (pg_op_add_factored)
struct HostFactor {
    std::vector<double> radial;  // [N1][b][b][N2]
    double w[2] = {1.0, 0.0};
    int slot = 0;
    std::vector<int> row, col;
    std::vector<double> coef;
};

// device form of all factors of an operator (factored.cu)
struct FactDev {
    int Q = 0, Qp = 0, A = 0, Ap = 0, N1 = 0, N2 = 0, N2p = 0, nct = 0, nE = 0;
    int tw = 0, ntiles = 0;        // radial kernel: points of the last rank per CTA, tiles per row
    int df = 0;                    // FP64 operator computing its radial stencil in double-float
    size_t radial_smem = 0;        // its dynamic shared memory
    CUtensorMap zmap, rmap;        // TMA maps of the scratch and of the radial factors
    int *row_ptr = nullptr;           // [A + 1] segments per output channel
    int *col = nullptr;               // [segments][4]: factor, first and last+1 pair, 0
    int *nzq = nullptr;               // [pairs] input channel of each nonzero (channel, factor) pair
    int *slot = nullptr;              // [Q]
    int *perm = nullptr;              // [A] channel held by each scratch slot
    void *coef = nullptr;             // [pairs] its coefficient (operator precision)
    unsigned char *chunk = nullptr;   // [Ap / 4][Q] factors touched by each group of 4 channels
    unsigned char *bflag = nullptr;   // [Q][nct] channel tiles with a nonzero row
    // FP64 operators: the exact nonzero pairs, per (channel, factor) segment
    int *seg_ptr = nullptr, *seg = nullptr, *pcol = nullptr;  // [A + 1], [segments][4], [pairs]
    void *pcoef = nullptr;            // [pairs]
    unsigned char *seg_gq = nullptr;  // [Ap / 4][Q] factors touched by each group of 4 slots
    void *radial = nullptr;           // [Q][N1][b][b][N2p] real
    cxd *w = nullptr;                 // [Q]
    void *Z = nullptr;                // [Q][N1*N2][Ap] complex scratch (slots innermost)
    double flops_mix = 0, flops_radial = 0, radial_bytes = 0, z_bytes = 0;
};

struct pg_op {
    pg_ctx *ctx = nullptr;
    int rank = 2;
    std::vector<int> shape;  // extents of the wavefunction ranks
    int nrows = 0, N = 0, kb = 0, b = 0;  // nrows: product of all but the last extent
    int precision = PG_FP64;
    std::vector<HostTerm> terms;
    bool finalized = false;
    // device arrays
    int *d_row_ptr = nullptr, *d_ent_col = nullptr, *d_ent_band = nullptr, *d_ent_slot = nullptr;
    void *d_bands = nullptr;
    int nbands = 0;
    long long nentries = 0;
    int ld = 0;
    int use_bulk = 1;
    // matvec kernel variant, chosen by measurement at finalize (pg_op_set_variant overrides):
    // 1 bulk-copy 64-row tiles, 2 bulk-copy 128-row tiles, 3 plain loads (128 threads)
    int variant = 1;
    float variant_us[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    // 7, 8: variant 4 with groups of 2 or 1 band blocks (smaller shared memory, more CTAs per SM)
    void *d_bands_rm = nullptr;  // 6: row-major band copy [band][ld][2kb+1], one bulk copy per block
    // 4: bulk matvec with one TMA tensor copy per band block (when the tensor map exists);
    // 5: persistent CTAs, double-buffered TMA stages
    CUtensorMap tmap;
    bool has_tmap = false;
    OpDev dev() const {
        OpDev o;
        o.nrows = nrows; o.N = N; o.ld = ld; o.kb = kb; o.b = b;
        o.row_ptr = d_row_ptr; o.ent_col = d_ent_col; o.ent_band = d_ent_band; o.ent_slot = d_ent_slot;
        o.bands = d_bands;
        return o;
    }
    // host copy of bands in diagonal-major form (complex128), kept for preconditioner setup
    std::vector<std::complex<double>> h_bands;   // [nbands][b][N]
    std::vector<int> h_row_ptr, h_ent_col, h_ent_band, h_ent_slot;
    // radial ranks stored dense (N x N per angular pair), a second CSR over the rows
    int ndense = 0;
    long long ndense_entries = 0;
    int *d_drow_ptr = nullptr, *d_dent_col = nullptr, *d_dent_mat = nullptr, *d_dent_slot = nullptr;
    void *d_dense = nullptr;  // [ndense][j][i] (transposed: thread i reads row j contiguously)
    // factorized rank-3 terms
    std::vector<HostFactor> factors;
    FactDev fact;
    bool tuning = false;  // the variant autotuner times the banded part alone
    bool fp64_emulation = false;  // FP64 operator: factorized radial stencil in double-float
};

// factorized terms (factored.cu): upload at finalize, release, and the two-kernel apply that
// adds them to dst after the banded part
int pg_factored_finalize(pg_op *op);
void pg_factored_free(pg_op *op);
int pg_factored_apply(pg_op *op, const pg_scales &scales, const cxd *scales_dev, const void *src, void *dst,
                      const double *src_inv_scale_dev);

// matvec launcher shared by the drivers: dst = acc*dst + sum scales * V src
// scales_dev (optional) overrides `scales` when non-null.
int pg_op_matvec_dev(pg_op *op, const pg_scales &scales, const cxd *scales_dev, const void *src,
                     void *dst, int accumulate, const double *src_inv_scale_dev, void *src_copy_out);
// kernels one pg_op_matvec_dev call launches (banded part, plus the dense part when present)
int pg_op_matvec_kernels(const pg_op *op);

// ------------------------------------------------------------------------------------
// banded fibre operators
// ------------------------------------------------------------------------------------
// One blocked triangular matrix set: for each matrix, nblk blocks of 32 rows:
//   inv[m][blk][s][t] = (T_blk^-1)[t][s]     (t = output row within block, s = input row)
//   cpl[m][blk][j][t] = T(row, row -/+ j) coupling to the neighbouring block, j = 1..w
struct TriDev {
    int N, nblk, w;
    int lower;           // 1: forward (lower) solve, 0: backward (upper)
    int complex_coef;    // 1: complex coefficients, 0: real
    const void *inv;     // real: double/float [nmat][nblk][32][32]; complex: cx
    const void *cpl;     // [nmat][nblk][w][32]
};

struct pg_banded {
    pg_op *op = nullptr;
    int kind = 0;            // 0 overlap, 1 block preconditioner, 2 two-electron Kronecker preconditioner
    int N = 0, kb = 0, nmat = 0;
    int fib_per_mat = 1;     // consecutive fibres sharing one factor (fibre f uses factor f / fib_per_mat)
    // overlap: U upper Cholesky factor rows (real) for multiplies, lower = U^T
    void *d_U = nullptr;     // [N][kb+1]  U(i, i+j) at [i][j]   (real, precision of op)
    void *d_S = nullptr;     // [N][2kb+1] S rows (real)
    // blocked solves: inverse 32x32 diagonal blocks and the coupling G = T^-1 C to the
    // neighbouring block's kb boundary values
    void *d_lo_inv = nullptr, *d_lo_cpl = nullptr;   // lower factor (U^T or L)
    void *d_up_inv = nullptr, *d_up_cpl = nullptr;   // upper factor (U)
    void *d_lo_rb = nullptr, *d_up_rb = nullptr;     // inverses of the block-boundary systems
    int complex_coef = 0;
    // kind 2: the factors along the first electron's rank (applied on the swapped copy)
    void *d_lo_inv1 = nullptr, *d_lo_cpl1 = nullptr, *d_lo_rb1 = nullptr;
    void *d_up_inv1 = nullptr, *d_up_cpl1 = nullptr, *d_up_rb1 = nullptr;
    int fib_per_mat1 = 1;
    // kind 3: fast diagonalization per channel (fdprec.cu): eigenvectors V_l [nl][NP][NP]
    // (row k, column = eigenvector), the inverse spectra D [A][N][N] (complex), the eigenvector
    // set of each channel's two electrons [A][2]
    void *d_fdV = nullptr, *d_fdD = nullptr;
    int *d_fdl = nullptr;
    int fdN = 0, fdNP = 0;
    int fdGlobal = 0;                        // products as batched GEMMs through global memory
    void *d_fdP0 = nullptr, *d_fdP1 = nullptr;  // their planar scratch [A][2][N][N]
};

// kind-3 solve x <- M^-1 x on every channel (fdprec.cu); largest radial size of the
// shared-memory kernel (larger sizes use batched GEMMs through global memory); kernels per solve
int pg_fd_apply_dev(pg_banded *b, void *x);
int pg_fd_max_n(int precision);
int pg_fd_kernels(const pg_banded *b);
// checks the shared memory the solve needs for padded size NP and raises the kernel's limit
int pg_fd_prepare(int precision, int NP);

int pg_banded_apply_dev(pg_banded *b, int which, void *x);
// kernels one PG_BAND_PREC_SOLVE launches (a two-electron Kronecker preconditioner: 2 solves, 2 swaps)
int pg_banded_solve_kernels(const pg_banded *b);
// y[a][j][i] = x[a][i][j], x [n0][n1][n2] (vector.cu)
int pg_swap_last2_dev(pg_ctx *ctx, int precision, const void *x, void *y, int n0, int n1, int n2);

// ------------------------------------------------------------------------------------
// learned preconditioner network (mlp.cu)
// ------------------------------------------------------------------------------------
struct pg_mlp;
int pg_mlp_describe(pg_mlp *m, pg_ctx **ctx, int *d_in, int *d_out);
int pg_mlp_reserve(pg_mlp *m, int batch);
// Y (FP32 [batch][d_out]) = network(X (BF16 [batch][d_in])) on the network's context stream
int pg_mlp_forward_dev(pg_mlp *m, const void *X, int batch, float *Y);
// X (BF16 [nblk][d_in]) = [y_{a-1}, y_a, y_{a+1}] of y (complex64 [nblk][N]), scaled by *inv_scale
int pg_mlp_block_features_dev(pg_ctx *ctx, const void *y, int nblk, int N, int d_in, const double *inv_scale,
                              void *X);

// ------------------------------------------------------------------------------------
// vector kernels (vector.cu)
// ------------------------------------------------------------------------------------
// h[j] = sum_i conj(V[j][i]) w[i] for j < J; nrm2 = sum |w|^2. Results FP64 in ctx->red_out:
// red_out[2j], red_out[2j+1] = h[j]; red_out[2J] = ||w||^2.
// With Jdev non-null the column count is *Jdev + 1 (read on the device; J is then the
// host-side upper bound used for the scratch check).
// With atomic != 0 the cross-CTA sums are FP64 atomic adds into out_dev, which must hold
// zeros on entry (the consumer clears it after reading); out_dev[2J+1] (the norm) is then
// not written. Otherwise the last CTA to finish sums the partials (deterministic order).
template <typename R>
int pg_multidot(pg_ctx *ctx, const cx<R> *V, long long ldv, int J, const cx<R> *w, long long n, double *out_dev,
                const int *Jdev = nullptr, int atomic = 0);
// w -= sum_j V[j] h[j] with h complex128 on device; then the dots V[0..J)^H w (want_dots)
// and ||w||^2 into out_dev as pg_multidot
template <typename R>
int pg_gs_update(pg_ctx *ctx, const cx<R> *V, long long ldv, int J, const double *h_dev, cx<R> *w, long long n,
                 int want_dots, double *out_dev, const int *Jdev = nullptr, int atomic = 0);
