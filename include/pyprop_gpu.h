/*
 * pyprop_gpu.h - C ABI of the GB300 propagation hot path.
 *
 * One shared library, libpyprop_gpu.so, built for sm_103a. Plain C types only: device
 * buffers are passed as pointers, complex numbers as interleaved (re, im) pairs of double
 * or float, streams as cudaStream_t cast to void*. Every entry point returns 0 on success
 * or a negative PG_ERR_* code; pg_error_string() names it. Nothing here falls back to the
 * CPU: without a usable CUDA device the calls fail with PG_ERR_CUDA.
 *
 * Wavefunction layout is the reference's C order: rank 2 (one electron) is [Nang][N]
 * (angular channel, B-spline); rank 3 (two electrons) is [Nang][N][N].
 */
#ifndef PYPROP_GPU_H
#define PYPROP_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------------------------- */
/* status codes, precision, context                                                   */
/* ---------------------------------------------------------------------------------- */

enum {
    PG_OK = 0,
    PG_ERR_ARG = -1,           /* bad argument (null pointer, size out of range) */
    PG_ERR_CUDA = -2,          /* a CUDA runtime call failed or no device */
    PG_ERR_STORAGE = -3,       /* storage id combination not supported */
    PG_ERR_SHAPE = -4,         /* extents disagree with the operator or wavefunction */
    PG_ERR_NONFINITE = -5,     /* NaN/Inf detected by a checking kernel */
    PG_ERR_BREAKDOWN = -6,     /* Krylov breakdown that the method cannot absorb */
    PG_ERR_NOT_CONVERGED = -7, /* iterative solve stopped at its iteration cap */
    PG_ERR_ALLOC = -8,         /* device allocation failed */
    PG_ERR_STATE = -9          /* object used before setup / after destroy */
};

enum { PG_FP64 = 0, PG_FP32 = 1 };

typedef struct pg_ctx pg_ctx;

/* Error name for a status code (static string). */
const char *pg_error_string(int code);

/* Library build string: compiler, arch, build flags. */
const char *pg_version(void);

/* Create a context on CUDA device `device` with its own non-blocking stream. */
int pg_ctx_create(int device, pg_ctx **out);
int pg_ctx_destroy(pg_ctx *ctx);
/* The context's stream (cudaStream_t as void*). */
void *pg_ctx_stream(pg_ctx *ctx);
/* Use the caller's stream for all later work of this context (NULL = the legacy default
 * stream, so that work stays ordered with the caller's default-stream work). */
int pg_ctx_set_stream(pg_ctx *ctx, void *stream);
/* Go back to the context's own non-blocking stream. */
int pg_ctx_use_own_stream(pg_ctx *ctx);
/* Count of kernels this context launched since creation (own kernels only). */
long long pg_ctx_kernel_launches(pg_ctx *ctx);
int pg_ctx_synchronize(pg_ctx *ctx);
/* Device error word: non-zero when a kernel's bounded wait ran out (1: an asynchronous copy,
 * 2: a grid barrier of the single-kernel Cayley step, 3: a factor copy of its cluster variant)
 * or when a single-kernel Cayley step was launched with another shape than it was built for
 * (4: a different grid, or the cluster variant without its thread-block clusters); the kernel
 * then skipped the rest of its work. Waits for the context's stream. */
int pg_ctx_device_error(pg_ctx *ctx, int *flag);
/* Clear the device error word (stream-ordered). */
int pg_ctx_clear_device_error(pg_ctx *ctx);

/* ---------------------------------------------------------------------------------- */
/* reference-layout tensor multiply                                                   */
/* ---------------------------------------------------------------------------------- */
/*
 * Device twins of the generated Fortran kernels tensorpotentialmultiply_<ids>_ for rank 2
 * (pyprop: core/tensorpotential/tensorpotentialmultiply_generator.py:1391-1495, storage
 * snippets Diag :403-432, Simp :302-363, Ident :436-462, BandNH :622-762). Same argument
 * order and meaning, all pointers on the device, complex128 interleaved:
 *     dest += scaling * V * source
 * The potential is in the reference's layout [pairs0][N*(2k+1)], BandNH slot
 * j*(2k+1) + (k+i-j) holding V(i, j). `bandCount` is k (super diagonals).
 */
int pg_tensor_multiply_diag_bandnh(const double *potential, int potExtent0, int potExtent1,
                                   double scaling,
                                   const double *source, int srcExtent0, int srcExtent1,
                                   double *dest, int dstExtent0, int dstExtent1,
                                   int bandCount, void *stream);
int pg_tensor_multiply_simp_bandnh(const double *potential, int potExtent0, int potExtent1,
                                   double scaling,
                                   const double *source, int srcExtent0, int srcExtent1,
                                   double *dest, int dstExtent0, int dstExtent1,
                                   const int *pair0, int pair0Extent0, int pair0Extent1,
                                   int bandCount, void *stream);
int pg_tensor_multiply_ident_bandnh(const double *potential, int potExtent0, int potExtent1,
                                    double scaling,
                                    const double *source, int srcExtent0, int srcExtent1,
                                    double *dest, int dstExtent0, int dstExtent1,
                                    int bandCount, void *stream);

/* ---------------------------------------------------------------------------------- */
/* fused device operator: sum over terms of scale[slot] * V_term                       */
/* ---------------------------------------------------------------------------------- */
/*
 * Replaces the Python loop over consolidated TensorPotentials
 * (pyprop/tensorpotential/BasisPropagator.py:116-159, TensorPotential.py:92-112) by one
 * resident operator applied in one launch. Terms are added in the reference layout and
 * converted once to the device layout (per-pair bands stored diagonal-major).
 */
typedef struct pg_op pg_op;

/* shape: rank-2 {Nang, N} or rank-3 {Nang, N, N}. bandCount k: the band of the last
 * (fibre) rank has 2k+1 diagonals. */
int pg_op_create(pg_ctx *ctx, int rank, const int *shape, int bandCount, int precision, pg_op **out);
int pg_op_destroy(pg_op *op);
/*
 * Add one term. storage: "<angular>_<radial>" as in the names of the reference's generated
 * kernels (core/tensorpotential/tensorpotentialmultiply_generator.py:1336-1346):
 *   angular Simp, Herm, Diag, Ident, Band, BandNH, Dense; radial BandNH, Band, Dense,
 *   Diag, Ident. Extents: potExtent0 = npairs (Simp, Herm), Nang (Diag), 1 (Ident),
 *   Nang*bandCount (Band, BandNH), Nang^2 (Dense); potExtent1 = N(2k+1) (BandNH), N(k+1)
 *   (Band), N^2 (Dense), N (Diag), 1 (Ident).
 * potential: host complex128 [potExtent0][potExtent1] in the reference layout.
 * pairs0: host int32 [npairs0][2] (row, col) for Simp and Herm (ignored otherwise).
 * slot: which scale multiplies this term (0 <= slot < 16).
 * Returns PG_ERR_STORAGE for other ids and PG_ERR_SHAPE for extents that do not match.
 */
int pg_op_add_term(pg_op *op, const char *storage, const double *potential, int potExtent0,
                   int potExtent1, const int *pairs0, int npairs0, int slot);
/*
 * Rank-general form (rank-2 and rank-3 operators; rank 3 is the two-electron layout
 * [Nang][N][N] of core/tensorpotential/tensorpotentialmultiply_generator.py's rank-3
 * kernels such as Diag_Simp_BandNH and Simp_Simp_BandNH). storage "<r0>_<r1>[_<r2>]";
 * extents[rank] as pg_op_add_term (Simp on the last rank: a pair list within or beyond the
 * band); pairs: the (row, col) lists of all Simp/Herm ranks concatenated in rank order,
 * npairs[rank] their lengths (0 for other ranks).
 */
int pg_op_add_term_ranks(pg_op *op, const char *storage, const double *potential, const int *extents,
                         const int *pairs, const int *npairs, int slot);
/*
 * Factorized rank-3 terms: V = sum_q w_q * scale[slot_q] * A_q (x) R_q, each factor q an
 * angular matrix A_q (sparse, real) times a radial operator R_q on both radial ranks that is
 * shared by every angular pair. This is the multipole form of the electron-electron
 * repulsion, V(pair) = sum_l3 c_l3(pair) r<^l3 / r>^(l3+1)
 * (examples/tensor/helium_stabilization/coupledspherical.cpp:7-127, potential data per pair
 * on SelectionRule_R12 x banded-packed x banded-nonhermitian): the reference stores the sum
 * per angular pair (Simp_Simp_BandNH, tensorpotentialmultiply_generator.py:302-363,622-762),
 * which at L <= 8, l <= 16, 200 splines is 14 TB; per factor it is one band x band block.
 * radial: host float64 [nfactors][N1][2k+1][2k+1][N2], element (i1, d1, d2, i2) coupling
 * output (i1, i2) to input (i1 + d1 - k, i2 + d2 - k) (k = bandCount, N1 = shape[1],
 * N2 = shape[2]). weights: complex128 [nfactors]; slots [nfactors]. Entries (factor, row,
 * col, coef): A_factor[row][col] += coef, dst[row] += ... src[col]. Several calls add
 * factors. Applied by every matvec after the banded terms (two more kernels: the angular
 * mix of src into per-factor scratch, then the radial stencil summed over factors into dst).
 */
int pg_op_add_factored(pg_op *op, int nfactors, const double *radial, const double *weights, const int *slots,
                       long long nentries, const int *ent_factor, const int *ent_row, const int *ent_col,
                       const double *ent_coef);
/* FP64 operators only, before pg_op_finalize (no reference counterpart): compute the radial
 * stencil of the factorized terms in double-float arithmetic (each value an FP32 pair hi + lo,
 * error-free products and sums: relative accuracy about 2^-48 instead of 2^-53) instead of FP64
 * FMAs, which run at a small fraction of the FP32 rate on this GPU. Meant for the FP64
 * residuals of mixed-precision solves. */
int pg_op_set_fp64_emulation(pg_op *op, int on);
/* Bookkeeping of the factorized part (no reference counterpart): info[0] factors, [1]
 * angular entries (row, col), [2] flops of the angular mix and [3] of the radial stencil per
 * matvec (real multiply-adds x 2, zero blocks skipped as the kernels skip them), [4] bytes
 * of radial factors, [5] bytes of the per-factor scratch. Zeros when there is none. */
int pg_op_factored_info(const pg_op *op, double *info);
/* Upload. Must be called once after the last add_term. */
int pg_op_finalize(pg_op *op);
/* Matvec kernel variant (no reference counterpart): pg_op_finalize times the candidates on
 * the operator's own shape (1 bulk-copy staging with 64-row tiles, 2 with 128-row tiles,
 * 3 plain coalesced loads, 4 one TMA tensor copy per band block, 5 persistent CTAs with
 * double-buffered TMA stages - 4 and 5 when the driver offers tensor maps - and 6 one bulk
 * copy per block from a row-major copy of the bands, kept only when chosen; 7 and 8 variant 4
 * with groups of two or one block) and keeps the fastest. variant 1..8 forces one (PG_ERR_ARG
 * for 4, 5, 7, 8 without a tensor map), variant < 0 only reads; current (optional) receives the
 * variant in use, times_us (optional, 9 floats) the tuning times per variant index (0: not
 * measured). */
int pg_op_variant(pg_op *op, int variant, int *current, float *times_us);
/* Number of complex band elements the operator stores (for roofline bookkeeping). */
long long pg_op_stored_elements(const pg_op *op);
/*
 * dst = (accumulate ? dst : 0) + sum_t scales[slot_t] * V_t * src
 * scales: host complex128 array [nscales] (interleaved), nscales <= 16.
 * src/dst: device arrays in the operator's precision (complex128 or complex64).
 */
int pg_op_matvec(pg_op *op, const double *scales, int nscales, const void *src, void *dst,
                 int accumulate);

/* ---------------------------------------------------------------------------------- */
/* banded fibre operators: overlap S = U^T U and block-diagonal preconditioner LU      */
/* ---------------------------------------------------------------------------------- */
/*
 * Replaces OverlapMatrix multiply/solve along the B-spline rank
 * (core/representation/overlapmatrix.cpp:123-229, zpbtrf factor :35-37) and the
 * per-channel banded LU of BSplineSolver (core/transform/bspline/bsplinesolver.h:43-162).
 * A fibre is one radial vector psi[a][:] (rank 2). Solves run one warp per fibre over
 * 32-row blocks with precomputed inverse diagonal blocks.
 */
typedef struct pg_banded pg_banded;

/*
 * Overlap: `overlap_rows` is host float64 [N][2k+1], row i column k+(j-i) = S(i, j).
 * The Cholesky factor is computed on the host in float64.
 */
int pg_overlap_create(pg_op *op, const double *overlap_rows, pg_banded **out);
/*
 * Block-diagonal preconditioner M_a = cS * S + cH * H_a for every angular channel a,
 * H_a from the Diag_BandNH terms of `op` with the given slots weighted by slot_weights
 * (complex128). Factored M = L U without pivoting (M has a positive definite Hermitian part).
 */
int pg_prec_blockdiag_create(pg_op *op, const double *overlap_rows, const double *cS,
                             const double *cH, const int *slots, const double *slot_weights,
                             int nslots, pg_banded **out);
/* Two-electron radial preconditioner for rank-3 operators [Nang][N][N], Kronecker-factorized
 * per angular channel: M_a = (cS S + cH h1_a) x (cS S + cH h2_a), h1_a, h2_a (host complex128
 * rows [Nang][N][2k+1], layout of overlap_rows) the one-electron radial Hamiltonians of the
 * channel's two electrons. Stands in for the reference's sparse direct / ILU block
 * preconditioners (examples/tensor/helium_stabilization/preconditioner.py:77-244): it omits
 * the electron-electron repulsion of the block. Applied by PG_BAND_PREC_SOLVE (one banded
 * block solve along each radial rank). */
int pg_prec_kron_create(pg_op *op, const double *overlap_rows, const double *cS, const double *cH,
                        const double *h1, const double *h2, pg_banded **out);
/* Two-electron radial preconditioner by fast diagonalization: per angular channel a the exact
 * inverse of cS S x S + cH (h_l1 x S + S x h_l2), applied as (V1 x V2) D_a (V1 x V2)^T with the
 * generalized eigenvectors of the one-electron Hamiltonians (h_l V_l = S V_l Lambda_l,
 * V_l^T S V_l = 1). V: host float64 [nl][N][N] (V[l][k][i] = component k of eigenvector i),
 * lam [nl][N], lidx [Nang][2] the eigenvector set of each channel's two electrons. In place of
 * the reference's per-channel sparse LU / ILU block preconditioners
 * (examples/tensor/helium_stabilization/preconditioner.py:77-244): exact for every term but
 * the electron-electron repulsion. Requires N1 = N2. Up to pg_prec_fd_max_n(precision) the
 * channel block lives in shared memory (one kernel per solve); beyond, the four products run
 * as batched GEMMs on planar copies in global memory (seven kernels, two scratch copies of the
 * wavefunction). Applied by PG_BAND_PREC_SOLVE. */
int pg_prec_fd_create(pg_op *op, int nl, const double *V, const double *lam, const int *lidx, const double *cS,
                      const double *cH, pg_banded **out);
int pg_prec_fd_max_n(int precision);
int pg_banded_destroy(pg_banded *b);

enum {
    PG_BAND_MUL_U = 0,     /* x <- U x            (MultiplySqrtOverlap(false)) */
    PG_BAND_MUL_UT = 1,    /* x <- U^H x          (MultiplySqrtOverlap(true)) */
    PG_BAND_SOLVE_U = 2,   /* x <- U^-1 x         (SolveSqrtOverlap(false)) */
    PG_BAND_SOLVE_UT = 3,  /* x <- U^-H x         (SolveSqrtOverlap(true)) */
    PG_BAND_MUL_S = 4,     /* x <- S x            (MultiplyOverlap) */
    PG_BAND_SOLVE_S = 5,   /* x <- S^-1 x         (SolveOverlap) */
    PG_BAND_PREC_SOLVE = 6 /* x <- M_a^-1 x per channel (preconditioner Solve) */
};
/* In place on a device wavefunction in the operator's precision. */
int pg_banded_apply(pg_banded *b, int which, void *x);

/* ---------------------------------------------------------------------------------- */
/* Krylov propagators and solvers                                                     */
/* ---------------------------------------------------------------------------------- */

typedef struct pg_krylov_stats {
    long long OpCount;           /* operator applications */
    long long InnerProductCount; /* block inner products (one per Gram-Schmidt pass) */
    long long ReOrthoCount;      /* second Gram-Schmidt passes */
    long long RestartCount;      /* pIRAM restarts */
    long long Iterations;        /* GMRES iterations in the last solve */
    double ErrorEstimate;        /* pAMP |last Krylov coefficient|^2 or GMRES residual */
    double TrueResidual;         /* GMRES: ||b - A x|| recomputed after the solve */
} pg_krylov_stats;

typedef struct pg_pamp pg_pamp;
/*
 * pAMP exp(-i dt H) psi (core/krylov/pamp/pamp/pamp.h:613-670) in the balanced-overlap
 * form of PamPropagator.AdvanceStep (pyprop/propagator/PamPropagator.py:50-75):
 * psi <- U psi; Krylov with U^-H H(t) U^-1; psi <- U^-1 psi. H is frozen at t.
 * basis_precision: PG_FP64 or PG_FP32 Arnoldi basis (psi itself is always complex128).
 * double_ortho: 1 always runs a second Gram-Schmidt pass (CGS2).
 */
int pg_pamp_create(pg_op *op64, pg_op *op_basis, pg_banded *ovl64, pg_banded *ovl_basis,
                   int basis_size, int basis_precision, int double_ortho, pg_pamp **out);
int pg_pamp_destroy(pg_pamp *p);
/*
 * One step. scales: host complex128 [nscales], H(t) slot values. psi: device complex128.
 * Three forms, all with the reference's order-6 Pade exponential (pamp.h:430-565) or, on the
 * host, the same for a Hermitian tridiagonal H_m by implicit QL:
 *  - complex64 basis: the single-kernel step below (the default where it qualifies);
 *  - otherwise, by default: two captured graphs with the m x m exponential on the host between
 *    them (the call waits every step; faster on this GPU than its FP64 Pade);
 *  - pg_pamp_set_device_exp(p, 1) (basis_size <= 48): one graph launch with the exponential in
 *    one CTA on the device; the call returns without waiting.
 * With stats != NULL the call waits and fills them. On the device forms a singular Pade
 * denominator zeroes that step's coefficients and is reported (PG_ERR_BREAKDOWN) by the next
 * call that reads statistics.
 */
int pg_pamp_step(pg_pamp *p, void *psi, double dt, const double *scales, int nscales,
                 pg_krylov_stats *stats);
int pg_pamp_set_device_exp(pg_pamp *p, int on); /* PG_ERR_STATE for on=1 when basis_size > 48 */
int pg_pamp_last_stats(pg_pamp *p, pg_krylov_stats *stats); /* waits for the last step */
/*
 * Single-kernel step (complex64 basis with double_ortho = 1; the default where it qualifies: a
 * rank-2 operator with real bands, at most 4 source channels per row, basis_size <= 48 and its
 * working set within a CTA's shared memory, one resident CTA per channel): one cooperative
 * launch runs the Arnoldi recurrence on T_j = U^-1 V_j (S-orthonormal, the same Krylov space
 * and Hessenberg matrix as the balanced form), the m x m exponential in
 * double-float arithmetic in every CTA, and psi = ||psi||_S sum_j c_j T_j. Two grid barriers
 * per Arnoldi step, each a bounded wait: one that runs out sets the context's error word to 2,
 * leaves psi unchanged, and the next call that reads statistics returns PG_ERR_NOT_CONVERGED.
 * pg_pamp_set_fused(p, 0) selects the graphs; on=1 returns PG_ERR_STORAGE/SHAPE/STATE when the
 * stepper does not qualify. pg_pamp_set_barrier_probe is a test hook: grid barrier number
 * at_barrier of later steps waits for extra_arrivals arrivals that never come.
 */
int pg_pamp_set_fused(pg_pamp *p, int on);
int pg_pamp_set_barrier_probe(pg_pamp *p, int extra_arrivals, int at_barrier);
/*
 * pAMP ensembles (no reference counterpart: the reference runs one wavefunction per process):
 * many pg_pamp members (each with its own operator, overlap and basis size) advanced together,
 * one launch per ensemble step. When every member has a complex64 basis (at most 24 vectors)
 * and a rank-2 operator with real bands, the step is one persistent kernel: each CTA takes
 * members from a device work list (largest first) and runs a member's whole pAMP step - psi
 * <- U psi, the Arnoldi steps with CGS2 and FP64 sums, the m x m exponential (scaling and
 * squaring of the order-6 Pade approximant, pamp.h:430-565) and psi = U^-1 V c. Its launch
 * shape (threads per CTA, CTAs) is chosen at the first step by timing the candidates on the
 * members themselves (their wavefunctions are saved and restored around the trials), and
 * the graph of every member's kernels (all exponentials in one kernel) is timed beside it: the
 * faster of the two is kept (a member runs on one SM in the persistent kernel and on the whole
 * GPU in the graph, so small ensembles of large members can favour the graph). Members that do
 * not qualify always take the graph. While a batch exists its members read their slot values
 * from the batch; pg_pamp_batch_destroy gives them back their own.
 * scales: [nmembers][nscales] complex.
 */
typedef struct pg_pamp_batch pg_pamp_batch;
int pg_pamp_batch_create(pg_pamp **members, int nmembers, pg_pamp_batch **out);
int pg_pamp_batch_destroy(pg_pamp_batch *b);
int pg_pamp_batch_step(pg_pamp_batch *b, void **psis, double dt, const double *scales, int nscales);
/* Per-member statistics of the last completed ensemble step (waits); Iterations = Krylov
 * basis size used (smaller after a happy breakdown). PG_ERR_BREAKDOWN if a Pade denominator
 * was singular. */
int pg_pamp_batch_stats(pg_pamp_batch *b, pg_krylov_stats *stats);
/* 1 = the persistent kernel (PG_ERR_STORAGE when a member does not qualify), 0 = the graph,
 * -1 = the faster of the two, timed at the next step (the default) */
int pg_pamp_batch_set_mode(pg_pamp_batch *b, int mode);
/* the mode in use, the tuned launch shape (0 before the first timed step) and the timed
 * ensemble steps in ms (graph_ms 0 when the graph was not timed); all outputs but mode may be
 * null */
int pg_pamp_batch_get_mode(pg_pamp_batch *b, int *mode, int *threads, int *ctas, float *persistent_ms,
                           float *graph_ms);

typedef struct pg_cayley pg_cayley;
/*
 * Cayley / Crank-Nicolson step (pyprop/propagator/CayleyPropagator.py:71-150):
 * (S + i dt/2 H) psi' = (S - i dt/2 H) psi with H at t + dt/2, GMRES
 * (core/krylov/gmres/gmres.h:433-505) left-preconditioned by the block-diagonal LU.
 * The step is one CUDA graph launch: GMRES iterations are a conditional WHILE node whose
 * last kernel applies the Givens rotations and sets the loop condition on the device.
 * basis_precision PG_FP64: the reference scheme (x0 = 0) in complex128. PG_FP32: the FP64
 * residual r = b - A psi, a complex64 GMRES for the correction (2e-6 relative), psi += d,
 * r -= A d in FP64, repeated while the true residual ||r|| > tolerance (at most 4 passes).
 * op64/op_basis must contain the overlap as slot 0 (Ident_BandNH term) and the terms of H
 * in slots >= 1. tolerance is floored at 1e-13 (gmres.h:223-229). basis_size <= 64.
 */
int pg_cayley_create(pg_op *op64, pg_op *op_basis, pg_banded *prec64, pg_banded *prec_basis,
                     int basis_size, int basis_precision, double tolerance, pg_cayley **out);
int pg_cayley_destroy(pg_cayley *c);
/* One step. scales: host complex128 [nscales] slot values of H(t + dt/2) (slot 0 is
 * ignored: the overlap weight is fixed). With stats non-NULL the call waits for the step and
 * fills them (Iterations, ErrorEstimate = last least-squares residual, TrueResidual); with
 * NULL it returns after enqueueing. PG_ERR_NOT_CONVERGED (with stats) when the step was
 * abandoned because a bounded wait ran out: the context's device error word is set (it stays
 * set, and later steps report the same, until pg_ctx_clear_device_error). A step abandoned
 * before its first refinement pass leaves psi unchanged; one abandoned later may leave psi
 * partly corrected. */
int pg_cayley_step(pg_cayley *c, void *psi, double dt, const double *scales, int nscales,
                   pg_krylov_stats *stats);
/* nsteps steps; scales_table: host complex128 [nsteps][nscales]. With stats non-NULL the
 * call waits and fills the last step's statistics; PG_ERR_NOT_CONVERGED when any of the steps
 * was abandoned (the device error word, as for pg_cayley_step). */
int pg_cayley_advance(pg_cayley *c, void *psi, double dt, int nsteps, const double *scales_table,
                      int nscales, pg_krylov_stats *stats);
/* Statistics of the last completed step (waits for the stream). */
int pg_cayley_last_stats(pg_cayley *c, pg_krylov_stats *stats);
/* GMRES iterations and refinement passes summed over every step of this stepper so far
 * (waits for the stream): totals of a run whose steps were enqueued without statistics. Same
 * reference step as pg_cayley_step (CayleyPropagator.py:71-150; the reference keeps per-solve
 * counters in GmresWrapper, gmreswrapper.h). */
int pg_cayley_totals(pg_cayley *c, long long *iterations, long long *passes);
/* FP64 mode: also compute ||(S + i dt/2 H) psi' - b|| every step (one extra matvec). */
int pg_cayley_set_true_residual(pg_cayley *c, int on);
/* Eager mode: the same kernels launched one by one with the GMRES/refinement loops driven
 * from the host (one wait per iteration). For profilers that cannot look inside
 * conditional graph nodes; results are identical to the graph mode. Eager steppers always
 * take the multi-kernel step. */
int pg_cayley_set_eager(pg_cayley *c, int on);
/* Single-kernel mixed step (the same scheme as the PG_FP32 step above, as one cooperative
 * launch: CTA a solves angular channel a, the FP64 residual rows are spread over all SMs,
 * grid barriers between the phases, each a bounded wait that sets the context's device error
 * flag to 2 when it runs out). The default for PG_FP32 steppers of a rank-2 banded operator
 * (no dense or factorized terms) with the block-diagonal LU preconditioner, basis_size <= 32
 * and no more channels than resident CTAs; the learned preconditioner and the eager mode
 * use the multi-kernel step. on = 0 selects the multi-kernel step; on = 1 on a stepper that
 * does not qualify returns why: PG_ERR_STATE (not PG_FP32), PG_ERR_STORAGE (operator or
 * preconditioner kind), PG_ERR_SHAPE (basis size, fibre length, channel count). Replaces the
 * same reference step as
 * pg_cayley_step (CayleyPropagator.py:71-150). */
int pg_cayley_set_fused(pg_cayley *c, int on);
/* Layout of the single-kernel step (same reference step as pg_cayley_step,
 * CayleyPropagator.py:71-150). variant 0 (default): each angular channel on a thread-block
 * cluster of three CTAs, each holding a third of that channel's preconditioner factors in
 * shared memory for the whole step, where the fibre length fits (about 700 B-splines of
 * order 7) and all clusters can be resident at once, else one CTA per channel; 1: one CTA per
 * channel; 2: the cluster layout (PG_ERR_SHAPE where it does not fit). Both give the same
 * states to the GMRES tolerance. PG_ERR_STATE etc. as pg_cayley_set_fused when the stepper
 * has no single-kernel step. pg_cayley_get_fused_variant: 1 or 2 for the layout the next
 * step uses, 0 when the step is not the single-kernel one. */
int pg_cayley_set_fused_variant(pg_cayley *c, int variant);
int pg_cayley_get_fused_variant(pg_cayley *c, int *variant);
/* Test hook for the bounded grid barriers of the single-kernel step (no counterpart in the
 * reference): with extra_arrivals > 0, grid barrier number at_barrier (0 = the first of a
 * step) of every later step waits for that many arrivals more than there are CTAs, so its
 * polls run out (a few seconds); the step returns early and sets the device error word to 2,
 * and the step call reports PG_ERR_NOT_CONVERGED. A step abandoned at barrier 0 leaves psi
 * unchanged. extra_arrivals = 0 restores normal steps. */
int pg_cayley_set_barrier_probe(pg_cayley *c, int extra_arrivals, int at_barrier);
/*
 * Learned preconditioner (no counterpart in the reference; mixed-precision steppers only).
 * With a network set, each refinement pass runs flexible GMRES right-preconditioned by
 *     P(v) = M^-1 v + s(t) * mlp(features(M^-1 v)),  s(t) = i dt/2 h_slot(t + dt/2)
 * (M the block-diagonal radial LU, features as pg_mlp_block_features, d_out >= 2N). The FP64
 * true residual judges each pass: a pass that does not halve it is discarded and the rest of
 * the step uses M^-1 alone (the fallback). mlp == NULL switches the learned part off. The
 * network must live on the stepper's context and outlive its use.
 */
struct pg_mlp;
int pg_cayley_set_learned(pg_cayley *c, struct pg_mlp *mlp, int coupling_slot);
/* passes rejected by the residual test so far (waits for the stream) */
int pg_cayley_learned_rejected(pg_cayley *c, long long *out);

/* Ensembles: many pg_cayley members (each with its own operator, basis size, field) advanced
 * together by one CUDA graph launch whose branches (one per member) run concurrently. The
 * members keep their own buffers; the batch owns the graph. While a batch exists, stepping a
 * member alone rebuilds that member's graph. */
typedef struct pg_cayley_batch pg_cayley_batch;
int pg_cayley_batch_create(pg_cayley **members, int nmembers, pg_cayley_batch **out);
int pg_cayley_batch_destroy(pg_cayley_batch *b);
/* One step of every member: psis[k] device complex128 wavefunction of member k,
 * scales host complex128 [nmembers][nscales] slot values of H_k(t + dt/2). Enqueues only. */
int pg_cayley_batch_step(pg_cayley_batch *b, void **psis, double dt, const double *scales, int nscales);
/* Per-member statistics of the last step (waits): stats[nmembers]. */
int pg_cayley_batch_stats(pg_cayley_batch *b, pg_krylov_stats *stats);

/* Arnoldi expansion used by pIRAM (core/krylov/piram/piram/piram.h:346-442), Euclidean
 * inner product, re-orthogonalisation on. Operator: S^-1 H(slot scales) or, when
 * shift_invert (a pg_prec_blockdiag_create object for M = H0 - sigma S) is given,
 * M^-1 S - the shift-invert operator of GMRESShiftInvertSolver
 * (pyprop/solver/GMRESShiftInvertSolver.py:103-131) for an H diagonal in the angular rank.
 * On entry V[0..j0] (device complex128 [m][Npsi]) hold the basis and f the residual; the
 * call fills V[j0+1..m-1], the Hessenberg columns of H (host complex128 [m][m], row
 * major) and leaves the last residual in f. If ||f|| < breakdown_tol before a new
 * vector, it stops with *steps_done = that vector's index so the caller can put a random
 * vector into f and call again with inject = 1 (f is then orthogonalised against the basis
 * and the subdiagonal entry set to 0). *steps_done = m when the expansion completed. */
int pg_arnoldi_expand(pg_op *op64, pg_banded *ovl64, pg_banded *shift_invert, const double *scales,
                      int nscales, void *V, int m, int j0, void *f, double *H, double breakdown_tol,
                      int inject, int *steps_done, double *residual_norm_out, pg_krylov_stats *stats);

/* ---------------------------------------------------------------------------------- */
/* vector utilities on device wavefunctions                                           */
/* ---------------------------------------------------------------------------------- */

/* out = sum conj(x) y over n complex elements, FP64 accumulation. precision selects the
 * element type. out: host complex128. */
int pg_vec_dot(pg_ctx *ctx, int precision, const void *x, const void *y, long long n, double *out);
/* y (precision) <- convert(x (other precision)); n complex elements. */
int pg_vec_convert(pg_ctx *ctx, int src_precision, const void *x, int dst_precision, void *y, long long n);
/* V (complex128 [k][n]) <- V (complex128 [m][n]) * Q (host complex128 [m][k], row major) */
int pg_vec_combine(pg_ctx *ctx, void *V, long long n, int m, const double *Q, int k);
/* y[a][j][i] = x[a][i][j] for x [n0][n1][n2] (device, precision PG_FP64/PG_FP32, x != y): the
 * two-electron wavefunction's radial ranks swapped, so that operations along the first
 * electron's rank run as fibre operations (CombinedRepresentation over two B-spline ranks,
 * core/representation/combinedrepresentation.cpp:164-238). */
int pg_vec_swap_last2(pg_ctx *ctx, int precision, const void *x, void *y, int n0, int n1, int n2);

/* ---------------------------------------------------------------------------------- */
/* learned preconditioner network                                                     */
/* ---------------------------------------------------------------------------------- */
/*
 * No counterpart in the reference (its Cayley preconditioners are fixed factorizations,
 * pyprop/propagator/CayleyPropagator.py:56-63, examples/tensor/helium_stabilization/
 * preconditioner.py:77-244). A bias-free 3-layer ReLU MLP, y = W3^T relu(W2^T relu(W1^T x)),
 * one row per angular block: BF16 weights and activations into tensor-core products with
 * FP32 accumulation; FP32 master weights, gradients and Adam moments. d_in, hidden and d_out
 * must be multiples of 8. Weights on the host: FP32 [W1 d_in x hidden | W2 hidden x hidden |
 * W3 hidden x d_out], row-major with fan-in rows. X is BF16 [batch][d_in], Y and T FP32
 * [batch][d_out], all device pointers; the loss is mean over rows of ||y - t||^2.
 */
typedef struct pg_mlp pg_mlp;
int pg_mlp_create(pg_ctx *ctx, int d_in, int hidden, int d_out, unsigned long long seed, pg_mlp **out);
int pg_mlp_destroy(pg_mlp *m);
long long pg_mlp_parameter_count(const pg_mlp *m);
int pg_mlp_get_weights(pg_mlp *m, float *host);
int pg_mlp_set_weights(pg_mlp *m, const float *host);  /* also resets the optimizer */
int pg_mlp_forward(pg_mlp *m, const void *X_bf16, int batch, float *Y);
/* loss and gradients (grads_host optional, FP32, layout of the weights) */
int pg_mlp_gradients(pg_mlp *m, const void *X_bf16, const float *T, int batch, double *loss, float *grads_host);
/* one Adam step (beta1 0.9, beta2 0.999, eps 1e-8); loss optional (waits when given) */
int pg_mlp_train_step(pg_mlp *m, const void *X_bf16, const float *T, int batch, float lr, double *loss);
/* network input of the block-preconditioned vector y (complex64 [nblk][N], device): row a =
 * [y_{a-1}, y_a, y_{a+1}] real/imaginary interleaved, zero outside, padded to d_in >= 6N */
int pg_mlp_block_features(pg_ctx *ctx, const void *y, int nblk, int N, int d_in, void *X_bf16);

/* ---------------------------------------------------------------------------------- */
/* operator construction: projection into B-spline band rows                          */
/* ---------------------------------------------------------------------------------- */
/*
 * pg_bspline_band_project: for every batch row b < nbatch, the band rows of
 *     M_b[i][j] = sum_{m < nint} sum_{p < q} w[m q + p] B[m][i - first[m]][p] B[m][j - first[m]][p]
 *                 F[b * in_bstride + (m q + p) * in_qstride],   |i - j| < k,
 * written to out[(b / bdiv) * ob1 + (b % bdiv) * ob2 + i * oi + d * od], d = (k - 1) + j - i
 * (all pointers device, FP64). B [nint][k][q]: the k splines nonzero on quadrature interval m
 * (first[m] + a, zero values outside [0, N)) at its q points; w [nint * q] the quadrature
 * weights. This is the representation of a grid function in the B-spline basis that the
 * tensor-potential generator performs on the host (TensorPotentialGenerator.py:80-274,
 * core/tensorpotential/basis_bspline.h:11-47, BSplineGlobalOverlapIntegral in
 * core/transform/bspline/bspline.cpp:373-466), without derivatives; two calls (along r2,
 * then along r1 over the first result's columns) give a two-electron radial factor. The row
 * and its band must fit in shared memory (PG_ERR_SHAPE otherwise).
 */
int pg_bspline_band_project(pg_ctx *ctx, const double *F, long long nbatch, int bdiv, long long in_bstride,
                            long long in_qstride, int nint, int k, int q, const int *first, const double *B,
                            const double *w, int N, double *out, long long ob1, long long ob2, long long oi,
                            long long od);

/* ---------------------------------------------------------------------------------- */
/* analysis: projections on products of single-electron radial states                 */
/* ---------------------------------------------------------------------------------- */
/*
 * For the angular indices `angular` [nidx] (distinct) of a two-electron wavefunction
 * [nang][N1][N2] (complex128, device), with the radial states as columns of V1 [N1][n1] and
 * V2 [N2][n2] (complex128, host, row-major):
 *   pg_radial_products_project: proj[q][i1][i2] = sum_{r1,r2} conj(V1[r1][i1]) psi_w[a_q][r1][r2]
 *       conj(V2[r2][i2]) into the host array proj [nidx][n1][n2] (complex128)
 *       (CalculateProjectionRadialProductStates, examples/tensor/helium_stabilization/
 *       analysis.cpp:39-81);
 *   pg_radial_products_remove: the same projections of psi_w, then psi[a_q] -= V1 proj_q V2^T
 *       (RemoveProjectionRadialProductStates, analysis.cpp:91-121).
 * psi_w is the wavefunction with the integration weights (the overlap on both radial ranks)
 * applied, as the reference's callers pass it. Both wait for the context's stream.
 */
int pg_radial_products_project(pg_ctx *ctx, const void *psi_w, int nang, int N1, int N2, const int *angular, int nidx,
                               const double *V1, int n1, const double *V2, int n2, double *proj);
int pg_radial_products_remove(pg_ctx *ctx, const void *psi_w, void *psi, int nang, int N1, int N2, const int *angular,
                              int nidx, const double *V1, int n1, const double *V2, int n2);

/* ---------------------------------------------------------------------------------- */
/* allocation-free entry point                                                        */
/* ---------------------------------------------------------------------------------- */
/*
 * pg_vec_multidot_noalloc: the block inner product of the Krylov Gram-Schmidt step,
 *     out[2j], out[2j+1] = sum_i conj(V[j][i]) w[i]   (j < J, complex128 result)
 *     out[2J] = ||w||^2, out[2J+1] = ||w||
 * for complex128 (PG_FP64) or complex64 (PG_FP32) device vectors, written to the caller's
 * device buffer `out` (2J+2 doubles), on `stream` (NULL = legacy default stream). No
 * counterpart in the reference. It is for callers that cannot allocate device memory: a host
 * application whose own pool allocator has reserved the GPU's memory at start-up (a
 * cudaMalloc from the library would fail, or take memory the application budgets itself),
 * and steady-state stepping loops that must not pay cudaMalloc/cudaFree's implicit
 * device-wide synchronization, which stalls the other streams. It needs no pg_ctx and calls
 * no cudaMalloc, cudaFree or allocating library routine: its scratch (per-CTA partial sums
 * and the arrival ticket) is a static device array of about 320 KB that every GPU loading the
 * library keeps until the process exits, so J is limited to 64 vectors (PG_ERR_ARG above
 * that). The first call on a device looks up the array's address on that device
 * (cudaGetSymbolAddress) and keeps it for the life of the process: do not use this entry
 * point across cudaDeviceReset. Make that first call before any stream capture. All calls
 * share the one array and it keeps the last call's contents (the arrival ticket is cleared
 * at the start of every call): calls that overlap on the GPU (two streams, two threads)
 * race and give wrong sums - serialize them.
 */
int pg_vec_multidot_noalloc(int precision, const void *V, long long ldv, int J, const void *w,
                            long long n, double *out, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* PYPROP_GPU_H */
