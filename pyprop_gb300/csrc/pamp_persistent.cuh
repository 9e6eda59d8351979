// The persistent pAMP ensemble step: one launch advances every member of an ensemble by one
// pAMP step. Each CTA takes members from a device work list (a queue counter over members
// sorted by size, largest first) and runs a member's whole step by itself: psi <- U psi, the
// m Arnoldi steps on U^-H H(t) U^-1 (complex64 basis, classical Gram-Schmidt with a second
// pass through the Gram matrix, FP64 CTA sums), the m x m exponential (pamp_expm_block) and
// psi = ||psi|| U^-1 V c (as the combination of the U^-1 V[j] the Arnoldi steps computed) -
// the same algorithm, layout and Hessenberg columns as the graph of per-member kernels in
// krylov.cu, with no wait between CTAs. krylov.cu fills one PmMember per member from its
// pg_pamp; pamp_persistent.cu holds the kernel, its launcher and the autotuned shape.
#pragma once
#include "pg_internal.cuh"
#include "pamp_expm.cuh"

struct PmMember {
    int nch = 0, N = 0, ld = 0, kb = 0, m = 0, double_ortho = 1, nent = 0;
    long long n = 0;                          // nch * N
    const int *row_ptr = nullptr, *ent_col = nullptr, *ent_band = nullptr, *ent_slot = nullptr;
    const float *bands = nullptr;             // real FP32 bands [nbands][2kb+1][ld]
    const float *U32 = nullptr;               // overlap Cholesky factor U(i, i+d) at [i][d], FP32
    const double *U64 = nullptr;              // the same in FP64
    cxf *V = nullptr, *w = nullptr;           // basis [m][n]; scratch [n]
    cxf *T = nullptr;                         // t_j = U^-1 V[j] of every Arnoldi step [m][n]
    cxd *psi = nullptr;                       // the member's wavefunction (complex128)
    const cxd *scales = nullptr;              // its slot values [PG_MAX_SLOTS]
    double *cols = nullptr;                   // Hessenberg columns [m][3][2(m+2)] (ArnoldiBuf layout)
    double *norm = nullptr;                   // out: ||U psi||^2, ||U psi||
    // nbasis > 0: the operator's bands are combinations of nbasis basis bands (basis [k][2kb+1][N],
    // FP32), and row_ptr / ent_col / ent_band / ent_slot / ent_coef describe terms (column, basis
    // band, slot, coefficient) instead of entries; the basis bands are staged in shared memory
    int nbasis = 0;
    const float *basis = nullptr;
    const float *ent_coef = nullptr;
    const float *G32u = nullptr, *G32l = nullptr;  // chunk responses of the FP32 solves (32-row chunks)
    PampExpArgs ex;                           // the exponential's arguments (cols, norm, c, stats)
};

// real FP32 copy of an operator's bands in its device layout; PG_ERR_STORAGE when a band has a
// non-zero imaginary part
int pm_real_bands(const pg_op *op, float **dev);

// The operator as terms over at most pm_max_basis_bands() basis bands, when its bands allow it
// (each a multiple of one basis band, or, for the blocks on the diagonal, of A + alpha D for a
// common A and D: a per-channel field-free band plus a multiple of the centrifugal one); fills
// M's term arrays and basis (appended to allocs) and sets M.nbasis, else leaves M.nbasis 0
int pm_member_basis(const pg_op *op, PmMember &M, std::vector<void *> &allocs);
int pm_max_basis_bands();

// the chunk tables of the member's banded solves and its scratch (from M.U64, M.N, M.kb, M.nch);
// the device allocations are appended to allocs (the caller frees them)
int pm_member_tables(PmMember &M, std::vector<void *> &allocs);

// the largest dynamic shared memory a launch for these members needs
size_t pm_smem_bytes(int Nmax, int kbmax, int mmax, int nchmax, int entmax, int basismax);

// one ensemble step: queue (device counter) cleared, then `grid` CTAs of `threads` threads;
// Nmax, kbmax, mmax, nchmax, entmax: the members' largest radial size, band half-width, basis
// size, channel count and operator-entry count
// wide: the instance bounded at 256 threads (all registers it wants), else at 512
int pm_launch(const PmMember *d_members, int nmembers, const int *d_order, unsigned *d_queue, const double *d_dt,
              int threads, int grid, size_t smem, bool kb6, bool wide, cudaStream_t s, int Nmax, int kbmax, int mmax,
              int nchmax, int entmax, int basismax);

// limits of the kernel: Krylov basis size and band half-width
int pm_max_basis();
int pm_max_halfwidth();

// CTAs of `threads` threads resident per SM with `smem` bytes (0 when the shape does not fit)
int pm_occupancy(int threads, size_t smem, bool kb6, bool wide);
