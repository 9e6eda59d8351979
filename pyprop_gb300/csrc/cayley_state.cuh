// Device state shared by the Cayley step drivers: the captured multi-kernel step (cayley.cu)
// and the single-kernel step (cayley_fused.cu).
#pragma once
#include "pg_internal.cuh"

static const int GM_MAXM = 64;

struct GmresStats {
    long long iterations;  // GMRES iterations of the step (all refinement passes)
    int k;                 // basis vectors used by the last solve
    int passes;            // refinement passes (mixed) / 1
    double resid;          // least-squares residual estimate of the last solve
    double true_resid;     // ||(S + i dt/2 H) psi' - b|| in FP64 (mixed; FP64 mode when requested)
    double beta0;          // norm of the preconditioned right-hand side of the last solve
    long long kernels;     // kernels run by all steps so far (never reset; see the K_* counts)
    long long rejected;    // learned-preconditioner passes rejected by the true residual (cumulative)
    long long cum_iterations;  // GMRES iterations of all steps so far (never reset)
    long long cum_passes;      // refinement passes of all steps so far (never reset)
};

struct GmresState {
    GmresStats stats;
    int j;            // Krylov vector being expanded in this iteration
    int cont_inner;   // loop decisions, mirrored for the eager (host-driven) mode
    int cont_outer;
    int learned_on;   // learned preconditioner in use for the rest of this step
    int accept;       // the last learned pass met the residual test
    int pad;
    double tol_eff;
    double beta_last;
    double cs[GM_MAXM];
    double sn[2 * GM_MAXM];
    double g[2 * (GM_MAXM + 1)];
    double R[2 * GM_MAXM * GM_MAXM];  // column-major R[col * GM_MAXM + row]
    double y[2 * GM_MAXM];
};

struct StepParams {
    double dt;
    double pad;
    cxd h[PG_MAX_SLOTS];  // slot values of H(t + dt/2); slot 0 is the overlap slot
};

// scale sets derived on the device from StepParams
enum { SC_PLUS = 0, SC_MINUS = 1, SC_DIFF = 2, SC_NEGPLUS = 3, SC_COUNT = 4 };

// Single-kernel mixed-precision step (cayley_fused.cu) for a rank-2 banded operator with the
// block-diagonal LU preconditioner: one cooperative launch of one CTA per angular channel.
struct FusedCayley;
// PG_OK and *out set when the operators qualify; an error code (and *out null) otherwise
int pg_cayley_fused_prepare(pg_op *op64, pg_op *opb, pg_banded *precb, int m, FusedCayley **out);
// one step on stream s: psi (complex128, device) advanced in place; st->stats updated. The
// step's parameters travel as kernel arguments; host_stats / host_err (device-visible aliases
// of mapped host memory, or null) receive the step's statistics and the error word from the
// kernel itself, so a step is one memset and one launch on the stream.
int pg_cayley_fused_launch(FusedCayley *f, cudaStream_t s, const StepParams &params, cxd *psi, GmresState *st,
                           double tol, int *err, GmresStats *host_stats, int *host_err);
void pg_cayley_fused_free(FusedCayley *f);
// 0: three CTAs per channel (a thread-block cluster) where the operator's shape fits, else
// one CTA per channel; 1: one CTA per channel; 2: the cluster variant (PG_ERR_SHAPE if it
// does not fit). pg_cayley_fused_which: the one selected (1 or 2).
int pg_cayley_fused_select(FusedCayley *f, int variant);
int pg_cayley_fused_which(const FusedCayley *f);
// test hook: arrivals that grid barrier number at_barrier (0 = the first of a step) of each
// later step waits for in addition, which no CTA makes (0: none)
void pg_cayley_fused_set_probe(FusedCayley *f, unsigned int extra_arrivals, unsigned int at_barrier);
