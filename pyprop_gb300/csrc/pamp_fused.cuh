// The single-kernel mixed-precision pAMP step (pamp_fused.cu) as krylov.cu drives it.
#pragma once
#include "pg_internal.cuh"

struct FusedPamp;

// Tables and scratch of the single-kernel step for a complex64-basis pAMP stepper whose
// operator opb (FP32, rank 2, real bands) and overlaps qualify; T: the stepper's [m][n]
// complex64 basis buffer (the kernel keeps T_j = U^-1 V_j there). PG_ERR_STORAGE / SHAPE when
// the stepper does not qualify.
int pg_pamp_fused_prepare(pg_op *opb, pg_banded *ovl64, pg_banded *ovlb, void *T, int m, double tol,
                          FusedPamp **out);
// One step of psi (complex128, device) with H frozen at the slot values h[PG_MAX_SLOTS];
// ex (device, 4 doubles): basis size, error estimate, singular flag, sticky singular flag.
int pg_pamp_fused_launch(FusedPamp *f, cudaStream_t s, cxd *psi, double dt, const cxd *h, double *ex, int *err);
void pg_pamp_fused_set_probe(FusedPamp *f, unsigned int extra_arrivals, unsigned int at_barrier);
void pg_pamp_fused_free(FusedPamp *f);
