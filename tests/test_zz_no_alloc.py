"""The allocation-free block inner product against the context-based entry point.

pg_vec_multidot_noalloc is for callers that cannot allocate device memory: an application
whose own pool allocator reserved the GPU's memory at start-up, or a stepping loop that must
not pay cudaMalloc's device-wide synchronization. It keeps its scratch in a static device
array instead. This file sorts last so that a run stopping at the first failure has already
run every other test; it also passes alone in a fresh process, because the first call looks
up the array's address itself.
"""
import ctypes as C

import numpy as np
import pytest

from pyprop_gb300 import _native as nat

pytestmark = pytest.mark.gpu


def test_multidot_noalloc_matches_vec_dot(gpu):
    """Two calls in a row per precision (the second reuses the array the first left behind):
    each sum equals the existing entry point's (pg_vec_dot) and numpy's, to 1e-13 relative in
    complex128 and 1e-5 in complex64 (FP32 element products, FP64 sums)."""
    import torch
    from pyprop_gb300.gpu import Context, ptr, vec_dot

    lib = nat.load()
    ctx = Context.get()
    rng = np.random.default_rng(31)
    cases = [(nat.PG_FP64, 5, 24600, 1e-13), (nat.PG_FP64, 9, 1650, 1e-13),
             (nat.PG_FP32, 7, 24600, 1e-5), (nat.PG_FP32, 20, 5000, 1e-5)]
    for call, (prec, J, n, tol) in enumerate(cases):
        dtype = torch.complex128 if prec == nat.PG_FP64 else torch.complex64
        V = rng.normal(size=(J, n)) + 1j * rng.normal(size=(J, n))
        w = rng.normal(size=n) + 1j * rng.normal(size=n)
        dV = torch.as_tensor(V, device="cuda").to(dtype)
        dw = torch.as_tensor(w, device="cuda").to(dtype)
        Vh = dV.cpu().numpy().astype(np.complex128)  # the values the GPU sees
        wh = dw.cpu().numpy().astype(np.complex128)
        out = torch.full((2 * J + 2,), np.nan, dtype=torch.float64, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        rc = lib.pg_vec_multidot_noalloc(prec, ptr(dV), n, J, ptr(dw), n, ptr(out), C.c_void_p(stream))
        assert rc == 0, lib.pg_error_string(rc)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        scale = np.linalg.norm(Vh, axis=1) * np.linalg.norm(wh)
        for j in range(J):
            val = complex(got[2 * j], got[2 * j + 1])
            ref = vec_dot(ctx, dV[j], dw, prec)    # the existing entry point (pg_vec_dot)
            assert abs(val - ref) <= tol * scale[j], (call, j)
            assert abs(val - np.vdot(Vh[j], wh)) <= tol * scale[j], (call, j)
        nrm2 = float(np.vdot(wh, wh).real)
        assert abs(got[2 * J] - vec_dot(ctx, dw, dw, prec).real) <= tol * nrm2
        assert abs(got[2 * J] - nrm2) <= tol * nrm2
        assert abs(got[2 * J + 1] - np.sqrt(nrm2)) <= tol * np.sqrt(nrm2)


def test_multidot_noalloc_rejects_too_many_vectors(gpu):
    import torch
    from pyprop_gb300.gpu import ptr
    lib = nat.load()
    dw = torch.zeros(8, dtype=torch.complex128, device="cuda")
    out = torch.zeros(200, dtype=torch.float64, device="cuda")
    assert lib.pg_vec_multidot_noalloc(nat.PG_FP64, ptr(dw), 8, 65, ptr(dw), 8, ptr(out), None) == -1
