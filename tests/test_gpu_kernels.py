"""GPU parity of the matvec and banded kernels against the oracle (through the C ABI)."""
import ctypes as C

import numpy as np
import pytest

from pyprop_gb300 import _native as nat
from tests.helpers import golden, hydrogen_problem, oracle_hamiltonian, relerr

pytestmark = pytest.mark.gpu


def _torch():
    import torch
    return torch


def _dev(a, dtype=None):
    t = _torch()
    return t.as_tensor(np.ascontiguousarray(a), device="cuda", dtype=dtype or t.complex128)


def _setup(lmax=3, N=40, rmax=40.0):
    prob = hydrogen_problem(lmax=lmax, nbsplines=N, rmax=rmax)
    ham = oracle_hamiltonian(prob)
    return prob, ham


def test_reference_layout_kernels(gpu):
    """pg_tensor_multiply_{diag,simp,ident}_bandnh vs the oracle's per-pair band products."""
    t = _torch()
    prob, ham = _setup()
    lib = nat.load()
    bp = prob.Propagator.BasePropagator
    nang, N = prob.psi.GetRepresentation().GetFullShape()
    rng = np.random.default_rng(5)
    src = rng.normal(size=(nang, N)) + 1j * rng.normal(size=(nang, N))
    for pot, term in zip(bp.PotentialList, ham.terms):
        ids = "_".join(g.GetStorageId() for g in pot.GeometryList)
        dst0 = rng.normal(size=(nang, N)) + 1j * rng.normal(size=(nang, N))
        ref = dst0.copy()
        term.multiply(src, ref, 0.37)
        d_pot, d_src, d_dst = _dev(pot.PotentialData), _dev(src), _dev(dst0)
        e0, e1 = pot.PotentialData.shape
        args = (C.c_void_p(d_pot.data_ptr()), e0, e1, 0.37, C.c_void_p(d_src.data_ptr()), nang, N,
                C.c_void_p(d_dst.data_ptr()), nang, N)
        if ids == "Diag_BandNH":
            code = lib.pg_tensor_multiply_diag_bandnh(*args, 6, None)
        else:
            pairs = _dev(pot.GeometryList[0].GetBasisPairs(), t.int32)
            code = lib.pg_tensor_multiply_simp_bandnh(*args, C.c_void_p(pairs.data_ptr()), e0, 2, 6, None)
        assert code == 0
        t.cuda.synchronize()
        assert relerr(d_dst.cpu().numpy(), ref) < 1e-14
    # Ident storage: the overlap band applied to every channel
    ident = np.zeros((1, N * 13), dtype=np.complex128)
    from pyprop_gb300.gpu import bandnh_from_rows
    ident[0] = bandnh_from_rows(ham.overlap_rows, 6)
    d_pot, d_src, d_dst = _dev(ident), _dev(src), _dev(np.zeros((nang, N), complex))
    assert lib.pg_tensor_multiply_ident_bandnh(C.c_void_p(d_pot.data_ptr()), 1, N * 13, 1.0,
                                               C.c_void_p(d_src.data_ptr()), nang, N, C.c_void_p(d_dst.data_ptr()),
                                               nang, N, 6, None) == 0
    t.cuda.synchronize()
    assert relerr(d_dst.cpu().numpy(), ham.overlap.multiply(src)) < 1e-14
    # shape mismatch is an error, not a silent launch
    assert lib.pg_tensor_multiply_diag_bandnh(C.c_void_p(d_pot.data_ptr()), 1, N * 13, 1.0,
                                              C.c_void_p(d_src.data_ptr()), nang, N, C.c_void_p(d_dst.data_ptr()),
                                              nang, N, 6, None) == -4


@pytest.mark.parametrize("lmax,N", [(3, 40), (0, 20), (10, 150), (6, 37)])
def test_fused_operator_fp64_fp32(gpu, lmax, N):
    """All terms in one launch, FP64 (1e-14) and FP32 (2e-6) vs the oracle, with time scales."""
    t = _torch()
    prob, ham = _setup(lmax, N, 40.0 if N < 100 else 100.0)
    bp = prob.Propagator.BasePropagator
    bp.SetupStep(0.01)
    nang = lmax + 1
    rng = np.random.default_rng(7)
    src = rng.normal(size=(nang, N)) + 1j * rng.normal(size=(nang, N))
    tt = 3.3
    ref = ham.apply_H(src, tt)
    for prec, tol in [(nat.PG_FP64, 1e-14), (nat.PG_FP32, 2e-6)]:
        op = bp.device_operator(prec)
        dt = t.complex128 if prec == nat.PG_FP64 else t.complex64
        d_src = _dev(src, dt)
        d_dst = _dev(np.ones((nang, N), complex), dt)
        op.matvec(op.scales(tt), d_src, d_dst, accumulate=False)
        t.cuda.synchronize()
        assert relerr(d_dst.cpu().numpy(), ref) < tol
        # accumulate adds to dst
        op.matvec(op.scales(tt), d_src, d_dst, accumulate=True)
        t.cuda.synchronize()
        assert relerr(d_dst.cpu().numpy(), 2 * ref) < tol
    g = golden("hydrogen_small.npz") if (lmax, N) == (3, 40) else None
    if g is not None:
        op = bp.device_operator(nat.PG_FP64)
        d_src, d_dst = _dev(g["psi"]), _dev(np.zeros_like(g["psi"]))
        op.matvec(op.scales(float(g["t"])), d_src, d_dst)
        t.cuda.synchronize()
        assert relerr(d_dst.cpu().numpy(), g["Hpsi"]) < 1e-14


@pytest.mark.parametrize("lmax,N", [(3, 40), (10, 150), (2, 70)])
def test_overlap_and_preconditioner_solves(gpu, lmax, N):
    t = _torch()
    from pyprop_gb300.gpu import Banded
    from oracle.operators import BandLU
    prob, ham = _setup(lmax, N, 40.0 if N < 100 else 100.0)
    bp = prob.Propagator.BasePropagator
    bp.SetupStep(0.01)
    nang = lmax + 1
    rows = prob.psi.GetRepresentation().overlap_rows
    rng = np.random.default_rng(11)
    x = rng.normal(size=(nang, N)) + 1j * rng.normal(size=(nang, N))
    ovl = ham.overlap
    expect = {
        nat.PG_BAND_MUL_U: ovl.multiply_sqrt(x, False), nat.PG_BAND_MUL_UT: ovl.multiply_sqrt(x, True),
        nat.PG_BAND_SOLVE_U: ovl.solve_sqrt(x, False), nat.PG_BAND_SOLVE_UT: ovl.solve_sqrt(x, True),
        nat.PG_BAND_MUL_S: ovl.multiply(x), nat.PG_BAND_SOLVE_S: ovl.solve(x),
    }
    dt = 0.01
    lu = BandLU(rows, [ham.terms[0]], nang, N, ham.kb, 1.0, 0.5j * dt)
    for prec, tol in [(nat.PG_FP64, 1e-12), (nat.PG_FP32, 5e-5)]:
        op = bp.device_operator(prec)
        cdt = t.complex128 if prec == nat.PG_FP64 else t.complex64
        b = Banded.overlap(op, rows)
        for which, ref in expect.items():
            d = _dev(x, cdt)
            b.apply(which, d)
            t.cuda.synchronize()
            assert relerr(d.cpu().numpy(), ref) < tol, which
        pre = Banded.blockdiag(op, rows, 1.0, 0.5j * dt, [1], [1.0])
        d = _dev(x, cdt)
        pre.apply(nat.PG_BAND_PREC_SOLVE, d)
        t.cuda.synchronize()
        assert relerr(d.cpu().numpy(), lu.solve(x)) < tol
