"""The reference's own Krylov templates, called from Python - TEST INFRASTRUCTURE ONLY.

``oracle/_ref/libref_krylov.so`` (built by ``oracle/ref/build_ref.py`` from the PyProp source
tree, where that tree is present) holds pAMP, GMRES and pIRAM exactly as the reference
compiles them (core/krylov/pamp/pamp/pamp.h, core/krylov/gmres/gmres.h,
core/krylov/piram/piram/piram.h) and a restatement of the generated
TensorPotentialMultiply_{Diag,Simp}_BandNH kernels over BLAS zgbmv. The classes below drive
them as the reference's Python layer does:

* ``RefHamiltonian.apply_H``: BasisPropagator.MultiplyPotential over every consolidated
  potential (TensorPotential.py:92-112), each a zgbmv per angular pair.
* ``RefPam.step``: PamPropagator.AdvanceStep with the balanced overlap
  (PamPropagator.py:50-75, BasisPropagator.py:131-159) around pAMP<cplx>::PropagateVector.
* ``RefCayley.step``: CayleyPropagator.AdvanceStep (CayleyPropagator.py:71-150) around
  GMRES<cplx>::SolveVector, left-preconditioned by the block-diagonal banded LU.

The overlap Cholesky transforms and the banded LU preconditioner come from ``operators``
(LAPACK band routines through scipy, as the reference calls zpbtrf/ztbsv and zgbtrf/zgbtrs).
These check the numpy restatement in ``krylov``/``propagators``; nothing in the package
imports them.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

LIB = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_ref", "libref_krylov.so")
APPLY = C.CFUNCTYPE(None, C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int)
_D = C.POINTER(C.c_double)
_lib = None


def available():
    return os.path.exists(LIB)


def load():
    global _lib
    if _lib is None:
        lib = C.CDLL(LIB)
        lib.ref_pamp_new.restype = C.c_void_p
        lib.ref_pamp_new.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, APPLY, C.c_void_p]
        lib.ref_pamp_propagate.argtypes = [C.c_void_p, _D, C.c_double, C.c_double, _D, C.POINTER(C.c_int)]
        lib.ref_pamp_free.argtypes = [C.c_void_p]
        lib.ref_gmres_new.restype = C.c_void_p
        lib.ref_gmres_new.argtypes = [C.c_int, C.c_int, C.c_double, APPLY, C.c_void_p]
        lib.ref_gmres_solve.argtypes = [C.c_void_p, _D, _D, _D, C.POINTER(C.c_int)]
        lib.ref_gmres_free.argtypes = [C.c_void_p]
        lib.ref_piram_solve.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, _D, APPLY,
                                        C.c_void_p, _D, _D, _D, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        lib.ref_multiply_bandnh.argtypes = [_D, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), C.c_double, _D, _D]
        _lib = lib
    return _lib


def _ptr(a):
    return a.ctypes.data_as(_D)


def _callback(op):
    """APPLY wrapper of op(v: complex128 [n]) -> complex128 [n]."""

    def fn(_user, pin, pout, n):
        x = np.ctypeslib.as_array(pin, shape=(2 * n,)).view(np.complex128)
        y = np.ctypeslib.as_array(pout, shape=(2 * n,)).view(np.complex128)
        y[:] = op(x.copy())

    return APPLY(fn)


class RefPampPropagator:
    """pamp::pAMP<cplx> of size n with basis m and the operator op."""

    def __init__(self, n, m, op, double_ortho=True, exponentiation=0):
        self.lib = load()
        self.n = n
        self._cb = _callback(op)
        self.h = self.lib.ref_pamp_new(n, m, int(bool(double_ortho)), exponentiation, self._cb, None)
        if not self.h:
            raise RuntimeError("ref_pamp_new failed")

    def propagate(self, v, dt):
        """exp(-i dt A) v; returns (vector, error estimate, operator count)."""
        out = np.ascontiguousarray(v, dtype=np.complex128).copy()
        err, ops = C.c_double(), C.c_int()
        dt = complex(dt)
        rc = self.lib.ref_pamp_propagate(self.h, _ptr(out.view(np.float64)), dt.real, dt.imag, C.byref(err),
                                         C.byref(ops))
        if rc != 0:
            raise RuntimeError("ref_pamp_propagate: %d" % rc)
        return out, err.value, ops.value

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.ref_pamp_free(self.h)
            self.h = None


class RefGmresSolver:
    """gmres::GMRES<cplx> of size n with basis m, tolerance tol and the operator op."""

    def __init__(self, n, m, tol, op):
        self.lib = load()
        self.n = n
        self._cb = _callback(op)
        self.h = self.lib.ref_gmres_new(n, m, float(tol), self._cb, None)
        if not self.h:
            raise RuntimeError("ref_gmres_new failed")

    def solve(self, b):
        """x with A x = b from x0 = 0; returns (x, error estimate, operator count)."""
        rhs = np.ascontiguousarray(b, dtype=np.complex128).copy()
        x = np.zeros_like(rhs)
        err, ops = C.c_double(), C.c_int()
        rc = self.lib.ref_gmres_solve(self.h, _ptr(rhs.view(np.float64)), _ptr(x.view(np.float64)), C.byref(err),
                                      C.byref(ops))
        if rc != 0:
            raise RuntimeError("ref_gmres_solve: %d" % rc)
        return x, err.value, ops.value

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.ref_gmres_free(self.h)
            self.h = None


def ref_piram(op, start, m, k, tol=0.0, max_restarts=10, largest_abs=False):
    """piram::pIRAM<cplx>: (eigenvalues [k], eigenvectors [k][n], convergence estimates [k],
    restarts, operator count). largest_abs selects the inverse-iteration ordering."""
    lib = load()
    start = np.ascontiguousarray(start, dtype=np.complex128)
    n = start.size
    evals = np.zeros(k, np.complex128)
    evecs = np.zeros((k, n), np.complex128)
    conv = np.zeros(k)
    restarts, ops = C.c_int(), C.c_int()
    cb = _callback(op)
    rc = lib.ref_piram_solve(n, m, k, float(tol), int(max_restarts), 1 if largest_abs else 0,
                             _ptr(start.view(np.float64)), cb, None, _ptr(evals.view(np.float64)),
                             _ptr(evecs.view(np.float64)), _ptr(conv), C.byref(restarts), C.byref(ops))
    if rc != 0:
        raise RuntimeError("ref_piram_solve: %d" % rc)
    return evals, evecs, conv, restarts.value, ops.value


def ref_multiply_bandnh(potential, pairs, N, b, scaling, src, dest):
    """dest += scaling * V src for a rank-2 Diag (pairs None) or Simp BandNH potential."""
    lib = load()
    pot = np.ascontiguousarray(potential, dtype=np.complex128)
    npairs = pot.shape[0] if pot.ndim == 2 else pot.size // (N * b)
    src = np.ascontiguousarray(src, dtype=np.complex128)
    assert dest.flags.c_contiguous and dest.dtype == np.complex128
    pp = None
    if pairs is not None:
        pr = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1, 2)
        assert len(pr) == npairs
        pp = pr.ctypes.data_as(C.POINTER(C.c_int))
    rc = lib.ref_multiply_bandnh(_ptr(pot.view(np.float64)), npairs, N, b, pp, float(scaling),
                                 _ptr(src.view(np.float64)), _ptr(dest.view(np.float64)))
    if rc != 0:
        raise RuntimeError("ref_multiply_bandnh: %d" % rc)
    return pairs


class RefHamiltonian:
    """H(t) psi of a rank-2 (Nang x N) model from its consolidated potentials in the
    reference layout: terms as (storage id, PotentialData, pairs, time function), every
    storage Diag_BandNH or Simp_BandNH."""

    def __init__(self, terms, nang, N, kb):
        self.nang, self.N, self.b = nang, N, 2 * kb + 1
        self.terms = []
        for storage, data, pairs, tf in terms:
            if storage not in ("Diag_BandNH", "Simp_BandNH"):
                raise ValueError("storage %s is not a rank-2 BandNH storage" % storage)
            self.terms.append((np.ascontiguousarray(np.asarray(data, np.complex128).reshape(-1, N * self.b)),
                               None if storage == "Diag_BandNH" else pairs, tf))

    def apply_H(self, psi, t):
        out = np.zeros((self.nang, self.N), np.complex128)
        src = np.ascontiguousarray(psi, np.complex128).reshape(self.nang, self.N)
        for data, pairs, tf in self.terms:
            s = 1.0 if tf is None else float(tf(t))
            ref_multiply_bandnh(data, pairs, self.N, self.b, s, src, out)
        return out


class RefPam:
    """PamPropagator.AdvanceStep with the balanced overlap around the reference's pAMP."""

    def __init__(self, ham: RefHamiltonian, overlap, basis_size=20, double_ortho=True):
        self.ham, self.ovl = ham, overlap
        self.shape = (ham.nang, ham.N)
        self.t = 0.0

        def op(v):
            u = self.ovl.solve_sqrt(v.reshape(self.shape), conj=False)
            return self.ovl.solve_sqrt(self.ham.apply_H(u, self.t), conj=True).ravel()

        self.pamp = RefPampPropagator(ham.nang * ham.N, basis_size, op, double_ortho)

    def step(self, psi, t, dt):
        self.t = t
        x = self.ovl.multiply_sqrt(psi, conj=False)
        y, self.last_error, _ = self.pamp.propagate(x.ravel(), dt)
        return self.ovl.solve_sqrt(y.reshape(self.shape), conj=False)


class RefCayley:
    """CayleyPropagator.AdvanceStep around the reference's GMRES; prec is the block-diagonal
    preconditioner (an object with solve(psi) -> M^-1 psi)."""

    def __init__(self, ham: RefHamiltonian, overlap, prec, basis_size=20, tolerance=0.0):
        self.ham, self.ovl, self.prec = ham, overlap, prec
        self.shape = (ham.nang, ham.N)
        self.h_factor, self.tt = 0.0, 0.0

        def op(v):
            v = v.reshape(self.shape)
            return self.prec.solve(self.ovl.multiply(v) + self.h_factor * self.ham.apply_H(v, self.tt)).ravel()

        self.gmres = RefGmresSolver(ham.nang * ham.N, basis_size, tolerance, op)

    def step(self, psi, t, dt):
        self.tt = t + abs(dt / 2.0)
        b = self.ovl.multiply(psi) - 1j * dt / 2.0 * self.ham.apply_H(psi, self.tt)
        self.h_factor = 1j * dt / 2.0
        x, self.last_error, self.last_iterations = self.gmres.solve(self.prec.solve(b).ravel())
        return x.reshape(self.shape)
