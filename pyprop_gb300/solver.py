"""``PiramSolverGPU``: implicitly restarted Arnoldi for the lowest eigenpairs of S^-1 H.

The Arnoldi expansion (operator, CGS2, norms) runs on the GPU through
``pg_arnoldi_expand``; the restart bookkeeping on the m x m Hessenberg matrix runs on the
host in FP64, as in the reference where it is LAPACK work
(``core/krylov/piram/piram/piram.h``: ``UpdateEigenvalues`` :473-535 with Ritz error bounds
and the ARPACK-style test ``bound <= tol * max(eps^(2/3), tol |theta|)``,
``PerformRestartStep`` :537-655 with exact shifts, ``Solve`` :698-753). Eigenvalues are
ordered by real part (``CompareComplexLessReal``), or by decreasing modulus in the
shift-invert mode (``inverse_iterations``, piramsolver.cpp:79-90); the unwanted ones,
sorted by their error bounds, are the shifts. When an invariant subspace is found
(||f|| < 1e-14 max|H|, e.g. H block diagonal in l) a random vector continues the
factorization with a zero subdiagonal entry - the reference would divide by zero there. Config keys follow ``pyprop/solver/PiramSolver.py``
([Arpack]: krylov_basis_size, krylov_eigenvalue_count, krylov_tolerance,
krylov_max_iteration_count, krylov_use_random_start).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as nat
from ._native import check
from .gpu import Banded, Context, ptr, torch


def _sort_real(values):
    """Stable exchange sort by real part, as ``ShiftFunctorSelectRitzValues`` does."""
    vals = list(values)
    order = list(range(len(vals)))
    n = len(vals)
    for i in range(n):
        for j in range(i + 1, n):
            if not (vals[i].real < vals[j].real):
                vals[i], vals[j] = vals[j], vals[i]
                order[i], order[j] = order[j], order[i]
    return np.array(vals), np.array(order)


def _sort_abs_desc(values):
    """Exchange sort, largest |theta| first (``CompareComplexGreaterAbs``)."""
    vals = list(values)
    order = list(range(len(vals)))
    n = len(vals)
    for i in range(n):
        for j in range(i + 1, n):
            if not (abs(vals[i]) > abs(vals[j])):
                vals[i], vals[j] = vals[j], vals[i]
                order[i], order[j] = order[j], order[i]
    return np.array(vals), np.array(order)


class PiramSolverGPU:
    def __init__(self, prop, start_vector=None, seed=None):
        self.BaseProblem = prop
        conf = prop.Config.Arpack
        self.BasisSize = int(conf.krylov_basis_size)
        self.EigenvalueCount = int(conf.krylov_eigenvalue_count)
        self.MaxRestartCount = int(conf.krylov_max_iteration_count)
        eps = np.finfo(float).eps
        self.Tolerance = max(float(getattr(conf, "krylov_tolerance", 0.0) or 0.0), eps)
        self.UseRandomStart = bool(getattr(conf, "krylov_use_random_start", True))
        if 2 * self.EigenvalueCount > self.BasisSize:
            raise ValueError("Basis size too small. should be at least 2*EigenvalueCount")
        self.start_vector = start_vector
        self.seed = seed
        self._rng = np.random.default_rng(12345 if seed is None else seed + 1)
        self.InverseIterations = bool(getattr(conf, "inverse_iterations", False))
        self.Shift = complex(getattr(conf, "krylov_eigenvalue_shift", 0.0))
        self.Stats = nat.KrylovStats()

    # operator S^-1 H at t = 0 (PiramSolver.py: ApplyMatrix(psi, tmp, 0, 0)), or the
    # shift-invert operator (H0 - sigma S)^-1 S when [Arpack] inverse_iterations is set
    def _setup_operator(self):
        bp = self.BaseProblem.Propagator.BasePropagator
        if not hasattr(bp, "_ops"):
            bp.SetupStep(0.0)
        self.op = bp.device_operator(nat.PG_FP64)
        repr_ = self.BaseProblem.psi.GetRepresentation()
        self.ovl = Banded.overlap(self.op, repr_.overlap_rows)
        self.scales = np.ascontiguousarray(self.op.scales(0.0), dtype=np.complex128)
        self.shift_invert = None
        if self.InverseIterations:
            # H at t = 0 must be diagonal in the angular rank for the exact block solve
            slots, weights = [], []
            for p, pot in enumerate(bp.PotentialList):
                ids = [g.GetStorageId() for g in pot.GeometryList]
                scale = pot.GetTimeScaling(0.0)
                if any(i != "Diag" for i in ids[:-1]):
                    if scale != 0.0:
                        raise ValueError("shift-invert pIRAM needs H(0) diagonal in the angular rank")
                    continue
                slots.append(1 + p)
                weights.append(scale)
            self.shift_invert = Banded.blockdiag(self.op, repr_.overlap_rows, -self.Shift, 1.0, slots, weights)

    def _expand(self, j0):
        lib = self.op.lib
        m = self.BasisSize
        inject = 0
        while True:
            Hf = self.H.view(np.float64)
            res = C.c_double(0.0)
            done = C.c_int(0)
            sc = self.scales.view(np.float64)
            tol = 1e-14 * max(float(np.max(np.abs(self.H))), 1e-300)
            self.op.ctx.bind_stream()
            check(lib.pg_arnoldi_expand(self.op.h, self.ovl.h, self.shift_invert.h if self.shift_invert else None,
                                        sc.ctypes.data_as(nat._DP), len(self.scales), ptr(self.V), m, j0,
                                        ptr(self.f), Hf.ctypes.data_as(nat._DP), tol, inject, C.byref(done),
                                        C.byref(res), C.byref(self.Stats)), "pg_arnoldi_expand")
            self.ResidualNorm = res.value
            if done.value >= m:
                return
            # invariant subspace found: continue from a random vector (made orthogonal on the device)
            t = torch()
            rnd = self._rng.uniform(-1.0, 1.0, self.f.numel()).astype(np.complex128)
            self.f.copy_(t.as_tensor(rnd, device="cuda"))
            j0 = done.value - 1
            inject = 1

    def Solve(self):
        t = torch()
        self._setup_operator()
        m, k = self.BasisSize, self.EigenvalueCount
        shape = self.BaseProblem.psi.GetData().shape
        n = int(np.prod(shape))
        self.V = t.zeros((m, n), dtype=t.complex128, device="cuda")
        if self.UseRandomStart:
            rng = np.random.default_rng(self.seed)
            start = rng.uniform(0.0, 1.0, n).astype(np.complex128)
        else:
            start = np.asarray(self.start_vector if self.start_vector is not None
                               else self.BaseProblem.psi.numpy().ravel(), dtype=np.complex128)
        self.f = t.as_tensor(start, device="cuda").clone()
        self.H = np.zeros((m, m), dtype=np.complex128)
        self.RestartCount = 0
        self._expand(-1)
        eps = np.finfo(float).eps
        eps23 = eps ** (2.0 / 3.0)
        while True:
            evals, evecs = np.linalg.eig(self.H)
            sorted_vals, order = _sort_abs_desc(evals) if self.InverseIterations else _sort_real(evals)
            bounds = np.abs(evecs[m - 1, :]) * self.ResidualNorm
            shift_idx = order[k:]
            shift_order = np.argsort(bounds[shift_idx], kind="stable")
            shifts = evals[shift_idx][shift_order]
            conv = []
            for i in range(k):
                b = abs(evecs[m - 1, order[i]]) * self.ResidualNorm
                acc = self.Tolerance * max(eps23, self.Tolerance * abs(sorted_vals[i]))
                conv.append(b - acc)
            self.Eigenvalues = sorted_vals
            self.Order = order
            self.HessenbergEigenvectors = evecs
            self.ConvergenceEstimates = np.array(conv)
            self.IsConverged = bool(np.all(self.ConvergenceEstimates <= 0.0))
            if self.IsConverged or self.RestartCount >= self.MaxRestartCount:
                break
            self._restart(shifts)
            self._expand(k - 1)
        self.Stats.RestartCount = self.RestartCount
        # eigenvectors Y = V X (wanted ones in sorted order)
        X = evecs[:, order[:k]]
        Xc = np.ascontiguousarray(X, dtype=np.complex128)
        check(self.op.lib.pg_vec_combine(self.op.ctx.h, ptr(self.V), n, m, Xc.view(np.float64).ctypes.data_as(nat._DP),
                                         k), "pg_vec_combine")
        self.Eigenvectors = self.V[:k].reshape((k,) + tuple(shape))

    def _restart(self, shifts):
        m, k = self.BasisSize, self.EigenvalueCount
        H = self.H.copy()
        Q = np.eye(m, dtype=np.complex128)
        for mu in shifts:
            Qi, R = np.linalg.qr(H - mu * np.eye(m))
            H = R @ Qi + mu * np.eye(m)
            Q = Q @ Qi
        sigma = Q[m - 1, k - 1]
        beta = H[k, k - 1]
        Qk = np.ascontiguousarray(Q[:, :k + 1], dtype=np.complex128)
        check(self.op.lib.pg_vec_combine(self.op.ctx.h, ptr(self.V), self.V.shape[1], m,
                                         Qk.view(np.float64).ctypes.data_as(nat._DP), k + 1), "pg_vec_combine")
        # f <- sigma f + beta V[k]
        self.f.mul_(complex(sigma)).add_(self.V[k], alpha=complex(beta))
        H[:, k:] = 0.0
        H[k:, :] = 0.0
        self.H = np.ascontiguousarray(H)
        self.RestartCount += 1

    def GetEigenvalues(self):
        """Real parts of the wanted eigenvalues of S^-1 H (shift-invert values mapped back
        through lambda = sigma + 1/theta)."""
        vals = self.Eigenvalues[: self.EigenvalueCount]
        if self.InverseIterations:
            vals = self.Shift + 1.0 / vals
        return np.real(vals).copy()

    def GetEigenvector(self, index):
        return self.Eigenvectors[index]

    def SetEigenvector(self, psi, index, normalize=True):
        psi.GetData().copy_(self.Eigenvectors[index])
        if normalize:
            psi.Normalize()

    def GetConvergenceEstimates(self):
        return self.ConvergenceEstimates


PiramSolver = PiramSolverGPU
