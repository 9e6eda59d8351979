"""Oracle propagation steps (complex128, CPU) - test infrastructure only.

* ``OraclePam.step``: PamPropagator.AdvanceStep with the balanced overlap
  (pyprop/propagator/PamPropagator.py:50-75, BasisPropagator.py:131-159): psi <- U psi,
  pAMP on U^-H H(t) U^-1 with H frozen at t (pampwrapper.cpp:84-92), psi <- U^-1 psi.
* ``OracleCayley.step``: CayleyPropagator.AdvanceStep (CayleyPropagator.py:71-150):
  b = M^-1 (S - i dt/2 H) psi with H at t + |dt|/2, GMRES on M^-1 (S + i dt/2 H), the
  block-diagonal banded LU M (BSplinePreconditioner) as left preconditioner.
* ``energy``: Problem.GetEnergyExpectationValue (pyprop/Problem.py:257-279).

Terms are given in the reference layout (PotentialData, storage id, pairs, time function).
"""
from __future__ import annotations

import numpy as np

from .krylov import gmres_solve, pamp_propagate
from .operators import BandLU, Overlap, TermOracle


class OracleHamiltonian:
    def __init__(self, terms, overlap_rows, nang, N):
        """terms: list of (storage_id, PotentialData, pairs or None, time_function or None)."""
        self.nang, self.N = nang, N
        rows = np.asarray(overlap_rows)
        self.kb = (rows.shape[1] - 1) // 2
        self.terms = [TermOracle(s, d, p, nang, N, self.kb, tf) for (s, d, p, tf) in terms]
        self.overlap = Overlap(rows)
        self.overlap_rows = rows

    def scalings(self, t):
        return [term.scaling(t) for term in self.terms]

    def apply_H(self, psi, t):
        out = np.zeros_like(psi)
        for term, s in zip(self.terms, self.scalings(t)):
            term.multiply(psi, out, s)
        return out

    def energy(self, psi, t=0.0):
        """<psi|H|psi> / <psi|S|psi> (H applied as S^-1 H, then the S inner product)."""
        n2 = np.vdot(psi, self.overlap.multiply(psi)).real
        phi = psi / np.sqrt(n2)
        tmp = self.overlap.solve(self.apply_H(phi, t))
        return np.vdot(phi, self.overlap.multiply(tmp)).real

    def norm(self, psi):
        return float(np.sqrt(np.vdot(psi, self.overlap.multiply(psi)).real))


class OraclePam:
    def __init__(self, ham: OracleHamiltonian, basis_size=20, double_ortho=True):
        self.ham = ham
        self.m = basis_size
        self.double_ortho = double_ortho

    def step(self, psi, t, dt):
        ovl = self.ham.overlap
        shape = psi.shape
        x = ovl.multiply_sqrt(psi, conj=False)

        def op(v):
            u = ovl.solve_sqrt(v.reshape(shape), conj=False)
            w = self.ham.apply_H(u, t)
            return ovl.solve_sqrt(w, conj=True).ravel()

        y, err = pamp_propagate(op, x.ravel(), dt, self.m, self.double_ortho)
        self.last_error = err
        return ovl.solve_sqrt(y.reshape(shape), conj=False)


class OracleCayley:
    def __init__(self, ham: OracleHamiltonian, dt, precond_terms_idx, basis_size=20, tolerance=0.0):
        """precond_terms_idx: indices of the (angular-diagonal, time-independent) terms in M."""
        self.ham = ham
        self.m = basis_size
        self.tol = tolerance
        diag = [ham.terms[i] for i in precond_terms_idx]
        self.prec = BandLU(ham.overlap_rows, diag, ham.nang, ham.N, ham.kb, 1.0, 1j * dt / 2.0)

    def multiply_SpH(self, psi, h_factor, t):
        return self.ham.overlap.multiply(psi) + h_factor * self.ham.apply_H(psi, t)

    def step(self, psi, t, dt):
        tt = t + abs(dt / 2.0)
        shape = psi.shape
        b = self.multiply_SpH(psi, -1j * dt / 2.0, tt)
        rhs = self.prec.solve(b)

        def op(v):
            return self.prec.solve(self.multiply_SpH(v.reshape(shape), 1j * dt / 2.0, tt)).ravel()

        x, err, k = gmres_solve(op, rhs.ravel(), self.m, self.tol)
        self.last_error, self.last_iterations = err, k
        x = x.reshape(shape)
        self.last_true_residual = np.linalg.norm(self.multiply_SpH(x, 1j * dt / 2.0, tt) - b)
        return x
