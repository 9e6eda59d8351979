"""Oracle operators (complex128, CPU) - test infrastructure only.

* ``tensor_multiply``: the generated TensorPotentialMultiply_<Diag|Simp|Ident>_BandNH
  (core/tensorpotential/tensorpotentialmultiply_generator.py:302-462 storage loops,
  :622-762 BandNH body calling zgbmv at :702-724): for each angular pair
  dest[row, :] += scaling * A_pair @ src[col, :], A_pair general banded with the BLAS
  layout slot j*(2k+1) + (k+i-j) (GeometryInfo.py:437-456).
* ``Overlap``: OverlapMatrix (core/representation/overlapmatrix.cpp): upper banded Cholesky
  S = U^H U (zpbtrf, :35-37) and the vector operations (:123-149) on every radial fibre.
* ``BandLU``: BSplineSolver's banded LU with partial pivoting (zgbtrf/zgbtrs,
  core/transform/bspline/bsplinesolver.h:43-162).
* ``dense_operator``: dense assembly from the tensor layout, after
  examples/tensor/helium_stabilization/twoelectron_test.py:31-56.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sl
from numpy.lib.stride_tricks import sliding_window_view


def bandnh_rows(potential_row, N, kb):
    """BLAS general-band storage (N*(2kb+1),) -> row-oriented (N, 2kb+1), [i, kb+(j-i)] = A(i,j)."""
    b = 2 * kb + 1
    out = np.zeros((N, b), dtype=np.complex128)
    for d in range(-kb, kb + 1):
        i = np.arange(max(0, -d), min(N, N - d))
        j = i + d
        out[i, kb + d] = potential_row[j * b + (kb + i - j)]
    return out


class TermOracle:
    """One consolidated tensor potential in the reference layout, ready to multiply."""

    def __init__(self, storage, potential, pairs, nang, N, kb, time_function=None):
        self.storage = storage
        self.nang, self.N, self.kb = nang, N, kb
        self.time_function = time_function
        pot = np.asarray(potential, dtype=np.complex128)
        if storage == "Diag_BandNH":
            self.rows = np.arange(nang)
            self.cols = np.arange(nang)
            self.bands = np.stack([bandnh_rows(pot[a], N, kb) for a in range(nang)])
        elif storage == "Ident_BandNH":
            self.rows = np.arange(nang)
            self.cols = np.arange(nang)
            self.bands = np.repeat(bandnh_rows(pot[0], N, kb)[None], nang, axis=0)
        elif storage == "Simp_BandNH":
            pairs = np.asarray(pairs)
            self.rows = pairs[:, 0]
            self.cols = pairs[:, 1]
            self.bands = np.stack([bandnh_rows(pot[p], N, kb) for p in range(len(pairs))]) if len(pairs) else \
                np.zeros((0, N, 2 * kb + 1), dtype=np.complex128)
        else:
            raise ValueError(storage)

    def scaling(self, t):
        return 1.0 if self.time_function is None else float(self.time_function(t))

    def multiply(self, src, dest, scaling):
        """dest += scaling * V src (loop over pairs, each a general band product)."""
        kb = self.kb
        pad = np.zeros((src.shape[0], src.shape[1] + 2 * kb), dtype=np.complex128)
        pad[:, kb:kb + src.shape[1]] = src
        win = sliding_window_view(pad, 2 * kb + 1, axis=1)  # (nang, N, b): win[c, i, d] = src[c, i+d-kb]
        y = np.einsum("pid,pid->pi", self.bands, win[self.cols])
        np.add.at(dest, self.rows, scaling * y)


def tensor_multiply(terms, scalings, src, dest):
    for term, s in zip(terms, scalings):
        term.multiply(src, dest, s)


def dense_operator(terms, scalings, nang, N):
    """Dense (nang*N)^2 matrix of sum_t s_t V_t (psi flattened C-order [a][i])."""
    M = np.zeros((nang * N, nang * N), dtype=np.complex128)
    kb = terms[0].kb if terms else 0
    for term, s in zip(terms, scalings):
        for p, (r, c) in enumerate(zip(term.rows, term.cols)):
            for d in range(-kb, kb + 1):
                i = np.arange(max(0, -d), min(N, N - d))
                M[r * N + i, c * N + i + d] += s * term.bands[p, i, kb + d]
    return M


class Overlap:
    """Banded overlap S (rows (N, 2kb+1), real) with its upper Cholesky factor."""

    def __init__(self, overlap_rows):
        rows = np.asarray(overlap_rows)
        self.N, b = rows.shape
        self.kb = (b - 1) // 2
        kb = self.kb
        N = self.N
        # upper storage for LAPACK: ab[kb + i - j, j] = S(i, j), i <= j
        ab = np.zeros((kb + 1, N))
        for d in range(0, kb + 1):
            j = np.arange(d, N)
            ab[kb - d, j] = rows[j - d, kb + d]
        self.ab = ab
        self.cho = sl.cholesky_banded(ab, lower=False)
        self.S = np.zeros((N, N))
        for d in range(-kb, kb + 1):
            i = np.arange(max(0, -d), min(N, N - d))
            self.S[i, i + d] = rows[i, kb + d]
        self.U = np.zeros((N, N))
        for d in range(0, kb + 1):
            j = np.arange(d, N)
            self.U[j - d, j] = self.cho[kb - d, j]

    # psi has shape (nang, N); every op acts on each row (fibre)
    def multiply(self, psi):
        return psi @ self.S.T

    def solve(self, psi):
        return sl.cho_solve_banded((self.cho, False), psi.T).T

    def multiply_sqrt(self, psi, conj=False):
        M = self.U.conj().T if conj else self.U
        return psi @ M.T

    def solve_sqrt(self, psi, conj=False):
        M = self.U.conj().T if conj else self.U
        return sl.solve_triangular(M, psi.T, lower=conj).T


class BandLU:
    """Per-channel banded LU with partial pivoting of M_a = cS S + cH H_a (zgbtrf/zgbtrs)."""

    def __init__(self, overlap_rows, diag_terms, nang, N, kb, cS, cH):
        self.kb = kb
        self.factors = []
        for a in range(nang):
            M = cS * np.asarray(overlap_rows, dtype=np.complex128).copy()
            for term in diag_terms:
                for p, (r, c) in enumerate(zip(term.rows, term.cols)):
                    if r == a and c == a:
                        M = M + cH * term.bands[p]
            ab = np.zeros((3 * kb + 1, N), dtype=np.complex128)
            for d in range(-kb, kb + 1):
                i = np.arange(max(0, -d), min(N, N - d))
                ab[2 * kb - d, i + d] = M[i, kb + d]
            lu, piv, info = sl.lapack.zgbtrf(ab, kb, kb)
            if info != 0:
                raise np.linalg.LinAlgError("zgbtrf info %d" % info)
            self.factors.append((lu, piv))

    def solve(self, psi):
        out = np.empty_like(psi)
        for a, (lu, piv) in enumerate(self.factors):
            x, info = sl.lapack.zgbtrs(lu, self.kb, self.kb, psi[a], piv)
            out[a] = x
        return out
