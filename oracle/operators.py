"""Oracle operators (complex128, CPU) - test infrastructure only.

* ``tensor_multiply``: the generated TensorPotentialMultiply_<angular>_<radial> kernels
  (core/tensorpotential/tensorpotentialmultiply_generator.py: angular storage loops
  :302-462, :467-618, :622-762, :1227-1330; radial bodies zgbmv :702-724, zhbmv :585-600,
  dense loop :1268-1275): for each angular block dest[row, :] += scaling * A @ src[col, :],
  BandNH blocks in the BLAS layout slot j*(2k+1) + (k+i-j) (GeometryInfo.py:437-456).
* ``Overlap``: OverlapMatrix (core/representation/overlapmatrix.cpp): upper banded Cholesky
  S = U^H U (zpbtrf, :35-37) and the vector operations (:123-149) on every radial fibre.
* ``BandLU``: BSplineSolver's banded LU with partial pivoting (zgbtrf/zgbtrs,
  core/transform/bspline/bsplinesolver.h:43-162).
* ``dense_operator``: dense assembly from the tensor layout, after
  examples/tensor/helium_stabilization/twoelectron_test.py:31-56.
* ``factored_multiply``: a two-electron term as angular coefficients x shared radial
  operators (the multipole sum of examples/tensor/helium_stabilization/coupledspherical.cpp:
  7-127 kept per multipole), applied point by point on the radial grid.
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


def outer_blocks(kind, e0, pairs, nang):
    """Angular-rank loops of the generated multiply kernels: list of (row, col, index, conj).

    Simp (tensorpotentialmultiply_generator.py:326-333), Herm (:380-386, second pass with
    row/col swapped and the potential conjugated), Diag (:416-421), Ident (:448-453, index 0
    for every row), Band (:507-552: (row, col >= row) at row*bc + col - row, then the mirrored
    (col, row) conjugated), BandNH (:662-694: (row, col) at col*bc + sub + row - col), Dense
    (:1268-1275: row*n + col)."""
    out = []
    if kind in ("Simp", "Herm"):
        pairs = np.asarray(pairs).reshape(-1, 2)
        out += [(int(r), int(c), p, False) for p, (r, c) in enumerate(pairs)]
        if kind == "Herm":
            out += [(int(c), int(r), p, True) for p, (r, c) in enumerate(pairs)]
    elif kind == "Diag":
        out += [(a, a, a, False) for a in range(nang)]
    elif kind == "Ident":
        out += [(a, a, 0, False) for a in range(nang)]
    elif kind == "Dense":
        out += [(r, c, r * nang + c, False) for r in range(nang) for c in range(nang)]
    elif kind == "Band":
        bc = e0 // nang
        i = 0
        for row in range(nang):  # first pass: upper part, row-major, bc slots per row
            for col in range(row, row + bc):
                if col < nang:
                    out.append((row, col, i, False))
                i += 1
        i = 0
        for herm_row in range(nang):  # mirrored part, diagonal slot skipped
            i += 1
            for herm_col in range(herm_row + 1, herm_row + bc):
                if herm_col < nang:
                    out.append((herm_col, herm_row, i, True))
                i += 1
    elif kind == "BandNH":
        bc = e0 // nang
        sub = (bc - 1) // 2
        for col in range(nang):
            for row in range(max(0, col - sub), min(nang, col + sub + 1)):
                out.append((row, col, col * bc + sub + row - col, False))
    else:
        raise ValueError(kind)
    return out


def radial_rows(kind, pot, N, kb, conj):
    """Radial block of one angular pair as band rows (N, 2kb+1), [i, kb + j - i] = A(i, j).

    BandNH: zgbmv layout j*(2kb+1) + kb + i - j (:700-723); conjugated through the explicit
    loop when the outer rank asks (:653-690). Band: zhbmv('L') (:585-600), lower triangle
    column-major with lda = kb + 1, upper = conjugate, diagonal real; the reference calls
    zhbmv whatever the conjugate flag. Diag: A(i, i) = pot[i]. Ident: A(i, i) = pot[0]."""
    b = 2 * kb + 1
    out = np.zeros((N, b), dtype=np.complex128)
    if kind == "BandNH":
        out[:] = bandnh_rows(pot, N, kb)
        if conj:
            out = out.conj()
    elif kind == "Band":
        k1 = kb + 1
        for i in range(N):
            for j in range(max(0, i - kb), min(N, i + kb + 1)):
                if i > j:
                    v = pot[j * k1 + (i - j)]
                elif i < j:
                    v = np.conj(pot[i * k1 + (j - i)])
                else:
                    v = complex(pot[j * k1].real, 0.0)
                out[i, kb + j - i] = v
    elif kind == "Diag":
        out[:, kb] = np.conj(pot[:N]) if conj else pot[:N]
    elif kind == "Ident":
        out[:, kb] = np.conj(pot[0]) if conj else pot[0]
    else:
        raise ValueError(kind)
    return out


def fibre_block(kind, pot, pairs, N, kb, conj):
    """Last-rank block as ("band", rows (N, 2kb+1)) or ("dense", (N, N)).

    Simp on the last rank (the generator's pair loop, :326-333) is a band when every pair
    lies within kb of the diagonal, else dense; Dense follows :1268-1275 (row*N + col)."""
    if kind == "Dense":
        m = pot.reshape(N, N)
        return "dense", (m.conj() if conj else m)
    if kind == "Simp":
        pairs = np.asarray(pairs).reshape(-1, 2)
        v = pot.conj() if conj else pot
        if np.all(np.abs(pairs[:, 0] - pairs[:, 1]) <= kb):
            rows = np.zeros((N, 2 * kb + 1), dtype=np.complex128)
            np.add.at(rows, (pairs[:, 0], kb + pairs[:, 1] - pairs[:, 0]), v)
            return "band", rows
        m = np.zeros((N, N), dtype=np.complex128)
        np.add.at(m, (pairs[:, 0], pairs[:, 1]), v)
        return "dense", m
    return "band", radial_rows(kind, pot, N, kb, conj)


class TermOracle:
    """One consolidated tensor potential in the reference layout, ready to multiply.

    ``storage`` is "<rank0>_<rank1>[_<rank2>]"; the loops of rank r nest inside those of
    rank r-1 (the generator's nesting), each mirrored Herm/Band pass toggling the conjugate
    flag. Rows and columns flatten all ranks but the last (C order); banded last-rank blocks
    are kept as band rows (``rows``, ``cols``, ``bands``), dense ones (:1227-1330) as matrices
    (``drows``, ``dcols``, ``dense``). For rank 2, ``pairs`` is the angular pair list; for
    rank 3 pass ``shape`` and a per-rank list of pair arrays."""

    def __init__(self, storage, potential, pairs, nang, N, kb, time_function=None, shape=None):
        self.storage = storage
        kinds = storage.split("_")
        self.shape = tuple(shape) if shape is not None else (nang, N)
        self.nang, self.N, self.kb = int(np.prod(self.shape[:-1])), self.shape[-1], kb
        self.time_function = time_function
        pot = np.asarray(potential, dtype=np.complex128)
        if pot.ndim == 1:
            pot = pot.reshape(1, -1)
        if len(kinds) == 2 and shape is None:
            pairs_list = [pairs, None]
        else:
            pairs_list = list(pairs) if pairs is not None else [None] * len(kinds)
        ext = pot.shape[:len(kinds) - 1] if pot.ndim >= len(kinds) else (pot.shape[0],)
        blocks = [(0, 0, 0, False)]
        for r, kind in enumerate(kinds[:-1]):
            n = self.shape[r]
            rb = outer_blocks(kind, ext[r], pairs_list[r], n)
            blocks = [(a[0] * n + q[0], a[1] * n + q[1], a[2] * ext[r] + q[2], a[3] != q[3]) for a in blocks for q in rb]
        flat = pot.reshape(int(np.prod(ext)), -1) if pot.size else np.zeros((0, 1), dtype=np.complex128)
        N, b = self.N, 2 * kb + 1
        bl, db = [], []
        for r, c, i, cj in blocks:
            what, m = fibre_block(kinds[-1], flat[i], pairs_list[-1], N, kb, cj)
            (bl if what == "band" else db).append((r, c, m))
        self.rows = np.array([x[0] for x in bl], dtype=np.int64)
        self.cols = np.array([x[1] for x in bl], dtype=np.int64)
        self.bands = np.stack([x[2] for x in bl]) if bl else np.zeros((0, N, b), dtype=np.complex128)
        self.drows = np.array([x[0] for x in db], dtype=np.int64)
        self.dcols = np.array([x[1] for x in db], dtype=np.int64)
        self.dense = np.stack([x[2] for x in db]) if db else np.zeros((0, N, N), dtype=np.complex128)

    def scaling(self, t):
        return 1.0 if self.time_function is None else float(self.time_function(t))

    def multiply(self, src, dest, scaling):
        """dest += scaling * V src (src/dest flattened to (fibres, N) internally)."""
        kb = self.kb
        shape = src.shape
        src = src.reshape(-1, self.N)
        d2 = dest.reshape(-1, self.N)
        if len(self.rows):
            pad = np.zeros((src.shape[0], src.shape[1] + 2 * kb), dtype=np.complex128)
            pad[:, kb:kb + src.shape[1]] = src
            win = sliding_window_view(pad, 2 * kb + 1, axis=1)  # win[c, i, d] = src[c, i+d-kb]
            y = np.einsum("pid,pid->pi", self.bands, win[self.cols])
            np.add.at(d2, self.rows, scaling * y)
        if len(self.drows):
            y = np.einsum("pij,pj->pi", self.dense, src[self.dcols])
            np.add.at(d2, self.drows, scaling * y)
        if d2.base is not dest and d2 is not dest:
            dest[...] = d2.reshape(shape)


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
        for p, (r, c) in enumerate(zip(term.drows, term.dcols)):
            M[r * N:(r + 1) * N, c * N:(c + 1) * N] += s * term.dense[p]
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


def stencil_apply(R, x, kb):
    """y[i1, i2] = sum_{d1, d2} R[i1, d1, d2, i2] x[i1 + d1 - kb, i2 + d2 - kb], zero outside
    the grid: one radial factor [N1][2kb+1][2kb+1][N2] on one channel's [N1][N2] block."""
    N1, b, _, N2 = R.shape
    xp = np.zeros((N1 + 2 * kb, N2 + 2 * kb), dtype=np.complex128)
    xp[kb:kb + N1, kb:kb + N2] = x
    y = np.zeros((N1, N2), dtype=np.complex128)
    for d1 in range(b):
        for d2 in range(b):
            y += R[:, d1, d2, :] * xp[d1:d1 + N1, d2:d2 + N2]
    return y


def factored_multiply(factored, scales, src, dest):
    """dest[row] += scale * weight_q * coef_q(row, col) * R_q applied to src[col], for
    factored = [(FactoredPotential, slot)] and src/dest [Nang][N1][N2]."""
    for fac, slot in factored:
        rows, cols = fac.entries()
        for q in range(fac.nfactors):
            c = fac.coefs[q]
            w = scales[slot] * fac.weights[q]
            cache = {}
            for r, col, v in zip(rows, cols, c):
                if v == 0.0:
                    continue
                if col not in cache:
                    cache[col] = stencil_apply(fac.stencil[q], src[col], fac.kb)
                dest[r] += w * v * cache[col]
    return dest
