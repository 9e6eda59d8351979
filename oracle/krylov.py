"""Oracle Krylov methods (complex128, CPU) - test infrastructure only.

Restatements of the reference's header-only templates:
  * ``pamp_propagate``  core/krylov/pamp/pamp/pamp.h:270-351 (Arnoldi, CGS with optional
    second pass when ||r|| < 0.717 ||r0||, :353-401), :430-468 (scaling: 2^ceil(log2 max|A|)),
    :470-565 (diagonal Pade, Horner in A^2), :613-670 (PropagateVector; error = |v_last|^2).
  * ``gmres_solve``     core/krylov/gmres/gmres.h:260-354 (Arnoldi with DGKS
    re-orthogonalisation, up to 5 passes), :433-505 (SolveVector: x0 = 0, zgels least
    squares every iteration, stop when the residual estimate <= max(tol, 1e-13)).
  * ``piram_solve``     core/krylov/piram/piram/piram.h:346-442, :473-535, :537-655, :698-753.
"""
from __future__ import annotations

import math

import numpy as np


def pade_exponential(A, order=6):
    """exp(A) by the diagonal Pade approximant without scaling (pamp.h:470-565)."""
    n = A.shape[0]
    A2 = A @ A
    c = [1.0]
    for i in range(order):
        c.append(c[i] * (order - i) / ((i + 1) * (2 * order - i)))
    Q = c[order] * np.eye(n, dtype=complex)
    P = c[order - 1] * np.eye(n, dtype=complex)
    odd = True
    for i in range(order - 2, -1, -1):
        if odd:
            Q = Q @ A2 + c[i] * np.eye(n)
        else:
            P = P @ A2 + c[i] * np.eye(n)
        odd = not odd
    if odd:
        Q = Q @ A
    else:
        P = P @ A
    Q = Q - P
    E = 2.0 * np.linalg.solve(Q, P) + np.eye(n)
    return -E if odd else E


def scaling_pade_exponential(A, order=6):
    """Scaling and squaring around :func:`pade_exponential` (pamp.h:430-468)."""
    maxv = np.max(np.abs(A))
    s = int(math.ceil(math.log2(maxv))) if maxv > 0 else 0
    s = max(0, s)
    E = pade_exponential(A / 2.0 ** s, order)
    for _ in range(s):
        E = E @ E
    return E


def _orthogonalize(V, r, double_ortho, max_count):
    """CGS projection + DGKS passes; returns (r, coefficients)."""
    orig = np.linalg.norm(r)
    h = V.conj() @ r
    r = r - V.T @ h
    res = np.linalg.norm(r)
    if double_ortho:
        count = 0
        while res < 0.717 * orig:
            count += 1
            if count > max_count:
                break
            h2 = V.conj() @ r
            r = r - V.T @ h2
            h = h + h2
            orig, res = res, np.linalg.norm(r)
    return r, h


def pamp_propagate(op, v, dt, m, double_ortho=False, tolerance=None, max_ortho=3):
    """exp(-i dt A) v with an m-dimensional Arnoldi basis (Euclidean inner product)."""
    tol = math.sqrt(np.finfo(float).eps) if tolerance is None else tolerance
    n = v.size
    V = np.zeros((m, n), dtype=complex)
    H = np.zeros((m, m), dtype=complex)
    norm = np.linalg.norm(v)
    r = v / norm
    V[0] = r
    r = op(V[0])
    alpha = np.vdot(V[0], r)
    r = r - alpha * V[0]
    H[0, 0] = alpha
    j = 0
    while j < m - 1:
        beta = np.linalg.norm(r)
        if beta < tol:
            break
        V[j + 1] = r / beta
        H[j + 1, j] = beta
        r = op(V[j + 1])
        r, h = _orthogonalize(V[:j + 2], r, double_ortho, max_ortho)
        H[:j + 2, j + 1] = h
        j += 1
    E = scaling_pade_exponential(-1j * dt * H)
    c = E[:, 0]
    return norm * (V.T @ c), abs(c[-1]) ** 2


def gmres_solve(op, b, m, tolerance=0.0, max_ortho=5):
    """Solve op(x) = b from x0 = 0 (gmres.h:433-505). Returns (x, residual estimate, iterations)."""
    tol = max(tolerance, 1e-13)
    n = b.size
    V = np.zeros((m, n), dtype=complex)
    H = np.zeros((m + 1, m), dtype=complex)
    inorm = np.linalg.norm(b)
    V[0] = b / inorm
    r = op(V[0])
    alpha = np.vdot(V[0], r)
    r = r - alpha * V[0]
    H[0, 0] = alpha
    beta = np.linalg.norm(r)
    happy = beta < tol
    H[1, 0] = beta
    j = 0
    if happy:
        y = np.array([inorm / alpha])
        return V[0] * y[0], 0.0, 1
    err = beta
    y = None
    while j < m - 1 and not happy and abs(err) > tol:
        V[j + 1] = r / H[j + 1, j]
        r = op(V[j + 1])
        r, h = _orthogonalize(V[:j + 2], r, True, max_ortho)
        H[:j + 2, j + 1] = h
        beta = np.linalg.norm(r)
        if beta < tol:
            happy = True
        H[j + 2, j + 1] = beta
        j += 1
        k = j + 1
        rhs = np.zeros(k + 1, dtype=complex)
        rhs[0] = inorm
        y, *_ = np.linalg.lstsq(H[:k + 1, :k], rhs, rcond=None)
        err = np.linalg.norm(H[:k + 1, :k] @ y - rhs)
    if y is None:
        y, *_ = np.linalg.lstsq(H[:2, :1], np.array([inorm, 0.0]), rcond=None)
    k = len(y)
    return V[:k].T @ y, err, k


def _sort_real(values):
    vals = list(values)
    order = list(range(len(vals)))
    for i in range(len(vals)):
        for j in range(i + 1, len(vals)):
            if not (vals[i].real < vals[j].real):
                vals[i], vals[j] = vals[j], vals[i]
                order[i], order[j] = order[j], order[i]
    return np.array(vals), np.array(order)


def _sort_abs_desc(values):
    vals = list(values)
    order = list(range(len(vals)))
    for i in range(len(vals)):
        for j in range(i + 1, len(vals)):
            if not (abs(vals[i]) > abs(vals[j])):
                vals[i], vals[j] = vals[j], vals[i]
                order[i], order[j] = order[j], order[i]
    return np.array(vals), np.array(order)


def piram_solve(op, start, m, k, tolerance=0.0, max_restarts=10, max_ortho=3, seed=12345, largest_abs=False):
    """Lowest-real-part eigenpairs by implicit restarts (piram.h:698-753).

    Returns (eigenvalues sorted by real part [:k], eigenvectors (k, n), restarts, converged).
    ``largest_abs`` selects the inverse-iteration ordering (largest |theta| first,
    ``CompareComplexGreaterAbs``, piramsolver.cpp:79-90) used with a shift-invert operator.
    One addition to the reference: when the new residual is numerically zero
    (||f|| < 1e-14 max|H|: an invariant subspace was found, e.g. for an operator that is
    block diagonal in l), a random vector orthogonal to the basis continues the
    factorization with a zero subdiagonal entry (ARPACK's remedy); the reference would
    divide by the vanishing norm.
    """
    rng = np.random.default_rng(seed)
    eps = np.finfo(float).eps
    tol = max(tolerance, eps)
    eps23 = eps ** (2.0 / 3.0)
    n = start.size
    V = np.zeros((m, n), dtype=complex)
    H = np.zeros((m, m), dtype=complex)
    r = start / np.linalg.norm(start)
    V[0] = r
    r = op(V[0])
    H[0, 0] = np.vdot(V[0], r)
    r = r - H[0, 0] * V[0]

    def expand(j0, r):
        for j in range(j0, m - 1):
            beta = np.linalg.norm(r)
            if beta < 1e-14 * max(np.max(np.abs(H)), 1e-300):
                r, _ = _orthogonalize(V[:j + 1], rng.uniform(-1, 1, n).astype(complex), True, max_ortho)
                r, _ = _orthogonalize(V[:j + 1], r, True, max_ortho)
                V[j + 1] = r / np.linalg.norm(r)
                H[j + 1, j] = 0.0
            else:
                V[j + 1] = r / beta
                H[j + 1, j] = beta
            r = op(V[j + 1])
            r, h = _orthogonalize(V[:j + 2], r, True, max_ortho)
            H[:j + 2, j + 1] = h
        return r

    r = expand(0, r)
    restarts = 0
    while True:
        evals, evecs = np.linalg.eig(H)
        svals, order = _sort_abs_desc(evals) if largest_abs else _sort_real(evals)
        rn = np.linalg.norm(r)
        bounds = np.abs(evecs[m - 1, :]) * rn
        shift_idx = order[k:]
        shifts = evals[shift_idx][np.argsort(bounds[shift_idx], kind="stable")]
        conv = np.array([abs(evecs[m - 1, order[i]]) * rn - tol * max(eps23, tol * abs(svals[i])) for i in range(k)])
        converged = bool(np.all(conv <= 0))
        if converged or restarts >= max_restarts:
            break
        Q = np.eye(m, dtype=complex)
        for mu in shifts:
            Qi, R = np.linalg.qr(H - mu * np.eye(m))
            H = R @ Qi + mu * np.eye(m)
            Q = Q @ Qi
        sigma = Q[m - 1, k - 1]
        beta = H[k, k - 1]
        V[:k + 1] = (V.T @ Q[:, :k + 1]).T
        r = sigma * r + beta * V[k]
        H[:, k:] = 0
        H[k:, :] = 0
        restarts += 1
        r = expand(k - 1, r)
    X = evecs[:, order[:k]]
    return svals[:k], (V.T @ X).T, restarts, converged
