"""The oracle against the reference's known answers and fixtures (CPU only)."""
import numpy as np
import scipy.linalg as sl

from oracle.krylov import gmres_solve, pade_exponential, piram_solve, scaling_pade_exponential
from oracle.operators import BandLU, dense_operator
from oracle.propagators import OracleCayley, OraclePam
from tests.helpers import golden, hydrogen_problem, oracle_hamiltonian, relerr


def test_pade_2x2_known_answer():
    """pampwrapper.h:79-101 TestPade: exp(iA) of [[-49, 24], [24, 31]] by scaling + Pade."""
    A = np.array([[-49.0, 24.0], [24.0, 31.0]], dtype=complex)
    w, V = np.linalg.eigh(A.real)
    exact = (V * np.exp(1j * w)) @ V.T
    assert np.max(np.abs(scaling_pade_exponential(1j * A) - exact)) < 1e-11
    small = 1e-2 * A
    assert np.max(np.abs(pade_exponential(small, 15) - sl.expm(small))) < 1e-13


def _qdot():
    g = golden("qdot_piram.npz")
    n = int(g["rows"].max()) + 1
    A = np.zeros((n, n))
    np.add.at(A, (g["rows"].astype(int), g["cols"].astype(int)), g["vals"])
    return A, g


def test_piram_qdot_fixture():
    """pIRAM on the reference's own test matrix and start vector (piramtest.cpp:153-182:
    m 50, 5 eigenvalues). With the test's 10 restarts the non-degenerate lowest values are
    found; with 40 restarts all five lowest (two doubly degenerate pairs) match the dense
    eigen-decomposition."""
    A, g = _qdot()
    op = lambda v: A @ v
    vals, vecs, rs, conv = piram_solve(op, g["init"].astype(complex), 50, 5, 0.0, 10)
    assert rs == 10
    assert abs(vals[0] - 1.0) < 1e-10 and abs(vals[1] - g["lowest5"][1]) < 1e-10
    vals, vecs, rs, conv = piram_solve(op, g["init"].astype(complex), 50, 5, 0.0, 40)
    assert np.max(np.abs(vals - g["lowest5"])) < 1e-9
    for i in range(5):
        assert np.linalg.norm(A @ vecs[i] - vals[i] * vecs[i]) < 1e-8 * np.linalg.norm(vecs[i])


def test_pamp_matches_expm():
    prob = hydrogen_problem()
    ham = oracle_hamiltonian(prob)
    g = golden("hydrogen_small.npz")
    psi, t, dt = g["psi"], float(g["t"]), float(g["dt"])
    nang, N = psi.shape
    H = dense_operator(ham.terms, ham.scalings(t), nang, N)
    S = np.kron(np.eye(nang), ham.overlap.S)
    exact = (sl.expm(-1j * dt * np.linalg.solve(S, H)) @ psi.ravel()).reshape(psi.shape)
    out = OraclePam(ham, 20, True).step(psi, t, dt)
    assert relerr(out, exact) < 1e-12
    assert relerr(out, g["pamp"]) < 1e-13  # golden fixture unchanged


def test_cayley_matches_direct_solve():
    prob = hydrogen_problem()
    ham = oracle_hamiltonian(prob)
    g = golden("hydrogen_small.npz")
    psi, t, dt = g["psi"], float(g["t"]), float(g["dt"])
    nang, N = psi.shape
    tt = t + dt / 2
    H = dense_operator(ham.terms, ham.scalings(tt), nang, N)
    S = np.kron(np.eye(nang), ham.overlap.S)
    exact = np.linalg.solve(S + 0.5j * dt * H, (S - 0.5j * dt * H) @ psi.ravel()).reshape(psi.shape)
    cay = OracleCayley(ham, dt, [0], 20, 1e-13)
    out = cay.step(psi, t, dt)
    assert relerr(out, exact) < 1e-11
    assert cay.last_true_residual < 1e-11
    assert relerr(out, g["cayley"]) < 1e-12
    assert relerr(ham.apply_H(psi, t), g["Hpsi"]) < 1e-14


def test_gmres_identity_breakdown_and_cap():
    rng = np.random.default_rng(3)
    b = rng.normal(size=30) + 0j
    x, err, k = gmres_solve(lambda v: 2.0 * v, b, 10)
    assert np.allclose(x, b / 2) and k == 1
    A = np.diag(np.linspace(1, 1000, 30)) + 0j
    x, err, k = gmres_solve(lambda v: A @ v, b, 5)
    assert k == 5 and err > 1e-13  # stopped at the basis size, estimate reported


def test_shift_invert_ground_state_config1():
    """Ground state of the N=150, lmax=10 hydrogen model by shift-invert pIRAM (sigma -0.7)."""
    prob = hydrogen_problem(lmax=10, nbsplines=150, rmax=100.0)
    ham = oracle_hamiltonian(prob)
    nang, N = 11, 150
    lu = BandLU(ham.overlap_rows, [ham.terms[0]], nang, N, ham.kb, 0.7, 1.0)
    op = lambda v: lu.solve(ham.overlap.multiply(v.reshape(nang, N))).ravel()
    start = np.random.default_rng(1234).uniform(size=nang * N).astype(complex)
    vals, vecs, rs, conv = piram_solve(op, start, 20, 2, 1e-12, 50, largest_abs=True)
    lam = -0.7 + 1.0 / vals
    assert abs(lam[0] + 0.5) < 1e-10
    psi = vecs[0].reshape(nang, N)
    assert abs(ham.energy(psi) + 0.5) < 1e-10


def test_pamp_arnoldi_on_u_inverse_basis_equals_balanced_form():
    """The recurrence the single-kernel pAMP step runs: Arnoldi on T_j = U^-1 V_j (S = U^T U)
    with y = H T_j, z = S^-1 y, h1 = T^H y, h2 = T^H S z', beta^2 = ||z'||_S^2 - |h2|^2 gives the
    Hessenberg matrix of the balanced form (Arnoldi on U^-T H U^-1 with CGS2) and the same
    psi(t + dt) = U^-1 ||U psi|| V c = ||psi||_S sum_j c_j T_j (complex128, random banded S > 0
    and Hermitian H)."""
    rng = np.random.default_rng(11)
    n, m, dt, kb = 48, 10, 0.05, 3
    S = np.zeros((n, n))
    for d in range(-kb, kb + 1):
        S += np.diag(rng.uniform(-0.2, 0.2, n - abs(d)), d) if d else 0.0
    S = (S + S.T) / 2 + 2.0 * np.eye(n)
    Hh = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    H = (Hh + Hh.conj().T) / 2
    psi = rng.normal(size=n) + 1j * rng.normal(size=n)
    U = sl.cholesky(S)
    Ui = np.linalg.inv(U)
    A = Ui.T @ H @ Ui
    x = U @ psi
    nrm = np.linalg.norm(x)
    V, Hm = [x / nrm], np.zeros((m, m), complex)
    for j in range(m):
        w = A @ V[j]
        for _ in range(2):
            h = np.array([v.conj() @ w for v in V])
            w = w - sum(hh * v for hh, v in zip(h, V))
            Hm[:j + 1, j] += h
        if j + 1 < m:
            Hm[j + 1, j] = np.linalg.norm(w)
        V.append(w / np.linalg.norm(w))
    ref = Ui @ (np.array(V[:m]).T @ (sl.expm(-1j * dt * Hm)[:, 0] * nrm))
    nrm_s = np.sqrt((psi.conj() @ S @ psi).real)
    T, Ht = [psi / nrm_s], np.zeros((m, m), complex)
    for j in range(m):
        y = H @ T[j]
        z = np.linalg.solve(S, y)
        h1 = np.array([t.conj() @ y for t in T])
        z1 = z - sum(hh * t for hh, t in zip(h1, T))
        u = S @ z1
        h2 = np.array([t.conj() @ u for t in T])
        beta = np.sqrt((z1.conj() @ u).real - np.sum(np.abs(h2) ** 2))
        Ht[:j + 1, j] = h1 + h2
        if j + 1 < m:
            Ht[j + 1, j] = beta
        T.append((z1 - sum(hh * t for hh, t in zip(h2, T))) / beta)
    out = np.array(T[:m]).T @ (sl.expm(-1j * dt * Ht)[:, 0] * nrm_s)
    assert np.abs(Hm - Ht).max() < 1e-12 * np.abs(Hm).max()
    assert np.linalg.norm(out - ref) < 1e-13 * np.linalg.norm(ref)
