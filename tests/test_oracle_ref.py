"""The oracle against the reference's own Krylov code (CPU only).

oracle/_ref/libref_krylov.so is the reference's pAMP, GMRES and pIRAM templates compiled
unchanged from its source tree, plus the generated BandNH multiply restated over BLAS zgbmv
(oracle/ref/build_ref.py). Where that tree is available the library is built on first use;
elsewhere (a machine without the reference) these tests are skipped, and the committed
fixtures they pin (tests/golden/*.npz) stay checked by the other tests.
"""
import os

import numpy as np
import pytest

from oracle.krylov import gmres_solve, piram_solve
from oracle.propagators import OracleCayley, OraclePam
from tests.helpers import golden, hydrogen_problem, infidelity, oracle_hamiltonian, oracle_terms, relerr


@pytest.fixture(scope="module")
def ref():
    from oracle import refkrylov
    from oracle.ref import build_ref
    tree = build_ref.reference_tree()
    if tree is None and not refkrylov.available():
        pytest.skip("the reference source tree is not on this machine")
    if tree is not None:
        build_ref.build(tree)
    return refkrylov


def _model(ref, **kw):
    prob = hydrogen_problem(**kw)
    ham = oracle_hamiltonian(prob)
    nang, N = prob.psi.GetRepresentation().GetFullShape()
    return prob, ham, ref.RefHamiltonian(oracle_terms(prob), nang, N, ham.kb)


def test_ref_bandnh_multiply_equals_oracle(ref):
    """The generated Diag/Simp BandNH kernels (one zgbmv per angular pair) equal the oracle's
    multiply of every consolidated potential, and the golden H psi."""
    g = golden("hydrogen_small.npz")
    prob, ham, rh = _model(ref)
    t = float(g["t"])
    assert relerr(rh.apply_H(g["psi"], t), ham.apply_H(g["psi"], t)) < 1e-14
    assert relerr(rh.apply_H(g["psi"], t), g["Hpsi"]) < 1e-14


def test_ref_pamp_and_cayley_reproduce_golden_steps(ref):
    """The golden pAMP and Crank-Nicolson steps (the GPU tests' reference values) equal the
    steps of the reference's own pAMP<cplx> and GMRES<cplx> driven as PamPropagator and
    CayleyPropagator drive them."""
    g = golden("hydrogen_small.npz")
    prob, ham, rh = _model(ref)
    t, dt = float(g["t"]), float(g["dt"])
    pam = ref.RefPam(rh, ham.overlap, 20, True)
    assert relerr(pam.step(g["psi"], t, dt), g["pamp"]) < 1e-13
    assert pam.last_error < 1e-20
    cay = OracleCayley(ham, dt, [0], 20, 1e-13)
    rc = ref.RefCayley(rh, ham.overlap, cay.prec, 20, 1e-13)
    assert relerr(rc.step(g["psi"], t, dt), g["cayley"]) < 1e-13


def test_ref_pamp_and_cayley_steps_equal_oracle_over_a_pulse(ref):
    """50 steps in the field (t from 2.5): the oracle restatements and the reference's
    templates stay together (relative 1e-12, infidelity 1e-24), with the same GMRES
    iteration counts."""
    g = golden("hydrogen_small.npz")
    prob, ham, rh = _model(ref)
    dt = 0.01
    op_pam, rf_pam = OraclePam(ham, 20, True), ref.RefPam(rh, ham.overlap, 20, True)
    op_cay = OracleCayley(ham, dt, [0], 20, 1e-12)
    rf_cay = ref.RefCayley(rh, ham.overlap, op_cay.prec, 20, 1e-12)
    a = b = c = d = g["psi"]
    for n in range(50):
        t = 2.5 + n * dt
        a, b = op_pam.step(a, t, dt), rf_pam.step(b, t, dt)
        c, d = op_cay.step(c, t, dt), rf_cay.step(d, t, dt)
        assert op_cay.last_iterations == rf_cay.last_iterations
    S = ham.overlap.S
    assert relerr(a, b) < 1e-12 and infidelity(b, a, S) < 1e-24
    assert relerr(c, d) < 1e-12 and infidelity(d, c, S) < 1e-24


def test_ref_gmres_equals_oracle_gmres(ref):
    """One preconditioned Crank-Nicolson solve at the pAMP model's size (lmax 10, 150
    B-splines): same solution, same number of operator applications."""
    prob, ham, rh = _model(ref, lmax=10, nbsplines=150, rmax=100.0)
    nang, N = ham.nang, ham.N
    dt, tt = 0.01, 5.0
    cay = OracleCayley(ham, dt, [0], 20, 1e-12)
    rng = np.random.default_rng(8)
    psi = rng.normal(size=(nang, N)) + 1j * rng.normal(size=(nang, N))
    op = lambda v: cay.prec.solve(cay.multiply_SpH(v.reshape(nang, N), 0.5j * dt, tt)).ravel()
    b = cay.prec.solve(cay.multiply_SpH(psi, -0.5j * dt, tt)).ravel()
    x_or, err_or, k_or = gmres_solve(op, b, 20, 1e-12)
    x_rf, err_rf, ops = ref.RefGmresSolver(nang * N, 20, 1e-12, op).solve(b)
    assert relerr(x_rf, x_or) < 1e-12
    # same count; the final least-squares estimates sit at the rounding floor (QR in zgels,
    # SVD in numpy's lstsq), both below the tolerance
    assert ops == k_or and err_rf <= 1e-12 and err_or <= 1e-12


def test_ref_piram_on_its_own_test_matrix(ref):
    """The reference's pIRAM on its own fixture (qdotmatrix.dat / init.dat as piramtest.cpp
    runs it: basis 50, 5 eigenvalues, 10 restarts) and the oracle's pIRAM give the same Ritz
    values wherever the reference's convergence estimate has converged; they differ only on
    the slower member of a degenerate pair, where the two restart sequences part (the oracle
    continues an invariant subspace with a random vector). With 40 restarts the reference
    reaches all five lowest eigenvalues of the dense decomposition."""
    g = golden("qdot_piram.npz")
    n = int(g["rows"].max()) + 1
    A = np.zeros((n, n))
    np.add.at(A, (g["rows"].astype(int), g["cols"].astype(int)), g["vals"])
    op = lambda v: A @ v
    start = g["init"].astype(complex)
    ev_rf, vec_rf, conv, rs_rf, _ = ref.ref_piram(op, start, 50, 5, 0.0, 10)
    ev_or, vec_or, rs_or, _ = piram_solve(op, start, 50, 5, 0.0, 10)
    order = np.argsort(ev_rf.real)
    ev_rf, conv, vec_rf = ev_rf[order], conv[order], vec_rf[order]
    assert rs_rf == rs_or == 10
    done = conv < 1e-9
    assert done.sum() >= 3
    assert np.max(np.abs(ev_rf[done] - ev_or[done])) < 1e-9
    assert abs(ev_rf[0] - 1.0) < 1e-10 and abs(ev_rf[1] - g["lowest5"][1]) < 1e-10
    for i in np.flatnonzero(done):
        v = vec_rf[i]
        assert np.linalg.norm(A @ v - ev_rf[i] * v) < 1e-6 * np.linalg.norm(v)
    ev_rf, _, _, _, _ = ref.ref_piram(op, start, 50, 5, 0.0, 40)
    assert np.max(np.abs(np.sort_complex(ev_rf) - g["lowest5"])) < 1e-7


def test_ref_shift_invert_ground_state(ref):
    """Ground state of the pAMP model (lmax 10, 150 B-splines) by the reference's pIRAM in
    inverse-iteration ordering on (H + 0.7 S)^-1 S (seeded start vector 1234): E = -1/2, the
    oracle's eigenvalue and state."""
    from oracle.operators import BandLU
    prob, ham, rh = _model(ref, lmax=10, nbsplines=150, rmax=100.0)
    nang, N = ham.nang, ham.N
    lu = BandLU(ham.overlap_rows, [ham.terms[0]], nang, N, ham.kb, 0.7, 1.0)
    op = lambda v: lu.solve(ham.overlap.multiply(v.reshape(nang, N))).ravel()
    start = np.random.default_rng(1234).uniform(size=nang * N).astype(complex)
    ev_rf, vec_rf, conv, _, _ = ref.ref_piram(op, start, 20, 2, 1e-12, 50, largest_abs=True)
    ev_or, vec_or, _, _ = piram_solve(op, start, 20, 2, 1e-12, 50, largest_abs=True)
    lam_rf = -0.7 + 1.0 / ev_rf
    assert abs(lam_rf[0] + 0.5) < 1e-10
    assert abs(ev_rf[0] - ev_or[0]) < 1e-10
    assert infidelity(vec_or[0].reshape(nang, N), vec_rf[0].reshape(nang, N), ham.overlap.S) < 1e-18


def test_full_length_runs_pinned_to_reference_templates():
    """The full-length fixtures hold, beside the oracle's final states, the final states of
    the same runs stepped by the reference's own pAMP and GMRES templates: they agree."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    for name in ("run_cayley_l40.npz", "run_pamp_l10.npz"):
        g = np.load(os.path.join(path, name))
        assert "psi_oracle" in g, name
        S = None
        assert relerr(g["psi"], g["psi_oracle"]) < 1e-10, name
        assert infidelity(g["psi"], g["psi_oracle"], S) < 1e-18, name
