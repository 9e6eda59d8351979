"""Host-side setup: breakpoints, B-spline matrix elements, tensor-potential layout, configs."""
import numpy as np
import pytest
import scipy.interpolate as si
import scipy.linalg as sl

from pyprop_gb300 import bspline as B
from pyprop_gb300.tensorpotential import bandnh_pairs, packed_band_pairs
from pyprop_gb300.spherical import dipole_selection_pairs, DefaultCoupledIndexIterator, ReducedSphericalTools
from tests.helpers import hydrogen_problem, oracle_hamiltonian


@pytest.mark.parametrize("rmax,total,N", [(100.0, 147, 150), (400.0, 597, 600)])
def test_exponential_linear_grid_sizes(rmax, total, N):
    rp, n = B.exponential_linear_params_for(0.0, rmax, total)
    bps = B.exponential_linear_breakpoints(0.0, rp, rmax, n, 2.0)
    assert len(bps) == total
    bs = B.BSplineBasis(7, bps, "zero", 0)
    assert bs.NumberOfBSplines == N
    # breakpoint rule of breakpointsequences.py:82-101: inner exponential, then uniform steps
    d = np.diff(bps[n - 1:])
    assert np.allclose(d, d[0])


def test_knots_and_continuity():
    bs = B.BSplineBasis(4, B.linear_breakpoints(0.0, 1.0, 6), "vanilla")
    assert list(bs.knots[:4]) == [0.0] * 4 and list(bs.knots[-4:]) == [1.0] * 4
    assert bs.NumberOfBSplines == len(bs.knots) - 4
    bz = B.BSplineBasis(4, B.linear_breakpoints(0.0, 1.0, 6), "zero")
    assert bz.NumberOfBSplines == bs.NumberOfBSplines - 2


def test_gauss_legendre():
    x, w = B.gauss_legendre(7)
    assert np.all(np.diff(x) > 0)
    xr, wr = np.polynomial.legendre.leggauss(7)
    assert np.allclose(x, xr, atol=1e-14) and np.allclose(w, wr, atol=1e-14)


def _scipy_splines(bs):
    """scipy B-splines on the knot vector padded to full end multiplicity; spline i + 1 of
    the padded vector is this basis' spline i ('zero' continuity drops the end splines)."""
    k = bs.MaxSplineOrder
    t = np.concatenate([[bs.knots[0]], bs.knots, [bs.knots[-1]]])
    out = []
    for i in range(bs.NumberOfBSplines):
        c = np.zeros(len(t) - k)
        c[i + 1] = 1.0
        out.append(si.BSpline(t, c, k - 1, extrapolate=False))
    return out


def test_matrix_elements_against_independent_bsplines():
    """Overlap, second-derivative and r-weighted elements vs scipy B-splines integrated with
    a 20-point rule per interval (exact for these polynomial integrands)."""
    bps = B.exponential_linear_breakpoints(0.0, 5.0, 20.0, 8, 2.0)
    bs = B.BSplineBasis(7, bps, "zero", 0)
    sp = _scipy_splines(bs)
    x, w = np.polynomial.legendre.leggauss(20)
    a, b = np.asarray(bps[:-1])[:, None], np.asarray(bps[1:])[:, None]
    X = ((x + 1) * (b - a) / 2 + a).ravel()
    W = ((b - a) / 2 * w).ravel()
    vals = np.array([np.nan_to_num(s(X)) for s in sp])
    d2 = np.array([np.nan_to_num(s.derivative(2)(X)) for s in sp])
    kb = 6
    for deriv, f, right in [(0, np.ones_like(X), vals), (2, np.ones_like(X), d2), (0, X, vals)]:
        ref = (vals * W * f) @ right.T
        band = bs.band_elements(np.interp(bs.grid, X, f) if f is not X else bs.grid, deriv)
        dense = bs.dense(band)
        assert np.max(np.abs(dense - ref)) < 1e-12 * np.max(np.abs(ref))
        if deriv == 2:  # zero boundary values make <B_i|B_j''> symmetric
            assert np.allclose(dense, dense.T, atol=1e-10 * np.abs(dense).max())


def test_overlap_spd_and_partition():
    bs = B.BSplineBasis(7, B.linear_breakpoints(0.0, 10.0, 20), "vanilla")
    S = bs.dense(bs.overlap_band()).real
    assert np.all(np.linalg.eigvalsh(S) > 0)
    Bt = bs.evaluate(np.linspace(0.01, 9.99, 50))
    assert np.allclose(Bt.sum(axis=0), 1.0)


def test_bandnh_layout():
    pairs = bandnh_pairs(10, 2)
    b = 5
    for i in range(10):
        for j in range(max(0, i - 2), min(10, i + 3)):
            assert tuple(pairs[j * b + (2 + i - j)]) == (i, j)
    assert len(packed_band_pairs(10, 3)) == 2 * 10 * 3 - 3 * 2 - 10


def test_dipole_pairs_and_coupling():
    pairs = dipole_selection_pairs(4)
    assert pairs.tolist() == [[0, 1], [1, 0], [1, 2], [2, 1], [2, 3], [3, 2]]
    tools = ReducedSphericalTools(10, 0)
    vals = np.cos(tools.ThetaGrid)
    c = tools.project_pairs(vals, dipole_selection_pairs(11))
    for (l, lp), v in zip(dipole_selection_pairs(11), c):
        lo = min(l, lp)
        assert abs(v - (lo + 1) / np.sqrt((2 * lo + 1) * (2 * lo + 3))) < 1e-14


def test_coupled_index_iterator():
    idx = list(DefaultCoupledIndexIterator(lmax=10, L=range(6), M=[0]))
    assert len(idx) == 291
    idx16 = list(DefaultCoupledIndexIterator(lmax=16, L=range(9), M=[0]))
    assert len(idx16) == 1017
    assert (idx[0].L, idx[0].l1, idx[0].l2) == (0, 0, 0)


def test_hydrogen_spectrum_config1_grid():
    """Assembled operator of the N=150, lmax=10 grid: E_n = -1/(2 n^2)."""
    prob = hydrogen_problem(lmax=10, nbsplines=150, rmax=100.0)
    ham = oracle_hamiltonian(prob)
    names = [p.Name for p in prob.Propagator.BasePropagator.PotentialList]
    assert names[0] == "RadialKineticEnergy+AngularKineticEnergy+CoulombPotential"
    assert names[1] == "LaserPotential"
    from oracle.operators import dense_operator
    nang, N = 11, 150
    H = dense_operator(ham.terms, ham.scalings(0.0), nang, N)
    S = np.kron(np.eye(nang), ham.overlap.S)
    ev = sl.eigh(H, S, eigvals_only=True)
    assert abs(ev[0] + 0.5) < 1e-10
    assert abs(ev[1] + 0.125) < 1e-10 and abs(ev[2] + 0.125) < 1e-10


def test_config_eval_base_and_interpolation():
    import pyprop_gb300 as pp
    conf = pp.LoadString("""
[A]
x = 2.0
y = %(x)s * 3
[B]
base = "A"
z = x + y
f = LaserFunctionSimpleLength
""")
    assert conf.A.y == 6.0
    assert conf.B.z == 8.0 and conf.B.f is pp.LaserFunctionSimpleLength
    conf2 = pp.UpdateConfig(conf, [("A", "x", 5.0)])
    assert conf2.A.x == 5.0


def test_laser_time_function():
    from pyprop_gb300.potentials import LaserFunctionSimpleLength
    from pyprop_gb300.workloads import omega_for_wavelength

    class C:
        amplitude = 0.05
        pulse_duration = 10.0
        frequency = omega_for_wavelength(800.0)
    assert abs(C.frequency - 0.056954) < 1e-5
    assert LaserFunctionSimpleLength(C, 0.0) == 0.0
    assert LaserFunctionSimpleLength(C, 10.0) == 0.0
    t = 5.0
    assert abs(LaserFunctionSimpleLength(C, t) - 0.05 * np.cos(C.frequency * t)) < 1e-15
