"""Two-electron (helium) model on the CPU: Clebsch-Gordan coefficients and known energies.

The operator is assembled by the oracle's rank-3 storage loops from the potentials this
package generates (coupled spherical harmonics x B-splines x B-splines, the terms of
examples/tensor/helium_stabilization/config.ini); its lowest generalized eigenvalue is
checked against known helium energies.
"""
import numpy as np
import pytest
import scipy.linalg as sl

from pyprop_gb300.spherical import clebsch_gordan
from tests.helpers import helium_dense, helium_problem

# s-wave (l1 = l2 = 0) limit of the helium ground state, and the nonrelativistic exact energy
S_LIMIT = -2.879028767
EXACT = -2.903724377


def test_clebsch_gordan_known_values_and_orthogonality():
    assert abs(clebsch_gordan(1, 1, 0, 0, 0, 0) + 1 / np.sqrt(3)) < 1e-14
    assert abs(clebsch_gordan(1, 1, 1, -1, 0, 0) - 1 / np.sqrt(3)) < 1e-14
    assert abs(clebsch_gordan(1, 1, 1, 0, 1, 1) - 1 / np.sqrt(2)) < 1e-14
    assert abs(clebsch_gordan(2, 1, 0, 0, 1, 0) + np.sqrt(2 / 5)) < 1e-14
    for j1, j2 in [(1, 1), (2, 1), (3, 2)]:
        for M in range(-(j1 + j2), j1 + j2 + 1):
            Js = range(abs(j1 - j2), j1 + j2 + 1)
            ms = [(m1, M - m1) for m1 in range(-j1, j1 + 1) if abs(M - m1) <= j2]
            C = np.array([[clebsch_gordan(j1, j2, m1, m2, J, M) for m1, m2 in ms] for J in Js if abs(M) <= J])
            assert np.allclose(C @ C.T, np.eye(C.shape[0]), atol=1e-13)


def _ground(lmax, N, rmax, q=10):
    prob = helium_problem(lmax=lmax, nbsplines=N, rmax=rmax, quad_order_additional=q)
    H, S3, _ = helium_dense(prob)
    assert np.abs(H - H.conj().T).max() < 1e-12
    return sl.eigh(H, S3, eigvals_only=True, subset_by_index=[0, 1])


def test_helium_s_wave_limit():
    w = _ground(0, 16, 15.0)
    assert abs(w[0] - S_LIMIT) < 5e-4, w


def test_helium_partial_waves_converge_from_above():
    e = [_ground(l, 16 if l < 2 else 20, 15.0 if l < 2 else 20.0)[0] for l in (0, 1, 2)]
    assert e[0] > e[1] > e[2] > EXACT, e
    # the reference's own table (doc/test_and_benchmark.tex:41) gives -2.903586 at lmax = 5;
    # l <= 2 is within 1e-3 of it
    assert abs(e[2] - (-2.903586)) < 1e-3, e


def test_laser_coupling_factors():
    from pyprop_gb300.spherical import (CoupledIndex, DefaultCoupledIndexIterator, laser_length_factors,
                                        rule_linear_polarized_field)
    # s -> p of electron 1 with electron 2 in s: <Y00|Y10|Y10> = 1/sqrt(4 pi)
    I1, I2 = laser_length_factors(CoupledIndex(0, 0, 0, 0), CoupledIndex(1, 0, 1, 0))
    assert abs(I1 - 1 / np.sqrt(4 * np.pi)) < 1e-14 and I2 == 0.0
    # the factors are evaluated on the selection rule's pairs only (the m-sum alone does not
    # enforce the spectator electron's delta); there they are symmetric, and the spectator's
    # factor vanishes
    idx = list(DefaultCoupledIndexIterator(3, L=[0, 1, 2, 3]))
    for a in idx:
        for b in idx:
            if not rule_linear_polarized_field(a, b):
                continue
            f, g = laser_length_factors(a, b), laser_length_factors(b, a)
            assert abs(f[0] - g[0]) < 1e-14 and abs(f[1] - g[1]) < 1e-14
            if a.l1 == b.l1:
                assert abs(f[0]) < 1e-14
            if a.l2 == b.l2:
                assert abs(f[1]) < 1e-14


def test_helium_with_laser_term_is_hermitian():
    prob = helium_problem(lmax=1, nbsplines=12, rmax=12.0, L=(0, 1), amplitude=0.1, frequency=1.0, pulse_duration=2.0)
    H, S3, terms = helium_dense(prob)
    assert np.abs(H - H.conj().T).max() < 1e-12
    pots = prob.Propagator.BasePropagator.PotentialList
    # factorized terms are not consolidated: 5 field-free terms, then the laser coupling
    assert [p.IsTimeDependent for p in pots] == [False] * 5 + [True]
    assert all(p.Factors is not None for p in pots)
    plain = helium_problem(lmax=1, nbsplines=12, rmax=12.0, L=(0, 1), amplitude=0.1, frequency=1.0,
                           pulse_duration=2.0, factorize=False).Propagator.BasePropagator.PotentialList
    assert len(plain) == 3 and [p.IsTimeDependent for p in plain] == [False, False, True]


def test_r12_closed_form_matches_m_sum():
    """The 6j closed form of the multipole coefficient equals the reference's m-sum over four
    Clebsch-Gordan coefficients (coupledspherical.cpp:63-92) on random coupled states."""
    from pyprop_gb300.spherical import CoupledIndex, r12_angular_factor, r12_angular_sum, r12_multipoles
    rng = np.random.default_rng(11)
    n = 0
    for _ in range(200):
        L = int(rng.integers(0, 5))
        while True:
            l = [int(v) for v in rng.integers(0, 6, size=4)]
            if abs(l[0] - l[1]) <= L <= l[0] + l[1] and abs(l[2] - l[3]) <= L <= l[2] + l[3]:
                break
        a, b = CoupledIndex(l[0], l[1], L, 0), CoupledIndex(l[2], l[3], L, 0)
        for l3 in r12_multipoles(a, b):
            assert abs(r12_angular_factor(a, b, l3) - r12_angular_sum(a, b, l3)) < 1e-13
            n += 1
    assert n > 300


def test_factored_terms_expand_to_the_per_pair_data():
    """Every two-electron term kept as angular coefficients x radial factors expands to the
    reference-layout data that the per-pair generation produces (same geometries,
    quadrature and differentiation), and the oracle's point-wise factored multiply equals the
    per-pair tensor multiply."""
    from collections import defaultdict
    from oracle.operators import TermOracle, factored_multiply
    pa = helium_problem(lmax=2, L=[0, 1], nbsplines=16, rmax=15.0, amplitude=0.05)
    pb = helium_problem(lmax=2, L=[0, 1], nbsplines=16, rmax=15.0, amplitude=0.05, factorize=False)
    la = pa.Propagator.BasePropagator.PotentialList
    lb = pb.Propagator.BasePropagator.PotentialList
    assert all(p.Factors is not None for p in la)
    assert all(p.Factors is None for p in lb)
    assert any(p.Factors.nfactors >= 4 for p in la)  # the multipoles l3 = 0..4

    def key(p):
        g0 = p.GeometryList[0].GetBasisPairs()
        return tuple(g.GetStorageId() for g in p.GeometryList), g0.tobytes(), p.IsTimeDependent

    sa, sb = defaultdict(lambda: 0), defaultdict(lambda: 0)
    for p in la:
        sa[key(p)] = sa[key(p)] + p.PotentialData
    for p in lb:
        sb[key(p)] = sb[key(p)] + p.PotentialData
    assert set(sa) == set(sb)
    for k in sb:
        assert np.abs(sa[k] - sb[k]).max() <= 1e-13 * np.abs(sb[k]).max()
    repr_ = pa.psi.GetRepresentation()
    shape = repr_.GetFullShape()
    rng = np.random.default_rng(2)
    x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    scales = [1.0] + [0.7 if p.IsTimeDependent else 1.0 for p in la]
    y1 = factored_multiply([(p.Factors, 1 + i) for i, p in enumerate(la)], scales, x, np.zeros(shape, complex))
    y2 = np.zeros(shape, complex)
    for p in lb:
        t = TermOracle("_".join(g.GetStorageId() for g in p.GeometryList), p.PotentialData,
                       [g.GetBasisPairs() for g in p.GeometryList], None, None, repr_.kb, shape=shape)
        t.multiply(x, y2, 0.7 if p.IsTimeDependent else 1.0)
    assert np.linalg.norm(y1 - y2) < 1e-12 * np.linalg.norm(y2)


def test_fast_diagonalization_inverts_the_separable_channel_block():
    """(V1 x V2) D (V1 x V2)^T, from the generalized eigenvectors of the one-electron radial
    Hamiltonians, is the inverse of cS S x S + cH (h_l1 x S + S x h_l2) (the separable part of
    a channel block of the Cayley matrix)."""
    import scipy.linalg as sl
    from pyprop_gb300.propagator import TwoElectronFastDiagonalizationPreconditioner
    prob = helium_problem(lmax=1, nbsplines=14, rmax=12.0)
    repr_ = prob.psi.GetRepresentation()
    pre = TwoElectronFastDiagonalizationPreconditioner(prob.psi)
    pre.Z, pre.Mass = 2.0, 1.0
    S = repr_.radial.BSplineObject.dense(repr_.overlap_rows)
    cS, cH = 1.0, 0.5j * 0.01
    h0, h1 = pre._dense(0), pre._dense(1)
    w0, v0 = sl.eigh(h0, S)
    w1, v1 = sl.eigh(h1, S)
    M = cS * np.kron(S, S) + cH * (np.kron(h0, S) + np.kron(S, h1))
    D = 1.0 / (cS + cH * (w0[:, None] + w1[None, :]))
    Minv = np.kron(v0, v1) @ np.diag(D.ravel()) @ np.kron(v0, v1).T
    assert np.abs(Minv @ M - np.eye(M.shape[0])).max() < 1e-10


def test_batched_band_elements_match_row_by_row():
    """The projection of many grid functions at once (the radial factors of two-electron terms)
    equals the projection of each row alone."""
    from tests.helpers import hydrogen_problem
    bs = hydrogen_problem(lmax=1, nbsplines=30, rmax=20.0).psi.GetRepresentation().radial.BSplineObject
    rng = np.random.default_rng(0)
    f = rng.standard_normal((5, 3, len(bs.grid)))
    for d in (0, 2):
        a = bs.band_elements(f, d)
        b = np.stack([np.stack([bs.band_elements(f[i, j], d) for j in range(3)]) for i in range(5)])
        assert np.abs(a - b).max() <= 1e-13 * np.abs(b).max()
