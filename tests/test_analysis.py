"""Two-electron analysis on the host: the oracle's projection loops, single-electron radial
states, ionization boxes (CPU only)."""
import numpy as np

from oracle import analysis as ora


def test_oracle_projection_equals_matrix_form_and_removal_projects_out():
    rng = np.random.default_rng(2)
    nang, N, n1, n2 = 3, 9, 4, 5
    psi = rng.normal(size=(nang, N, N)) + 1j * rng.normal(size=(nang, N, N))
    V1 = rng.normal(size=(N, n1)) + 1j * rng.normal(size=(N, n1))
    V2 = rng.normal(size=(N, n2)) + 1j * rng.normal(size=(N, n2))
    idx = [0, 2]
    proj = ora.projection(V1, V2, psi, idx)
    for q, a in enumerate(idx):
        assert np.allclose(proj[q], V1.conj().T @ psi[a] @ V2.conj(), atol=1e-12)
    # with orthonormal states (Euclidean) the removal leaves nothing to project
    Q1, _ = np.linalg.qr(V1)
    Q2, _ = np.linalg.qr(V2)
    out = ora.remove(Q1, Q2.conj(), psi.copy(), idx, psi.copy())
    assert np.max(np.abs(ora.projection(Q1, Q2.conj(), out, idx))) < 1e-12
    pop = ora.population(V1, V2, psi, idx)
    assert abs(sum(p for _, _, p in pop) - np.sum(np.abs(proj) ** 2)) < 1e-9


def test_radial_eigenstates_are_hydrogenic():
    """He+ (Z = 2) radial states in a 60-spline basis on [0, 40]: E = -Z^2 / 2n^2 for the
    lowest states of each l, unit S-norm."""
    import pyprop_gb300 as pp
    from pyprop_gb300.analysis import SetupRadialEigenstates
    from pyprop_gb300.workloads import hydrogen
    prob = pp.Problem(pp.LoadString(hydrogen(lmax=0, nbsplines=60, rmax=40.0)))
    bs = prob.psi.GetRepresentation().radial.BSplineObject
    E, V = SetupRadialEigenstates(bs, 2.0, 2)
    assert abs(E[0][0] + 2.0) < 1e-8 and abs(E[0][1] + 0.5) < 1e-6 and abs(E[1][0] + 0.5) < 1e-6
    assert abs(E[2][0] + 2.0 / 9.0) < 1e-5
    S = bs.dense(bs.overlap_band())
    assert np.allclose(V[1].conj().T @ S @ V[1], np.eye(V[1].shape[1]), atol=1e-9)


def test_ionization_boxes_regions():
    from pyprop_gb300.potentials import DoubleIonizationBox, SingleIonizationBox
    r1 = np.array([1.0, 30.0, 30.0, 1.0, 15.0])[:, None]
    r2 = np.array([1.0, 2.0, 30.0, 25.0, 15.0])[None, :]
    s, d = SingleIonizationBox(), DoubleIonizationBox()
    vs = s.GetPotentialValue((np.zeros(1)[:, None], r1, r2))
    vd = d.GetPotentialValue((np.zeros(1)[:, None], r1, r2))
    assert vs[1, 1] == 1.0 and vs[0, 3] == 1.0 and vs[2, 2] == 0.0 and vs[0, 0] == 0.0
    assert vd[2, 2] == 1.0 and vd[1, 1] == 0.0 and vd[4, 4] == 0.0
