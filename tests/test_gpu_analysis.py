"""Two-electron analysis on the GPU against the oracle: projections on products of radial
states (and their removal), ionization-box expectation values, completeness of the
product-state populations."""
import numpy as np
import pytest

from tests.helpers import helium_problem, relerr

pytestmark = pytest.mark.gpu

BOXES = """
[SingleIonizationBox]
classname = "SingleIonizationBox"
geometry0 = "Diagonal"
geometry1 = "banded-packed"
geometry2 = "banded-nonhermitian"
angular_rank = 0
radial_rank_1 = 1
radial_rank_2 = 2
inner_box_size = 5.0
width = 5.0

[DoubleIonizationBox]
classname = "DoubleIonizationBox"
geometry0 = "Diagonal"
geometry1 = "banded-packed"
geometry2 = "banded-nonhermitian"
angular_rank = 0
radial_rank_1 = 1
radial_rank_2 = 2
inner_box_size = 5.0
width = 5.0
"""


def _problem():
    import pyprop_gb300 as pp
    from pyprop_gb300.workloads import helium
    prob = pp.Problem(pp.LoadString(helium(lmax=1, L=(0, 1), nbsplines=16, rmax=15.0) + BOXES))
    prob.SetupStep(skipWavefunctionSetup=True)
    return prob


def _random_state(prob, seed):
    import torch
    shape = prob.psi.GetRepresentation().GetFullShape()
    rng = np.random.default_rng(seed)
    x = rng.normal(size=shape) + 1j * rng.normal(size=shape)
    prob.psi.GetData().copy_(torch.as_tensor(x, device="cuda"))
    prob.psi.Normalize()
    return prob.psi.numpy()


def test_projection_and_removal_match_oracle(gpu):
    """Projections of a weighted random state on He+ radial product states for every (l1, l2)
    pair equal the oracle's loops (1e-12 relative); removing them leaves a state whose
    projections vanish and which equals the oracle's removal."""
    from oracle import analysis as ora
    from pyprop_gb300.analysis import (CalculateProjectionRadialProductStates, GetLocalCoupledSphericalHarmonicIndices,
                                       RemoveProjectionRadialProductStates, SetupRadialEigenstates)
    prob = _problem()
    x = _random_state(prob, 1)
    repr_ = prob.psi.GetRepresentation()
    bs = repr_.GetRepresentation(1).BSplineObject
    E, V = SetupRadialEigenstates(bs, 2.0, 1)
    w = prob.psi.Copy()
    repr_.MultiplyIntegrationWeights(w)
    xw = w.numpy()
    out_ref = x.copy()
    for l1 in (0, 1):
        for l2 in (0, 1):
            idx = GetLocalCoupledSphericalHarmonicIndices(prob.psi, lambda c: c.l1 == l1 and c.l2 == l2)
            if not idx:
                continue
            V1, V2 = V[l1][:, :6], V[l2][:, 2:9]
            got = CalculateProjectionRadialProductStates(l1, V1, l2, V2, w.GetData(), idx)
            ref = ora.projection(V1, V2, xw, idx)
            assert relerr(got, ref) < 1e-12, (l1, l2)
            RemoveProjectionRadialProductStates(l1, V1, l2, V2, w.GetData(), idx, prob.psi.GetData())
            ora.remove(V1, V2, xw, idx, out_ref)
    assert relerr(prob.psi.numpy(), out_ref) < 1e-12
    w2 = prob.psi.Copy()
    repr_.MultiplyIntegrationWeights(w2)
    for l1 in (0, 1):
        for l2 in (0, 1):
            idx = GetLocalCoupledSphericalHarmonicIndices(prob.psi, lambda c: c.l1 == l1 and c.l2 == l2)
            if idx:
                left = CalculateProjectionRadialProductStates(l1, V[l1][:, :6], l2, V[l2][:, 2:9], w2.GetData(), idx)
                assert np.max(np.abs(left)) < 1e-12


def test_ionization_box_expectation_values_match_oracle(gpu):
    """<psi|box|psi> of the single- and double-ionization boxes (inner size and width 5 a.u.),
    evaluated on the GPU as TensorPotential.GetExpectationValue does, against psi^H V psi of
    the oracle's rank-3 storage loops over the same projected box."""
    from oracle.operators import TermOracle, dense_operator
    prob = _problem()
    x = _random_state(prob, 2)
    bp = prob.Propagator.BasePropagator
    repr_ = prob.psi.GetRepresentation()
    shape = repr_.GetFullShape()
    tmp = prob.psi.Copy()
    vals = {}
    for name in ("SingleIonizationBox", "DoubleIonizationBox"):
        pot = bp.GeneratePotential(prob.Config.GetSection(name))
        pot.SetupStep(0.0)
        got = pot.GetExpectationValue(prob.psi, tmp, 0.0, 0.0)
        term = TermOracle("_".join(g.GetStorageId() for g in pot.GeometryList), pot.PotentialData,
                          [g.GetBasisPairs() for g in pot.GeometryList], None, None, repr_.kb, shape=shape)
        Vd = dense_operator([term], [1.0], shape[0] * shape[1], shape[2])
        ref = np.vdot(x.ravel(), Vd @ x.ravel())
        assert abs(got - ref) < 1e-11 * max(1.0, abs(ref)), (name, got, ref)
        assert abs(ref.imag) < 1e-12 and 0.0 < ref.real < 1.0
        vals[name] = got.real
    assert vals["SingleIonizationBox"] > 0.0 and vals["DoubleIonizationBox"] > 0.0


def test_product_state_populations_are_complete(gpu):
    """With every radial eigenstate of He+ (bound and continuum) for l <= lmax, the bound,
    single- and double-ionization populations of a state add up to its S-norm squared."""
    from pyprop_gb300.analysis import ProductStateIonization
    prob = _problem()
    _random_state(prob, 3)
    pops = ProductStateIonization(prob.psi, 2.0, 1)
    total = pops["bound"] + pops["single"] + pops["double"]
    assert abs(total - pops["norm"]) < 1e-10 * pops["norm"], pops
    assert min(pops["bound"], pops["single"], pops["double"]) > 0.0
