"""Ensemble stepping (one graph launch for many members) against members stepped alone."""
import numpy as np
import pytest

from tests.helpers import hydrogen_problem, oracle_hamiltonian, relerr

pytestmark = pytest.mark.gpu


def _members(precision, fused=True):
    specs = [dict(lmax=3, nbsplines=40, rmax=40.0, amplitude=0.05),
             dict(lmax=5, nbsplines=33, rmax=30.0, amplitude=0.08, wavelength_nm=400.0),
             dict(lmax=2, nbsplines=55, rmax=50.0, amplitude=0.02, wavelength_nm=1600.0)]
    probs = []
    for k, sp in enumerate(specs):
        p = hydrogen_problem(propagator="CayleyPropagatorGPU", precision=precision, gmres_tolerance=1e-12, **sp)
        p.Propagator.FusedStep = fused
        p.SetupStep(skipWavefunctionSetup=True)
        rng = np.random.default_rng(100 + k)
        shape = p.psi.GetRepresentation().GetFullShape()
        psi = rng.normal(size=shape) + 1j * rng.normal(size=shape)
        p.psi.SetData(psi / np.linalg.norm(psi))
        p.PropagatedTime = 1.0
        probs.append(p)
    return probs


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_ensemble_matches_single_members(gpu, precision):
    from pyprop_gb300.ensemble import CayleyEnsembleGPU
    # the ensemble graph runs the multi-kernel step of every member: members stepped alone on
    # that step agree to rounding; mixed-precision members on the single-kernel step agree
    # to the GMRES tolerance
    alone = _members(precision, fused=False)
    alone_fused = _members(precision) if precision == "fp32" else []
    together = _members(precision)
    for _ in range(3):
        for p in alone + alone_fused:
            p.AdvanceStep()
    ens = CayleyEnsembleGPU(together)
    for _ in range(3):
        ens.AdvanceStep()
    stats = ens.Stats()
    for a, b, st in zip(alone, together, stats):
        assert relerr(b.psi.numpy(), a.psi.numpy()) < 1e-13
        assert st["Iterations"] >= 1
        assert abs(a.PropagatedTime - b.PropagatedTime) < 1e-12
    for a, b in zip(alone_fused, together):
        assert a.Propagator.Fused
        assert relerr(b.psi.numpy(), a.psi.numpy()) < 1e-10


def test_ensemble_member_against_oracle(gpu):
    from pyprop_gb300.ensemble import CayleyEnsembleGPU
    from oracle.propagators import OracleCayley
    together = _members("fp64")
    psi0 = [p.psi.numpy() for p in together]
    ens = CayleyEnsembleGPU(together)
    for _ in range(2):
        ens.AdvanceStep()
    for p, start in zip(together, psi0):
        ham = oracle_hamiltonian(p)
        cay = OracleCayley(ham, 0.01, [0], 20, 1e-13)
        ref = cay.step(cay.step(start, 1.0, 0.01), 1.01, 0.01)
        assert relerr(p.psi.numpy(), ref) < 1e-10


def _pamp_members(precision, with_field=True):
    specs = [dict(lmax=3, nbsplines=40, rmax=40.0, amplitude=0.05 if with_field else 0.0),
             dict(lmax=5, nbsplines=33, rmax=30.0, amplitude=0.08 if with_field else 0.0, wavelength_nm=400.0),
             dict(lmax=2, nbsplines=55, rmax=50.0, amplitude=0.02 if with_field else 0.0, wavelength_nm=1600.0)]
    probs = []
    for k, sp in enumerate(specs):
        p = hydrogen_problem(propagator="PamPropagatorGPU", precision=precision, **sp)
        p.SetupStep(skipWavefunctionSetup=True)
        rng = np.random.default_rng(200 + k)
        shape = p.psi.GetRepresentation().GetFullShape()
        psi = rng.normal(size=shape) + 1j * rng.normal(size=shape)
        p.psi.SetData(psi / np.linalg.norm(psi))
        p.PropagatedTime = 1.0
        probs.append(p)
    return probs


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_pamp_ensemble_matches_single_members(gpu, precision):
    """pAMP members of different sizes and fields advanced by one graph launch per step (the
    m x m exponentials on the device, Pade of order 6) against the same members stepped alone
    (host exponential), and a second batch built on the same members after the first is
    destroyed."""
    from pyprop_gb300.ensemble import PamEnsembleGPU
    alone = _pamp_members(precision)
    together = _pamp_members(precision)
    for _ in range(4):
        for p in alone:
            p.AdvanceStep()
    ens = PamEnsembleGPU(together)
    for _ in range(4):
        ens.AdvanceStep()
    stats = ens.Stats()
    tol = 1e-11 if precision == "fp64" else 1e-6
    for a, b, st in zip(alone, together, stats):
        assert relerr(b.psi.numpy(), a.psi.numpy()) < tol, (precision, relerr(b.psi.numpy(), a.psi.numpy()))
        assert st["Iterations"] == 20
        assert 0.0 <= st["ErrorEstimate"] < 1e-6
        assert abs(a.PropagatedTime - b.PropagatedTime) < 1e-12
    del ens
    # members step alone again (their own slots back) and agree with the lone copies
    for p, q in zip(alone, together):
        p.AdvanceStep()
        q.AdvanceStep()
        assert relerr(q.psi.numpy(), p.psi.numpy()) < tol
