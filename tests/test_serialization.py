"""Checkpoints: wavefunctions and tensor potentials saved to and loaded from .npz archives
(the layout of pyprop/serialization/*HDF.py without HDF5), on host buffers (no GPU)."""
import numpy as np
import pytest


def _cpu_psi(prob, data):
    import torch
    prob.psi.data = torch.as_tensor(data, dtype=torch.complex128)
    return prob.psi


def test_wavefunction_round_trip_and_shape_check(tmp_path):
    import pyprop_gb300 as pp
    from tests.helpers import hydrogen_problem
    prob = hydrogen_problem(lmax=2, nbsplines=20, rmax=20.0)
    shape = prob.psi.GetRepresentation().GetFullShape()
    rng = np.random.default_rng(0)
    data = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    _cpu_psi(prob, data)
    f = str(tmp_path / "run.npz")
    pp.SaveWavefunction(f, "/group/psi", prob.psi, prob.Config)
    pp.SaveWavefunction(f, "/other", prob.psi)
    _cpu_psi(prob, np.zeros(shape))
    pp.LoadWavefunction(f, "/group/psi", prob.psi)
    assert np.array_equal(prob.psi.GetData().numpy(), data)
    assert "[Propagation]" in pp.GetConfigText(f, "/group/psi")
    assert pp.GetConfigText(f, "/other") is None
    other = hydrogen_problem(lmax=3, nbsplines=20, rmax=20.0)
    _cpu_psi(other, np.zeros(other.psi.GetRepresentation().GetFullShape()))
    with pytest.raises(ValueError):
        pp.LoadWavefunction(f, "/group/psi", other.psi)
    with pytest.raises(ValueError):
        pp.SaveWavefunction(f, "/", prob.psi)


def test_checkpoint_resumes_time(tmp_path):
    from tests.helpers import hydrogen_problem
    prob = hydrogen_problem(lmax=1, nbsplines=20, rmax=20.0)
    shape = prob.psi.GetRepresentation().GetFullShape()
    data = np.arange(np.prod(shape)).reshape(shape) * (1 + 0.5j)
    _cpu_psi(prob, data)
    prob.PropagatedTime = 3.25
    f = str(tmp_path / "ck.npz")
    prob.SaveCheckpoint(f)
    again = hydrogen_problem(lmax=1, nbsplines=20, rmax=20.0)
    _cpu_psi(again, np.zeros(shape))
    assert again.LoadCheckpoint(f) == 3.25
    assert np.array_equal(again.psi.GetData().numpy(), data)


def test_tensor_potentials_round_trip_with_basis_pair_check(tmp_path):
    """Per-pair (hydrogen) and factorized (two-electron) potentials come back identical; a
    potential with other basis pairs is refused (TensorPotentialHDF.py:140-157)."""
    import pyprop_gb300 as pp
    from tests.helpers import helium_problem, hydrogen_problem
    f = str(tmp_path / "pots.npz")
    h = hydrogen_problem(lmax=3, nbsplines=20, rmax=20.0)
    he = helium_problem(lmax=2, L=[0, 1], nbsplines=14, rmax=12.0, amplitude=0.05)
    hp = h.Propagator.BasePropagator.PotentialList
    hep = he.Propagator.BasePropagator.PotentialList
    for k, p in enumerate(hp):
        pp.SaveTensorPotential(f, "/hydrogen/%d" % k, p)
    r12 = [p for p in hep if "ElectronicCoupling" in p.Name][0]
    pp.SaveTensorPotential(f, "/helium/r12", r12)
    for k, p in enumerate(hp):
        ref = p.PotentialData.copy()
        p.PotentialData = None
        pp.LoadTensorPotential(f, "/hydrogen/%d" % k, p)
        assert np.array_equal(p.PotentialData, ref)
    ref = r12.PotentialData.copy()
    stencil = r12.Factors.stencil.copy()
    r12.Factors = None
    r12.PotentialData = None
    pp.LoadTensorPotential(f, "/helium/r12", r12)
    assert np.array_equal(r12.Factors.stencil, stencil)
    assert np.abs(r12.PotentialData - ref).max() == 0.0
    dip = [p for p in hp if p.IsTimeDependent][0]
    with pytest.raises(ValueError):
        pp.LoadTensorPotential(f, "/hydrogen/0", dip)  # other pairs
