"""pyprop_gb300 - GB300 (sm_103a) implementation of PyProp's propagation hot path.

The tensor-potential matvec over banded B-spline x spherical-harmonic ranks and the Krylov
loops that drive it (pAMP, Cayley/GMRES, pIRAM) run as hand-written CUDA kernels in
``libpyprop_gpu.so`` behind a C ABI (``include/pyprop_gpu.h``). This package keeps the
reference's Python-facing API: INI configs with evaluated values, ``Problem``,
``TensorPotential``, ``Wavefunction``, propagator and solver classes. There is no CPU
fallback.
"""
from __future__ import annotations

from . import config as _config
from .config import Config, Load, LoadString, ProjectNamespace, Section, UpdateConfig
from .potentials import (AngularKineticEnergyPotential, ComplexAbsorbingPotential, CoulombPotential,
                         DipoleLaserPotentialLength, KineticEnergyPotential, LaserFunctionFlatTop,
                         LaserFunctionLength, LaserFunctionSimpleLength, LaserFunctionVelocity, OverlapPotential,
                         SingleActiveElectronPotential, register_potential)
from .problem import InitBSpline, InitialConditionType, Problem, core
from .propagator import (BasisPropagator, BasisPropagatorGPU, BSplinePreconditioner, CayleyPropagator,
                         CayleyPropagatorGPU, PamPropagator, PamPropagatorGPU, RadialPreconditioner,
                         RadialTwoElectronPreconditionerIfpack, RadialTwoElectronPreconditionerSuperLU,
                         TwoElectronFastDiagonalizationPreconditioner, TwoElectronKroneckerPreconditioner)
from .serialization import (CheckBasisPairs, GetConfigText, LoadTensorPotential, LoadWavefunction,
                            SaveTensorPotential, SaveWavefunction)
from .solver import PiramSolver, PiramSolverGPU
from .spherical import DefaultCoupledIndexIterator

ProjectNamespace.update({
    name: obj for name, obj in dict(globals()).items() if not name.startswith("_")
})

__all__ = sorted(n for n in ProjectNamespace)
