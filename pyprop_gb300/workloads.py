"""Config files for the hydrogen-in-a-laser workloads the hot path is measured on.

One electron, reduced spherical harmonics (m = 0) x B-splines of order 7 on an
exponential-linear grid with 'zero' continuity, potentials kinetic (d^2/dr^2),
centrifugal l(l+1)/2r^2, Coulomb -1/r (no softening) and the length-gauge dipole
E(t) r cos(theta) with a sin^2 envelope (``LaserFunctionSimpleLength``). Each potential
section uses the reference's geometry and differentiation keys
(``examples/tensor/helium_stabilization_sae/config.ini``).

* ``hydrogen(lmax=10, nbsplines=150, rmax=100)``: N = 150 B-splines from 147 breakpoints.
* ``hydrogen(lmax=40, nbsplines=600, rmax=400)``: N = 600 from 597 breakpoints.
The inner exponential part starts at ``xpartition`` 10 with gamma 2; the inner point count
(and, when no count hits the total, ``xpartition`` in steps of 0.25) is searched so the
breakpoint total is exact. The chosen values are written into the config text.
"""
from __future__ import annotations

import math

from .bspline import exponential_linear_params_for

C_AU = 137.035999084
BOHR_NM = 0.0529177210903


# Full-length runs of the hydrogen model whose final states are checked against the
# complex128 oracle (tests/golden/run_*.npz). Each is a keyword set of ``hydrogen`` plus the
# propagator and the number of steps (duration / timestep).
#   * Crank-Nicolson: lmax 40, 600 B-splines on [0, 400], GMRES(20) with the block-diagonal
#     LU, dt 0.01 through a 50 a.u. sin^2 pulse of 800 nm and 0.05 a.u. (5000 steps) - the
#     benchmark's workload;
#   * pAMP: lmax 10, 150 B-splines on [0, 100], Krylov basis 20, dt 0.01 through a 10 a.u.
#     pulse of 800 nm and 0.05 a.u. (1000 steps), started from the field-free ground state;
#   * ensemble members: lmax, B-splines, peak field and wavelength drawn by
#     ``ensemble.hydrogen_ensemble_params``, r in [0, 100], dt 0.01, 10 a.u. pulse (1000 steps).
HYDROGEN_L40_CAYLEY = dict(lmax=40, nbsplines=600, rmax=400.0, timestep=0.01, pulse_duration=50.0, duration=50.0,
                           amplitude=0.05, wavelength_nm=800.0, krylov_basis_size=20, gmres_tolerance=1e-12)
HYDROGEN_L10_PAMP = dict(lmax=10, nbsplines=150, rmax=100.0, timestep=0.01, pulse_duration=10.0, duration=10.0,
                         amplitude=0.05, wavelength_nm=800.0, krylov_basis_size=20)
# GMRES tolerances of the Crank-Nicolson workload at equal final-state error: the loosest
# (of 1e-12 ... 1e-4 in factors of 10) whose state after the whole 5000-step pulse stays within
# an infidelity of 1e-8 of the complex128 reference run. Mixed precision (one refinement pass
# then suffices): 1e-7, infidelity 3.6e-11 (1e-6 gives 5e-8); plain FP64: 1e-6, infidelity
# 5.3e-10 (1e-5 gives 2.2e-7). Measured on a GB300 over the full pulse.
EQUAL_ERROR_TOLERANCE = {"fp32": 1e-7, "fp64": 1e-6}
ENSEMBLE_MEMBER = dict(rmax=100.0, timestep=0.01, pulse_duration=10.0, duration=10.0, krylov_basis_size=20,
                       gmres_tolerance=1e-12)


def run_steps(kw):
    """Number of steps of a run: duration / timestep, rounded."""
    return int(round(kw["duration"] / kw["timestep"]))


def field_free_ground_state(prob):
    """Field-free ground state of the l = 0 channel of a hydrogen ``Problem`` (host
    generalized eigenproblem of the time-independent radial band against the overlap, setup
    only): (psi [Nang][N] complex128 with unit S-norm, energy)."""
    import numpy as np
    import scipy.linalg as sl
    repr_ = prob.psi.GetRepresentation()
    nang, N = repr_.GetFullShape()
    h0 = prob.Propagator.BasePropagator.PotentialList[0].PotentialData[0]
    kb = repr_.kb
    b = 2 * kb + 1
    H = np.zeros((N, N), dtype=complex)
    S = np.zeros((N, N))
    for i in range(N):
        for j in range(max(0, i - kb), min(N, i + kb + 1)):
            H[i, j] = h0[j * b + (kb + i - j)]
            S[i, j] = repr_.overlap_rows[i, kb + j - i]
    w, v = sl.eigh(H.real, S)
    psi = np.zeros((nang, N), dtype=complex)
    psi[0] = v[:, 0] / np.sqrt(v[:, 0] @ S @ v[:, 0])
    return psi, float(w[0])


def omega_for_wavelength(nm):
    """Photon angular frequency (a.u.) for a wavelength in nm: 2 pi c / lambda."""
    return 2.0 * math.pi * C_AU / (nm / BOHR_NM)


def hydrogen(lmax=10, nbsplines=150, rmax=100.0, propagator="PamPropagatorGPU", precision="fp64",
             timestep=0.01, duration=10.0, krylov_basis_size=20, amplitude=0.05, wavelength_nm=800.0,
             pulse_duration=10.0, gmres_tolerance=1e-12, order=7):
    total = nbsplines - 3 if order == 7 else nbsplines - (order - 4)
    rpart, xsize = exponential_linear_params_for(0.0, rmax, total, gamma=2.0, rpartition=10.0)
    omega = omega_for_wavelength(wavelength_nm)
    return f"""
[Representation]
rank = 2
type = core.CombinedRepresentation_2
representation0 = "AngularRepresentation"
representation1 = "RadialRepresentation"

[AngularRepresentation]
type = core.ReducedSphericalHarmonicRepresentation
maxl = {lmax}
m = 0

[RadialRepresentation]
type = core.BSplineRepresentation
init_function = InitBSpline
xmin = 0.0
xmax = {rmax!r}
xsize = {xsize}
gamma = 2.0
xpartition = {rpart!r}
bpstype = 'exponentiallinear'
continuity = 'zero'
order = {order}
quad_order_additional = 0
projection_algorithm = 0

[InitialCondition]
type = InitialConditionType.Function
function = lambda conf, x: 1.0 * (x[0] == 0)

[PulseParameters]
frequency = {omega!r}
amplitude = {amplitude!r}
pulse_duration = {pulse_duration!r}

[Propagation]
base = "PulseParameters"
grid_potential_list = ["RadialKineticEnergy", "AngularKineticEnergy", "CoulombPotential", "LaserPotential"]
propagator = {propagator}
base_propagator = BasisPropagatorGPU
preconditioner = "RadialPreconditioner"
timestep = {timestep!r}
duration = {duration!r}
renormalization = False
krylov_basis_size = {krylov_basis_size}
krylov_tolerance = {gmres_tolerance!r}
krylov_double_orthogonalization = True
gpu_precision = "{precision}"
silent = True

[RadialPreconditioner]
type = BSplinePreconditioner
rank = 1
potential_evaluation = ["RadialKineticEnergy", "AngularKineticEnergy", "CoulombPotential"]

[Arpack]
krylov_basis_size = 20
krylov_tolerance = 1e-12
krylov_eigenvalue_count = 2
krylov_max_iteration_count = 50
krylov_use_random_start = True

[RadialKineticEnergy]
classname = "KineticEnergyPotential"
geometry0 = "Diagonal"
geometry1 = "banded-nonhermitian"
differentiation0 = 0
differentiation1 = 2
mass = 1

[AngularKineticEnergy]
classname = "AngularKineticEnergyPotential"
geometry0 = "Diagonal"
geometry1 = "banded-nonhermitian"
mass = 1
angular_rank = 0
radial_rank = 1

[CoulombPotential]
classname = "CoulombPotential"
geometry0 = "Diagonal"
geometry1 = "banded-nonhermitian"
radial_rank = 1
z = 1.0
soft = 0.0

[LaserPotential]
base = "PulseParameters"
classname = "DipoleLaserPotentialLength"
geometry0 = "dipoleselectionrule"
geometry1 = "banded-nonhermitian"
angular_rank = 0
radial_rank = 1
charge = -1.0
time_function = LaserFunctionSimpleLength
"""


def helium(lmax=2, L=(0,), nbsplines=20, rmax=20.0, order=7, quad_order_additional=10, z=2.0,
           propagator="PamPropagatorGPU", precision="fp64", timestep=0.01, duration=1.0, krylov_basis_size=20,
           amplitude=0.0, frequency=1.0, pulse_duration=10.0, gmres_tolerance=1e-12, factorize=True,
           preconditioner_type="RadialTwoElectronPreconditionerSuperLU"):
    """Two-electron (helium-like) model in the layout of
    examples/tensor/helium_stabilization/config.ini:1-188: coupled spherical harmonics
    (``DefaultCoupledIndexIterator(lmax, L, M=0)``) x B-splines x B-splines, radial kinetic
    energy of each electron, angular kinetic energy, nuclear attraction -z/r1 - z/r2, the
    electron-electron repulsion on ``SelectionRule_R12`` pairs and, with amplitude != 0, the
    length-gauge laser coupling on ``SelectionRule_LinearPolarizedField`` pairs with a sin^2
    pulse (L must then hold neighbouring values). factorize=False stores every term per
    angular pair as the reference does (by default the two-electron terms are kept as angular
    coefficients x shared radial operators)."""
    total = nbsplines - 3 if order == 7 else nbsplines - (order - 4)
    laser_name = ', "LaserPotential"' if amplitude else ""
    cayley = "Cayley" in str(propagator)
    prec_key = 'preconditioner = "RadialPreconditioner"' if cayley else ""
    prec_sec = f"""
[RadialPreconditioner]
type = {preconditioner_type}
z = {z!r}
""" if cayley else ""
    laser = f"""
[PulseParameters]
frequency = {frequency!r}
amplitude = {amplitude!r}
pulse_duration = {pulse_duration!r}

[LaserPotential]
base = "PulseParameters"
classname = "CustomPotential_LaserLength"
geometry0 = "SelectionRule_LinearPolarizedField"
geometry1 = "banded-packed"
geometry2 = "banded-packed"
angular_rank = 0
radial_rank1 = 1
radial_rank2 = 2
time_function = LaserFunctionLength
""" if amplitude else ""
    rpart, xsize = exponential_linear_params_for(0.0, rmax, total, gamma=2.0, rpartition=min(10.0, rmax / 2))
    Ls = list(L)
    text = f"""
[Representation]
rank = 3
type = core.CombinedRepresentation_3
representation0 = "AngularRepresentation"
representation1 = "RadialRepresentation"
representation2 = "RadialRepresentation"

[AngularRepresentation]
type = core.CoupledSphericalHarmonicRepresentation
index_iterator = DefaultCoupledIndexIterator(lmax={lmax}, L={Ls!r}, M=[0])

[RadialRepresentation]
type = core.BSplineRepresentation
init_function = InitBSpline
xmin = 0.0
xmax = {rmax!r}
xsize = {xsize}
gamma = 2.0
xpartition = {rpart!r}
bpstype = 'exponentiallinear'
continuity = 'zero'
order = {order}
quad_order_additional = {quad_order_additional}
projection_algorithm = 0

[InitialCondition]
type = InitialConditionType.Function
function = lambda conf, x: 1.0 * (x[0] == 0)

[Propagation]
grid_potential_list = ["RadialKineticEnergy1", "RadialKineticEnergy2", "AngularKineticEnergy", "CoulombPotential", "ElectronicCouplingPotential"{laser_name}]
propagator = {propagator}
base_propagator = BasisPropagatorGPU
timestep = {timestep!r}
duration = {duration!r}
renormalization = False
krylov_basis_size = {krylov_basis_size}
krylov_tolerance = {gmres_tolerance if cayley else 0!r}
krylov_double_orthogonalization = True
gpu_precision = "{precision}"
silent = True
{prec_key}
{prec_sec}
[RadialKineticEnergy1]
classname = "KineticEnergyPotential"
geometry0 = "Diagonal"
geometry1 = "banded-packed"
geometry2 = "banded-packed"
differentiation0 = 0
differentiation1 = 2
differentiation2 = 0
mass = 1

[RadialKineticEnergy2]
classname = "KineticEnergyPotential"
geometry0 = "Diagonal"
geometry1 = "banded-packed"
geometry2 = "banded-packed"
differentiation0 = 0
differentiation1 = 0
differentiation2 = 2
mass = 1

[AngularKineticEnergy]
classname = "CoupledSphericalKineticEnergyEvaluator"
geometry0 = "Diagonal"
geometry1 = "banded-packed"
geometry2 = "banded-packed"
angular_rank = 0
radial_rank1 = 1
radial_rank2 = 2
mass = 1

[CoulombPotential]
classname = "CoupledSphericalCoulombPotential"
geometry0 = "Diagonal"
geometry1 = "banded-packed"
geometry2 = "banded-packed"
radial_rank1 = 1
radial_rank2 = 2
z = {z!r}

[ElectronicCouplingPotential]
classname = "CustomPotentialEvaluationR12"
geometry0 = "SelectionRule_R12"
geometry1 = "banded-packed"
geometry2 = "banded-nonhermitian"
angular_rank = 0
radial_rank1 = 1
radial_rank2 = 2
{laser}"""
    if not factorize:
        text = text.replace('\nclassname = ', '\nfactorize = False\nclassname = ')
    return text
