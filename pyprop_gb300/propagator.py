"""GPU propagators behind the reference's propagator interface.

* ``BasisPropagatorGPU`` - generates and consolidates the tensor potentials
  (``pyprop/tensorpotential/BasisPropagator.py:1-168``) and owns the device operators.
* ``PamPropagatorGPU`` - ``pyprop/propagator/PamPropagator.py``: pAMP with the balanced
  overlap (psi <- U psi, Krylov on U^-H H U^-1, psi <- U^-1 psi), H frozen at the step start.
* ``CayleyPropagatorGPU`` - ``pyprop/propagator/CayleyPropagator.py``: Crank-Nicolson at
  t + |dt|/2 solved by GMRES, left-preconditioned by the block-diagonal radial LU
  (``BSplinePreconditioner``, ``examples/tensor/helium_stabilization_sae/example.py:275-318``).

A config switches to these by naming them: ``propagator = PamPropagatorGPU`` or
``CayleyPropagatorGPU``, ``base_propagator = BasisPropagatorGPU`` (``BasisPropagator`` is
accepted as the same class). GPU-only keys in [Propagation]: ``gpu_precision``
("fp64" or "fp32": precision of the Krylov basis and of the operator it multiplies);
``gpu_fused_step`` (default True: a mixed-precision Cayley or pAMP step of a one-electron
banded operator runs as one cooperative kernel; False keeps the captured multi-kernel step);
``gpu_step_stats`` (default True: each step waits and keeps its statistics; False only
enqueues, and the statistics are read when asked for); ``gpu_device_exponential`` (pAMP graph
path, default False: the m x m exponential on the host between two graphs; True on the device).
"""
from __future__ import annotations

import logging

import numpy as np

from . import _native as nat
from .gpu import Banded, CayleyStepper, Context, DeviceOperator, PampStepper, precision_of, torch
from .tensorpotential import TensorPotential

_log = logging.getLogger("pyprop_gb300.propagator")


class PropagatorBase:
    """``pyprop/propagator/Propagator.py``: config plumbing shared by the propagators."""

    def __init__(self, psi):
        self.psi = psi
        self.Rank = psi.GetRank()
        self.PotentialList = []
        self.RenormalizeActive = False

    def ApplyConfig(self, config):
        self.Config = config
        config.Propagation.Apply(self)

    def ApplyConfigSection(self, conf):
        self.RenormalizeActive = bool(getattr(conf, "renormalization", False))
        self.PropagationSection = conf

    def SetupStep(self, dt):
        pass

    def RestartPropagation(self, timestep, startTime, propagationTime):
        pass


class BasisPropagatorGPU(PropagatorBase):
    """Holds the consolidated tensor potentials and applies H on the device."""

    def ApplyConfig(self, config):
        PropagatorBase.ApplyConfig(self, config)
        self.GeneratePotentials(config)
        self.ConsolidatePotentials()

    def GeneratePotential(self, conf):
        pot = TensorPotential(self.psi)
        conf.Apply(pot)
        return pot

    def GeneratePotentials(self, config):
        names = getattr(config.Propagation, "grid_potential_list", [])
        for name in names:
            pot = self.GeneratePotential(config.GetSection(name))
            for existing in self.PotentialList:
                if existing.CanConsolidate(pot):
                    existing.PotentialData = existing.PotentialData + pot.PotentialData
                    existing.Name += "+" + pot.Name
                    pot = None
                    break
            if pot is not None:
                self.PotentialList.append(pot)

    def ConsolidatePotentials(self):
        """Merge potentials with equal storage, pairs and time dependence (BasisPropagator.py:68-105)."""
        pots = list(self.PotentialList)
        i = 0
        while i < len(pots) - 1:
            cur = pots[i]
            for other in list(pots[i + 1:]):
                if cur.CanConsolidate(other):
                    cur.PotentialData = cur.PotentialData + other.PotentialData
                    cur.Name += "+" + other.Name
                    pots.remove(other)
            i += 1
        self.PotentialList = pots

    def SetupStep(self, dt):
        for pot in self.PotentialList:
            pot.SetupStep(dt)
        self._ops = {}

    # device operators, built on first use
    def device_operator(self, precision, with_overlap=False, fp64_emulation=False):
        key = (precision, with_overlap, bool(fp64_emulation))
        if key not in getattr(self, "_ops", {}):
            if not hasattr(self, "_ops"):
                self._ops = {}
            repr_ = self.psi.GetRepresentation()
            self._ops[key] = DeviceOperator(Context.get(), self.PotentialList, repr_.GetFullShape(), repr_.kb,
                                            precision, repr_.overlap_rows if with_overlap else None,
                                            fp64_emulation=fp64_emulation)
        return self._ops[key]

    def MultiplyPotential(self, srcPsi, destPsi, t, dt):
        op = self.device_operator(nat.PG_FP64)
        op.matvec(op.scales(t), srcPsi.GetData(), destPsi.GetData(), accumulate=True)

    def MultiplyHamiltonianNoOverlap(self, srcPsi, destPsi, t, dt):
        op = self.device_operator(nat.PG_FP64)
        op.matvec(op.scales(t), srcPsi.GetData(), destPsi.GetData(), accumulate=False)

    def MultiplyHamiltonian(self, srcPsi, destPsi, t, dt):
        """dest = S^-1 H src (BasisPropagator.py:116-124)."""
        self.MultiplyHamiltonianNoOverlap(srcPsi, destPsi, t, dt)
        destPsi.GetRepresentation().SolveOverlap(destPsi)

    def MultiplyHamiltonianBalancedOverlap(self, srcPsi, destPsi, t, dt):
        """dest = U^-H H U^-1 src, src unchanged (BasisPropagator.py:131-159)."""
        tmp = srcPsi.Copy()
        repr_ = srcPsi.GetRepresentation()
        repr_.SolveSqrtOverlap(False, tmp)
        self.MultiplyHamiltonianNoOverlap(tmp, destPsi, t, dt)
        repr_.SolveSqrtOverlap(True, destPsi)


BasisPropagator = BasisPropagatorGPU


def _basis_propagator(config, psi):
    cls = getattr(config.Propagation, "base_propagator", BasisPropagatorGPU)
    if cls not in (BasisPropagatorGPU,):
        cls = BasisPropagatorGPU
    bp = cls(psi)
    config.Apply(bp)
    return bp


class PamPropagatorGPU(PropagatorBase):
    def ApplyConfig(self, config):
        PropagatorBase.ApplyConfig(self, config)
        self.BasePropagator = _basis_propagator(config, self.psi)
        conf = config.Propagation
        self.BasisSize = int(getattr(conf, "krylov_basis_size", 20))
        self.DoubleOrthogonalization = bool(getattr(conf, "krylov_double_orthogonalization", True))
        self.Precision = precision_of(getattr(conf, "gpu_precision", "fp64"))
        method = getattr(conf, "krylov_exponentiation_method", 0)
        if method not in (0, "pade", "Pade"):
            _log.warning("krylov_exponentiation_method=%r: the GPU path uses the Pade exponential", method)
        self.StepStats = bool(getattr(conf, "gpu_step_stats", True))
        self.DeviceExponential = bool(getattr(conf, "gpu_device_exponential", False))
        self.FusedStep = bool(getattr(conf, "gpu_fused_step", True))

    def SetupStep(self, dt):
        self.BasePropagator.SetupStep(dt)
        repr_ = self.psi.GetRepresentation()
        bp = self.BasePropagator
        self.op64 = bp.device_operator(nat.PG_FP64)
        self.opb = bp.device_operator(self.Precision)
        self.ovl64 = Banded.overlap(self.op64, repr_.overlap_rows)
        self.ovlb = self.ovl64 if self.Precision == nat.PG_FP64 else Banded.overlap(self.opb, repr_.overlap_rows)
        self.stepper = PampStepper(self.op64, self.opb, self.ovl64, self.ovlb, self.BasisSize, self.Precision,
                                   self.DoubleOrthogonalization)
        if self.DeviceExponential and self.BasisSize <= 48:
            self.stepper.set_device_exp(True)
        # the single-kernel step (complex64 basis) where it qualifies
        self.Fused = self.stepper.set_fused(self.FusedStep and self.Precision == nat.PG_FP32)

    def AdvanceStep(self, t, dt):
        """One step at H(t). With ``gpu_step_stats`` (default) the call waits for the step and
        keeps its statistics; otherwise it only enqueues and ``GetErrorEstimate`` waits."""
        scales = self.op64.scales(t)
        self._last_stats = None
        st = self.stepper.step(self.psi.GetData(), dt, scales, want_stats=self.StepStats)
        if st is not None:
            self.LastStats = st

    @property
    def LastStats(self):
        if getattr(self, "_last_stats", None) is None:
            self._last_stats = self.stepper.last_stats()
        return self._last_stats

    @LastStats.setter
    def LastStats(self, value):
        self._last_stats = value

    def MultiplyHamiltonian(self, srcPsi, destPsi, t, dt):
        self.BasePropagator.MultiplyHamiltonian(srcPsi, destPsi, t, dt)

    def GetErrorEstimate(self):
        return self.LastStats.ErrorEstimate


class BSplinePreconditioner:
    """Block-diagonal radial preconditioner M_l = cS S + cH H_l (example.py:275-318):
    the potentials listed in ``potential_evaluation`` (diagonal in the angular rank) are
    summed per channel and each band is factored on the host, solved on the device."""

    def __init__(self, psi):
        self.psi = psi
        self.PotentialSections = []

    def ApplyConfigSection(self, conf):
        self.PreconditionRank = getattr(conf, "rank", 1)
        names = getattr(conf, "potential_evaluation", [])
        self.PotentialSections = [conf.Config.GetSection(s) for s in names]

    def SetHamiltonianScaling(self, scalingH):
        self.HamiltonianScaling = scalingH

    def SetOverlapScaling(self, scalingS):
        self.OverlapScaling = scalingS

    def Setup(self, prop, precision=nat.PG_FP64):
        pots = []
        for conf in self.PotentialSections:
            pot = prop.BasePropagator.GeneratePotential(conf)
            ids = [g.GetStorageId() for g in pot.GeometryList]
            if ids[-1] != "BandNH" or any(i != "Diag" for i in ids[:-1]):
                raise ValueError("preconditioner potentials must be Diag in the angular rank and BandNH radially")
            pots.append(pot)
        repr_ = self.psi.GetRepresentation()
        self.ops = {}
        self.solvers = {}
        for prec in (nat.PG_FP64, precision):
            if prec in self.solvers:
                continue
            op = DeviceOperator(Context.get(), pots, repr_.GetFullShape(), repr_.kb, prec)
            self.ops[prec] = op
            self.solvers[prec] = Banded.blockdiag(op, repr_.overlap_rows, self.OverlapScaling, self.HamiltonianScaling,
                                                  list(range(1, 1 + len(pots))), [1.0] * len(pots))

    def Solve(self, psi):
        self.solvers[nat.PG_FP64].apply(nat.PG_BAND_PREC_SOLVE, psi.GetData())


RadialPreconditioner = BSplinePreconditioner


class TwoElectronKroneckerPreconditioner(BSplinePreconditioner):
    """Two-electron radial preconditioner for the Cayley step on [channel][r1][r2]: per coupled
    channel (l1, l2, L, M) the Kronecker product (cS S + cH h_l1) x (cS S + cH h_l2) of the
    one-electron radial operators h_l = -1/2 d^2/dr^2 + l(l+1)/(2 r^2) - z/r, factored on the
    host and solved on the device along each radial rank. It takes the place of the
    reference's RadialTwoElectronPreconditionerSuperLU / Ifpack
    (examples/tensor/helium_stabilization/preconditioner.py:77-244), which factor the full
    channel block including the electron-electron repulsion; this one leaves the repulsion out
    (the learned preconditioner can add the missing part). Config keys: z (default 2), mass."""

    def ApplyConfigSection(self, conf):
        self.Z = float(getattr(conf, "z", 2.0))
        self.Mass = float(getattr(conf, "mass", 1.0))

    def _one_electron(self, l):
        bs = self.psi.GetRepresentation().radial.BSplineObject
        r = bs.grid
        kin = bs.band_elements(np.full(r.shape, -1.0 / (2.0 * self.Mass)), 2)
        pot = bs.band_elements(l * (l + 1.0) / (2.0 * self.Mass * r * r) - self.Z / r, 0)
        return np.asarray(kin + pot, dtype=np.complex128)

    def Setup(self, prop, precision=nat.PG_FP64):
        repr_ = self.psi.GetRepresentation()
        shape = repr_.GetFullShape()
        if len(shape) != 3:
            raise ValueError("TwoElectronKroneckerPreconditioner needs a two-electron representation")
        self.Method = "kronecker-product"
        indices = repr_.bases[0].indices
        cache = {}

        def h(l):
            if l not in cache:
                cache[l] = self._one_electron(l)
            return cache[l]

        h1 = np.stack([h(ix.l1) for ix in indices])
        h2 = np.stack([h(ix.l2) for ix in indices])
        self.ops, self.solvers = {}, {}
        for prec in (nat.PG_FP64, precision):
            if prec in self.solvers:
                continue
            op = DeviceOperator(Context.get(), [], shape, repr_.kb, prec)
            self.ops[prec] = op
            self.solvers[prec] = Banded.kron(op, repr_.overlap_rows, self.OverlapScaling, self.HamiltonianScaling,
                                             h1, h2)


class TwoElectronFastDiagonalizationPreconditioner(TwoElectronKroneckerPreconditioner):
    """Two-electron radial preconditioner for the Cayley step: per coupled channel the exact
    inverse of the part of the channel block that is separable in r1 and r2,
        M_a = cS S x S + cH (h_l1 x S + S x h_l2),
    by fast diagonalization: with the generalized eigenvectors h_l V_l = S V_l Lambda_l
    (V^T S V = 1, from scipy on the host once per l), M_a^-1 = (V1 x V2) D_a (V1 x V2)^T with
    D_a = 1 / (cS + cH (lambda_l1 + lambda_l2)), four dense N x N products per channel on the
    device. Unlike the Kronecker product (cS S + cH h1) x (cS S + cH h2), it has no cH^2 h1 x h2
    error, so GMRES is left only with the electron-electron repulsion that the reference's
    RadialTwoElectronPreconditionerSuperLU / Ifpack also put in the block
    (examples/tensor/helium_stabilization/preconditioner.py:77-244). Radial sizes beyond the
    shared-memory limit of the one-kernel solve run as batched GEMMs through global memory."""

    def _dense(self, l):
        band = self._one_electron(l).real  # rows [N][2k+1], [i, k + j - i] = h(i, j)
        N, b = band.shape
        kb = (b - 1) // 2
        D = np.zeros((N, N))
        for d in range(-kb, kb + 1):
            i = np.arange(max(0, -d), min(N, N - d))
            D[i, i + d] = band[i, kb + d]
        return 0.5 * (D + D.T)

    def Setup(self, prop, precision=nat.PG_FP64):
        import scipy.linalg as sl
        repr_ = self.psi.GetRepresentation()
        shape = repr_.GetFullShape()
        if len(shape) != 3:
            raise ValueError("TwoElectronFastDiagonalizationPreconditioner needs a two-electron representation")
        ctx = Context.get()
        self.Method = "fast-diagonalization"
        indices = repr_.bases[0].indices
        S = repr_.radial.BSplineObject.dense(repr_.overlap_rows)
        ls = sorted(set(ix.l1 for ix in indices) | set(ix.l2 for ix in indices))
        pos = {l: k for k, l in enumerate(ls)}
        V, lam = [], []
        for l in ls:
            w, v = sl.eigh(self._dense(l), S)
            V.append(v)
            lam.append(w)
        lidx = np.array([(pos[ix.l1], pos[ix.l2]) for ix in indices], dtype=np.int32)
        self.ops, self.solvers = {}, {}
        for prec in (nat.PG_FP64, precision):
            if prec in self.solvers:
                continue
            op = DeviceOperator(ctx, [], shape, repr_.kb, prec)
            self.ops[prec] = op
            self.solvers[prec] = Banded.fast_diagonalization(op, np.stack(V), np.stack(lam), lidx,
                                                             self.OverlapScaling, self.HamiltonianScaling)


# the reference's two-electron preconditioner names select the GPU one
RadialTwoElectronPreconditionerSuperLU = TwoElectronFastDiagonalizationPreconditioner
RadialTwoElectronPreconditionerIfpack = TwoElectronFastDiagonalizationPreconditioner


class CayleyPropagatorGPU(PropagatorBase):
    def ApplyConfig(self, config):
        PropagatorBase.ApplyConfig(self, config)
        self.BasePropagator = _basis_propagator(config, self.psi)
        conf = config.Propagation
        self.BasisSize = int(getattr(conf, "krylov_basis_size", 20))
        tol = float(getattr(conf, "krylov_tolerance", 0.0) or 0.0)
        self.Tolerance = max(tol, 1e-13)  # gmres.h:223-229 floor
        self.Precision = precision_of(getattr(conf, "gpu_precision", "fp64"))
        self.StepStats = bool(getattr(conf, "gpu_step_stats", True))
        self.TrueResidual = bool(getattr(conf, "gpu_true_residual", False))
        self.Eager = bool(getattr(conf, "gpu_eager", False))
        # mixed precision, rank-2 banded operator: the whole step as one kernel unless
        # gpu_fused_step = False
        self.FusedStep = bool(getattr(conf, "gpu_fused_step", True))
        # its layout: 0 a cluster of three CTAs per channel where it fits, 1 one CTA per channel
        self.FusedVariant = int(getattr(conf, "gpu_fused_variant", 0))
        # mixed precision: the FP64 residual operator computes its factorized (two-electron)
        # terms in double-float arithmetic unless gpu_fp64_emulation = False
        self.Fp64Emulation = bool(getattr(conf, "gpu_fp64_emulation", True))
        name = getattr(conf, "preconditioner", None)
        self.Preconditioner = None
        if name:
            sec = config.GetSection(name)
            ptype = getattr(sec, "type", BSplinePreconditioner)
            if not isinstance(ptype, type) or not issubclass(ptype, BSplinePreconditioner):
                ptype = BSplinePreconditioner
            pre = ptype(self.psi)
            sec.Apply(pre)
            self.Preconditioner = pre

    def SetupStep(self, dt):
        self.BasePropagator.SetupStep(dt)
        if self.Preconditioner is None:
            raise ValueError("CayleyPropagatorGPU needs a block-diagonal preconditioner section")
        self.Preconditioner.SetHamiltonianScaling(1.0j * dt / 2.0)
        self.Preconditioner.SetOverlapScaling(1.0)
        self.Preconditioner.Setup(self, self.Precision)
        bp = self.BasePropagator
        emulate = self.Precision != nat.PG_FP64 and self.Fp64Emulation
        self.op64 = bp.device_operator(nat.PG_FP64, with_overlap=True, fp64_emulation=emulate)
        self.opb = bp.device_operator(self.Precision, with_overlap=True)
        self.stepper = CayleyStepper(self.op64, self.opb, self.Preconditioner.solvers[nat.PG_FP64],
                                     self.Preconditioner.solvers[self.Precision], self.BasisSize, self.Precision,
                                     self.Tolerance, self.TrueResidual)
        if self.Eager:
            self.stepper.set_eager(True)
        self.Fused = self.stepper.set_fused(self.FusedStep and not self.Eager)
        if self.Fused and self.FusedVariant:
            self.stepper.set_fused_variant(self.FusedVariant)

    def AdvanceStep(self, t, dt):
        """One step at H(t + |dt|/2). With ``gpu_step_stats`` (default) the call waits for the
        step and warns when the GMRES estimate exceeds 1e-4 (CayleyPropagator.py:103-111);
        otherwise it only enqueues and ``GetErrorEstimate`` waits."""
        scales = self.op64.scales(t + abs(dt / 2.0))
        self._last_stats = None
        st = self.stepper.step(self.psi.GetData(), dt, scales, want_stats=self.StepStats)
        if st is not None:
            self.LastStats = st
            if st.ErrorEstimate > 1e-4:
                _log.warning("GMRES error estimate %g", st.ErrorEstimate)

    @property
    def LastStats(self):
        if getattr(self, "_last_stats", None) is None:
            self._last_stats = self.stepper.last_stats()
        return self._last_stats

    @LastStats.setter
    def LastStats(self, value):
        self._last_stats = value

    def MultiplyHamiltonian(self, srcPsi, destPsi, t, dt):
        self.BasePropagator.MultiplyHamiltonian(srcPsi, destPsi, t, dt)

    def GetErrorEstimate(self):
        return self.LastStats.ErrorEstimate


class PamPropagator:
    """Name of the reference's CPU propagator: this package has no CPU path."""

    def __init__(self, psi):
        raise RuntimeError("PamPropagator is the reference CPU propagator; name PamPropagatorGPU in the config")


class CayleyPropagator:
    def __init__(self, psi):
        raise RuntimeError("CayleyPropagator is the reference CPU propagator; name CayleyPropagatorGPU in the config")
