"""``Problem``: config -> wavefunction + propagator, time stepping, observables.

Follows ``pyprop/Problem.py:62-307`` (``SetupStep``, ``AdvanceStep``, ``Advance``,
``GetEnergyExpectationValue``) and the representation factory of
``pyprop/CreateInstance.py:11-93`` for the ranks this path supports: a
``ReducedSphericalHarmonicRepresentation`` angular rank and a ``BSplineRepresentation``
radial rank (one electron), or a ``CoupledSphericalHarmonicRepresentation`` angular rank and
two B-spline radial ranks (two electrons).
"""
from __future__ import annotations

import numpy as np

from .bspline import bspline_from_config
from .representation import CombinedRepresentation, Wavefunction
from .tensorpotential import BSplineRankBasis, CoupledSphericalRankBasis, ReducedSphericalRankBasis


class _CoreNamespace:
    """Stand-ins for the reference's ``core.*`` type names used in [Representation] sections."""

    class CombinedRepresentation_2:
        pass

    class ReducedSphericalHarmonicRepresentation:
        pass

    class BSplineRepresentation:
        pass

    class CombinedRepresentation_3:
        pass

    class CoupledSphericalHarmonicRepresentation:
        pass


core = _CoreNamespace()


def InitBSpline(conf):
    """``pyprop/bspline/BSpline.py:5-11``."""
    return bspline_from_config(conf)


class InitialConditionType:
    Function = "Function"
    Custom = "Custom"
    Vector = "Vector"


def CreateRepresentation(config):
    sec = config.Representation
    rank = int(getattr(sec, "rank", 2))
    bases = []
    for r in range(rank):
        sub = config.GetSection(getattr(sec, "representation%d" % r))
        t = sub.type
        if t is core.ReducedSphericalHarmonicRepresentation or getattr(t, "__name__", "") == \
                "ReducedSphericalHarmonicRepresentation":
            bases.append(ReducedSphericalRankBasis(int(sub.maxl), int(getattr(sub, "m", 0))))
        elif t is core.BSplineRepresentation or getattr(t, "__name__", "") == "BSplineRepresentation":
            bases.append(BSplineRankBasis(bspline_from_config(sub)))
        elif t is core.CoupledSphericalHarmonicRepresentation or getattr(t, "__name__", "") == \
                "CoupledSphericalHarmonicRepresentation":
            bases.append(CoupledSphericalRankBasis(sub.index_iterator))
        else:
            raise NotImplementedError("representation type %r is outside the GPU path" % (t,))
    return CombinedRepresentation(bases)


def CreateWavefunction(config):
    return Wavefunction(CreateRepresentation(config))


def CreatePropagator(config, psi):
    cls = config.Propagation.propagator
    prop = cls(psi)
    config.Apply(prop)
    return prop


class Problem:
    def __init__(self, config):
        self.Config = config
        self.psi = CreateWavefunction(config)
        self.Propagator = CreatePropagator(config, self.psi)
        config.Propagation.Apply(self)
        self.TempPsi = None

    def ApplyConfigSection(self, conf):
        self.TimeStep = conf.timestep
        self.StartTime = getattr(conf, "start_time", 0.0)
        self.Duration = getattr(conf, "duration", 0.0)
        self.PropagatedTime = self.StartTime

    def SetupStep(self, skipWavefunctionSetup=False):
        self.Propagator.SetupStep(self.TimeStep)
        if not skipWavefunctionSetup:
            self.SetupWavefunction()

    def SetupWavefunction(self):
        """``pyprop/Problem.py:320-344``: Function initial conditions evaluated on the basis
        index grid (``lambda conf, x: ...`` with x the index tuple)."""
        sec = getattr(self.Config, "InitialCondition", None)
        if sec is None:
            return
        kind = getattr(sec, "type", None)
        if kind == InitialConditionType.Function:
            shape = self.psi.GetRepresentation().GetFullShape()
            idx = np.indices(shape)
            vals = np.vectorize(lambda *x: sec.function(sec, x), otypes=[complex])(*idx)
            self.psi.SetData(vals)
        elif kind == InitialConditionType.Vector:
            self.psi.SetData(np.asarray(sec.vector, dtype=complex).reshape(self.psi.GetRepresentation().GetFullShape()))

    def RestartPropagation(self, timestep, startTime, propagationTime):
        self.TimeStep = timestep
        self.PropagatedTime = startTime
        self.StartTime = startTime
        self.Duration = propagationTime

    def SaveCheckpoint(self, filename, datasetPath="/checkpoint"):
        """Wavefunction, propagated time and time step in one ``.npz`` file (see
        :mod:`pyprop_gb300.serialization`), with the config as an attribute."""
        from .serialization import SaveWavefunction, _norm, _read, _write
        SaveWavefunction(filename, datasetPath + "/psi", self.psi, self.Config)
        entries = _read(filename)
        path = _norm(datasetPath)
        entries[path + "/time"] = np.array([self.PropagatedTime, np.real(self.TimeStep), np.imag(self.TimeStep)])
        _write(filename, entries)

    def LoadCheckpoint(self, filename, datasetPath="/checkpoint"):
        """Restore the wavefunction and the propagated time written by SaveCheckpoint (the
        problem must have the same representation)."""
        from .serialization import LoadWavefunction, _norm
        LoadWavefunction(filename, datasetPath + "/psi", self.psi)
        with np.load(filename, allow_pickle=False) as z:
            t = z[_norm(datasetPath) + "/time"]
        self.PropagatedTime = float(t[0])
        return self.PropagatedTime

    def AdvanceStep(self):
        self.Propagator.AdvanceStep(self.PropagatedTime, self.TimeStep)
        if self.Propagator.RenormalizeActive:
            self.psi.Normalize()
        self.PropagatedTime += abs(self.TimeStep) if abs(np.real(self.TimeStep)) < 1e-10 else np.real(self.TimeStep)

    def Advance(self, yieldCount, duration=None, yieldEnd=False):
        """Generator over time steps (``pyprop/Problem.py:185-244``)."""
        if duration is None:
            duration = self.Duration
        if isinstance(yieldCount, bool):
            yieldStep = 1
        else:
            yieldStep = max(1, int((duration / abs(self.TimeStep)) / yieldCount))
        endTime = self.StartTime + np.sign(np.real(self.TimeStep)) * duration
        index = 0
        prev = np.nan
        while abs(self.PropagatedTime - endTime) > 0.5 * abs(self.TimeStep):
            self.AdvanceStep()
            index += 1
            if index % yieldStep == 0:
                yield self.PropagatedTime
                prev = self.PropagatedTime
        if yieldEnd and prev != self.PropagatedTime:
            yield self.PropagatedTime

    def MultiplyHamiltonian(self, srcPsi, dstPsi):
        self.Propagator.MultiplyHamiltonian(srcPsi, dstPsi, self.PropagatedTime, self.TimeStep)

    def GetTempPsi(self):
        if self.TempPsi is None:
            self.TempPsi = self.psi.Copy()
        return self.TempPsi

    def GetEnergyExpectationValue(self):
        """E = <psi|H|psi> / <psi|S|psi> with H applied as S^-1 H (``Problem.py:257-279``)."""
        self.psi.Normalize()
        tmp = self.GetTempPsi()
        tmp.Clear()
        self.MultiplyHamiltonian(self.psi, tmp)
        return self.psi.InnerProduct(tmp).real

    GetEnergy = GetEnergyExpectationValue
