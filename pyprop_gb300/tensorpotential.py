"""Tensor potentials: geometry infos, generation from grid potentials, consolidation.

Host-side setup, following ``pyprop/tensorpotential``:

* storage ids and basis pairs per rank (``GeometryInfo.py``; BandNH index map
  ``j*(2k+1) + (k+i-j)`` at ``GeometryInfo.py:409-462``; dipole selection pairs
  ``basis/ReducedSphericalHarmonic.py:5-45``; packed band pairs ``basis/BSpline.py:8-57``);
* generation: evaluate the potential on the tensor grid, then represent it in the basis
  rank by rank from the last rank to the first (``TensorPotentialGenerator.py:80-274``);
* ``TensorPotential`` with ``CanConsolidate`` (``TensorPotential.py:3-163``).

The arrays produced here (``PotentialData``, ``BasisPairs``) have the reference's layout;
the GPU operator is built from them in :mod:`pyprop_gb300.operator`.
"""
from __future__ import annotations

import numpy as np

from .bspline import BSplineBasis
from .potentials import POTENTIAL_CLASSES
from .spherical import ReducedSphericalTools, dipole_selection_pairs


class GeometryInfo:
    """Storage description of one rank of a tensor potential."""

    def __init__(self, storage_id, pairs, use_grid, band_count=None):
        self.StorageId = storage_id
        self.Pairs = None if pairs is None else np.asarray(pairs, dtype=np.int32).reshape(-1, 2)
        self.UseGrid = use_grid
        self.BandCount = band_count  # BandNH: number of super diagonals (order - 1)

    def GetStorageId(self):
        return self.StorageId

    def GetBasisPairs(self):
        return self.Pairs

    def GetGlobalBasisPairCount(self):
        return 1 if self.StorageId == "Ident" else len(self.Pairs)

    def UseGridRepresentation(self):
        return self.UseGrid


def bandnh_pairs(N, kb):
    """Pairs of ``GeometryInfoCommonBandedNonHermitian`` (GeometryInfo.py:437-456): slot
    ``j*(2kb+1) + (kb+i-j)`` holds (i, j); unused slots hold (0, N-1)."""
    b = 2 * kb + 1
    pairs = np.zeros((N * b, 2), dtype=np.int32)
    pairs[:, 1] = N - 1
    for i in range(N):
        for j in range(max(0, i - kb), min(N, i + kb + 1)):
            pairs[j * b + (kb + i - j)] = (i, j)
    return pairs


def packed_band_pairs(N, k):
    """Pairs of ``GeometryInfoBSplineBanded`` (basis/BSpline.py:25-44): row-major |i-j| < k."""
    return np.asarray([(i, j) for i in range(N) for j in range(max(0, i - k + 1), min(i + k, N))],
                      dtype=np.int32)


def hermitian_band_pairs(N, k):
    """Pairs of ``GeometryInfoBSplineBandedBlas`` (basis/BSpline.py:75-100): (i, i+j), j < k."""
    pairs = np.zeros((N * k, 2), dtype=np.int32)
    pairs[:, 1] = N - 1
    for i in range(N):
        for j in range(k):
            if i + j < N:
                pairs[i * k + j] = (i, i + j)
    return pairs


# ---------------------------------------------------------------------------------------
# bases of the ranks
# ---------------------------------------------------------------------------------------


class BSplineRankBasis:
    """Radial B-spline rank (``BasisfunctionBSpline``, basis/BSpline.py:175-235)."""

    orthogonal = False

    def __init__(self, bspline: BSplineBasis):
        self.BSplineObject = bspline
        self.size = bspline.NumberOfBSplines

    def GetGeometryInfo(self, name):
        geom = name.lower().strip()
        N = self.BSplineObject.NumberOfBSplines
        k = self.BSplineObject.MaxSplineOrder
        if geom == "banded-nonhermitian":
            return GeometryInfo("BandNH", bandnh_pairs(N, k - 1), True, k - 1)
        if geom == "banded-packed":
            return GeometryInfo("Simp", packed_band_pairs(N, k), True)
        if geom == "banded-hermitian":
            return GeometryInfo("Band", hermitian_band_pairs(N, k), True)
        if geom in ("dense", "hermitian"):
            return GeometryInfo("Dense", [(i, j) for i in range(N) for j in range(N)], True)
        if geom == "identity":
            return GeometryInfo("Ident", None, True)
        raise ValueError("Geometry '%s' not supported by the B-spline rank" % name)

    def grid(self, geometry):
        return self.BSplineObject.grid

    def represent(self, values, geometry, differentiation):
        """Project the last axis (quadrature grid) to the storage of ``geometry``."""
        bs = self.BSplineObject
        if geometry.StorageId == "Ident":
            raise ValueError("identity storage in the B-spline rank is not a band matrix")
        band = bs.band_elements(values, differentiation)  # (..., N, 2k-1)
        kb = bs.MaxSplineOrder - 1
        pairs = geometry.Pairs
        i, j = pairs[:, 0], pairs[:, 1]
        inside = np.abs(j - i) <= kb
        out = np.zeros(values.shape[:-1] + (len(pairs),), dtype=band.dtype)
        out[..., inside] = band[..., i[inside], kb + (j - i)[inside]]
        if geometry.StorageId == "Herm":
            out[..., i == j] *= 0.5
        return out


class ReducedSphericalRankBasis:
    """Angular rank of reduced spherical harmonics (basis/ReducedSphericalHarmonic.py:83-147)."""

    orthogonal = True

    def __init__(self, lmax, m=0):
        self.tools = ReducedSphericalTools(lmax, m)
        self.LMax = lmax
        self.M = m
        self.size = lmax + 1 - abs(m)

    def GetGeometryInfo(self, name):
        geom = name.lower().strip()
        use_grid = True
        if geom.startswith("custom-"):
            use_grid = False
            geom = geom[len("custom-"):]
        n = self.size
        if geom == "identity":
            return GeometryInfo("Ident", None, use_grid)
        if geom == "diagonal":
            return GeometryInfo("Diag", [(i, i) for i in range(n)], False)
        if geom == "dense":
            return GeometryInfo("Simp", [(i, j) for i in range(n) for j in range(n)], use_grid)
        if geom == "dipoleselectionrule":
            return GeometryInfo("Simp", dipole_selection_pairs(n), use_grid)
        raise ValueError("Geometry '%s' not supported by the reduced spherical rank" % name)

    def grid(self, geometry):
        if geometry.UseGrid:
            return self.tools.ThetaGrid
        return self.tools.l_values.astype(np.float64)

    def represent(self, values, geometry, differentiation):
        """Project the first axis (theta) onto the angular pairs."""
        if geometry.StorageId == "Ident":
            return values[:1]
        return self.tools.project_pairs(values, geometry.Pairs, differentiation)


class CoupledSphericalRankBasis:
    """Two-electron angular rank (``CoupledSphericalHarmonicRepresentation``,
    pyprop/tensorpotential/basis/CoupledSphericalHarmonic.py:94-170): never on a grid; its
    geometries are pair lists from selection rules (core/tensorpotential/
    coupledsphericalselectionrule.h) and its matrix elements come from custom evaluators."""

    orthogonal = True

    def __init__(self, index_iterator):
        from .spherical import CoupledSphericalBasis
        self.basis = CoupledSphericalBasis(index_iterator)
        self.indices = self.basis.indices
        self.size = self.basis.size

    def GetGeometryInfo(self, name):
        from .spherical import rule_diagonal, rule_linear_polarized_field, rule_r12_old
        geom = name.lower().strip()
        n = self.size
        if geom == "identity":
            return GeometryInfo("Ident", None, False)
        if geom == "diagonal":
            return GeometryInfo("Simp", self.basis.pairs(rule_diagonal), False)
        if geom == "dense":
            return GeometryInfo("Dense", [(i, j) for i in range(n) for j in range(n)], False)
        if geom == "selectionrule_r12":
            return GeometryInfo("Simp", self.basis.pairs(rule_r12_old), False)
        if geom == "selectionrule_linearpolarizedfield":
            return GeometryInfo("Simp", self.basis.pairs(rule_linear_polarized_field), False)
        raise ValueError("Geometry '%s' not supported by the coupled spherical rank" % name)

    def grid(self, geometry):
        n = 1 if geometry.Pairs is None else len(geometry.Pairs)
        return np.arange(n, dtype=np.float64)

    def represent(self, values, geometry, differentiation):
        raise ValueError("coupled spherical harmonics are already a basis")


# ---------------------------------------------------------------------------------------
# generator + tensor potential
# ---------------------------------------------------------------------------------------


def _evaluator_from_section(conf):
    classname = conf.classname
    cls = POTENTIAL_CLASSES.get(classname) if isinstance(classname, str) else classname
    if cls is None:
        raise KeyError("Unknown potential class %r" % (classname,))
    pot = cls()
    conf.Apply(pot)
    return pot


def generate_potential(bases, conf):
    """Evaluate ``conf``'s potential on the tensor grid and represent it in the bases.

    Returns ``(geometry_list, PotentialData)`` with ``PotentialData`` of shape
    ``(pairs_rank0, pairs_rank1, ...)``.
    """
    rank = len(bases)
    geoms = [bases[r].GetGeometryInfo(conf.Get("geometry%d" % r)) for r in range(rank)]
    evaluator = _evaluator_from_section(conf)
    if getattr(evaluator, "needs_basis", False):
        evaluator.bind(bases, geoms)
    grids = [bases[r].grid(geoms[r]) for r in range(rank)]
    pos = tuple(np.asarray(g).reshape([-1 if rr == r else 1 for rr in range(rank)]) for r, g in enumerate(grids))
    data = np.asarray(evaluator(pos), dtype=np.complex128)
    data = np.broadcast_to(data, tuple(len(g) for g in grids)).copy()
    for r in reversed(range(rank)):
        geom = geoms[r]
        if not geom.UseGrid:
            continue
        diff = conf.Get("differentiation%d" % r) if conf.Exists("differentiation%d" % r) else 0
        moved = np.moveaxis(data, r, -1 if isinstance(bases[r], BSplineRankBasis) else 0)
        projected = bases[r].represent(moved, geom, diff)
        data = np.moveaxis(projected, -1 if isinstance(bases[r], BSplineRankBasis) else 0, r)
    return geoms, np.ascontiguousarray(data)


class TensorPotential:
    """A potential stored in the basis (``pyprop/tensorpotential/TensorPotential.py``).

    ``PotentialData`` has one axis per rank, each indexed by that rank's basis pairs;
    ``MultiplyPotential`` adds ``f(t) * V * src`` to ``dst`` (``:92-112``).
    """

    def __init__(self, psi):
        self.psi = psi
        self.GeometryList = None
        self.PotentialData = None
        self.Name = None
        self.IsTimeDependent = False
        self.TimeFunction = None
        self.OriginalTimeFunction = None
        self.DebugPotential = False

    def ApplyConfigSection(self, conf):
        self.DebugPotential = bool(getattr(conf, "debug_potential", False))
        if conf.Exists("time_function"):
            self.IsTimeDependent = True
            tf = conf.time_function
            self.OriginalTimeFunction = tf
            self.TimeFunction = lambda t, _c=conf, _f=tf: _f(_c, t)
        self.Name = conf.name
        bases = self.psi.GetRepresentation().bases
        self.GeometryList, self.PotentialData = generate_potential(bases, conf)

    def SetupStep(self, timestep):
        self.BasisPairs = [g.GetBasisPairs() for g in self.GeometryList]
        self.StorageIds = "_".join(g.GetStorageId() for g in self.GeometryList)

    def GetTimeScaling(self, t):
        return float(self.TimeFunction(t)) if self.IsTimeDependent else 1.0

    def CanConsolidate(self, other):
        """Same time dependence, same storage and basis pairs in every rank (``:128-163``)."""
        if self.IsTimeDependent != other.IsTimeDependent:
            return False
        if self.IsTimeDependent and self.OriginalTimeFunction is not other.OriginalTimeFunction:
            return False
        if self.DebugPotential or other.DebugPotential:
            return False
        for a, b in zip(self.GeometryList, other.GeometryList):
            if a.GetStorageId() != b.GetStorageId():
                return False
            pa, pb = a.GetBasisPairs(), b.GetBasisPairs()
            if (pa is None) != (pb is None):
                return False
            if pa is not None and (pa.shape != pb.shape or np.any(pa != pb)):
                return False
        return True
