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


def _project(bases, geoms, conf, data, ranks):
    """Represent the grid axes ``ranks`` of ``data`` in their bases, last rank first
    (``TensorPotentialGenerator.py:80-274``)."""
    for r in reversed(ranks):
        geom = geoms[r]
        if not geom.UseGrid:
            continue
        diff = conf.Get("differentiation%d" % r) if conf.Exists("differentiation%d" % r) else 0
        moved = np.moveaxis(data, r, -1 if isinstance(bases[r], BSplineRankBasis) else 0)
        projected = bases[r].represent(moved, geom, diff)
        data = np.moveaxis(projected, -1 if isinstance(bases[r], BSplineRankBasis) else 0, r)
    return data


def generate_potential(bases, conf):
    """Evaluate ``conf``'s potential on the tensor grid and represent it in the bases.

    Returns ``(geometry_list, PotentialData)`` with ``PotentialData`` of shape
    ``(pairs_rank0, pairs_rank1, ...)``, or ``(geometry_list, FactoredPotential)`` for a
    two-electron term that factorizes (see :func:`factorize_potential`).
    """
    rank = len(bases)
    geoms = [bases[r].GetGeometryInfo(conf.Get("geometry%d" % r)) for r in range(rank)]
    evaluator = _evaluator_from_section(conf)
    if getattr(evaluator, "needs_basis", False):
        evaluator.bind(bases, geoms)
    grids = [bases[r].grid(geoms[r]) for r in range(rank)]
    pos = tuple(np.asarray(g).reshape([-1 if rr == r else 1 for rr in range(rank)]) for r, g in enumerate(grids))
    fac = factorize_potential(bases, geoms, conf, evaluator, pos)
    if fac is not None:
        return geoms, fac
    data = np.asarray(evaluator(pos), dtype=np.complex128)
    data = np.broadcast_to(data, tuple(len(g) for g in grids)).copy()
    return geoms, np.ascontiguousarray(_project(bases, geoms, conf, data, list(range(rank))))


class FactoredPotential:
    """A two-electron term as a sum of factors, angular coefficients x one radial operator:
    V(pair) = sum_q weights[q] * coefs[q][pair] * R_q.

    The reference evaluates such terms per angular pair (the electron-electron repulsion's
    multipoles in examples/tensor/helium_stabilization/coupledspherical.cpp:7-127, the laser
    coupling's two radial functions in coupledlength.cpp:9-124, and every term that does not
    depend on the angular pair) and stores one radial block per pair. Here each radial
    operator is kept once, as ``stencil[q][i1][d1][d2][i2]`` (the coupling of output
    (i1, i2) to input (i1 + d1 - k, i2 + d2 - k), real), with the coefficients per pair of
    the angular geometry. ``reference_data()`` expands it to the reference layout
    ``[pairs0][pairs1][pairs2]`` (small cases only: tests and the oracle)."""

    def __init__(self, pairs, coefs, weights, stencil, radial_pairs, kb, nangular):
        self.pairs = pairs            # [npairs][2] of the angular rank, or None (identity)
        self.coefs = coefs            # [Q][npairs] float64
        self.weights = weights        # [Q] complex128
        self.stencil = stencil        # [Q][N1][2k+1][2k+1][N2] float64
        self.radial_pairs = radial_pairs  # pair lists of ranks 1 and 2 (reference layout)
        self.kb = kb
        self.nangular = nangular

    @property
    def nfactors(self):
        return len(self.weights)

    def entries(self):
        """(rows, cols) of the angular pairs."""
        if self.pairs is None:
            a = np.arange(self.nangular, dtype=np.int32)
            return a, a
        return self.pairs[:, 0].astype(np.int32), self.pairs[:, 1].astype(np.int32)

    def reference_data(self):
        kb = self.kb
        p1, p2 = self.radial_pairs
        i1, j1 = p1[:, 0], p1[:, 1]
        i2, j2 = p2[:, 0], p2[:, 1]
        m1 = np.abs(j1 - i1) <= kb
        m2 = np.abs(j2 - i2) <= kb
        out = np.zeros((self.coefs.shape[1], len(p1), len(p2)), dtype=np.complex128)
        for q in range(self.nfactors):
            blk = np.zeros((len(p1), len(p2)))
            R = self.stencil[q]
            blk[np.ix_(m1, m2)] = R[i1[m1][:, None], (j1 - i1 + kb)[m1][:, None], (j2 - i2 + kb)[m2][None, :],
                                    i2[m2][None, :]]
            out += (self.weights[q] * self.coefs[q])[:, None, None] * blk[None]
        return out


def _radial_stencil(data2, pairs1, pairs2, N1, N2, kb):
    """Reference-layout radial block [pairs1][pairs2] -> stencil [N1][2k+1][2k+1][N2]."""
    b = 2 * kb + 1
    R = np.zeros((N1, b, b, N2), dtype=data2.dtype)
    i1, j1 = pairs1[:, 0], pairs1[:, 1]
    i2, j2 = pairs2[:, 0], pairs2[:, 1]
    m1 = np.abs(j1 - i1) <= kb
    m2 = np.abs(j2 - i2) <= kb
    sub = data2[np.ix_(m1, m2)]
    np.add.at(R, (i1[m1][:, None], (j1 - i1 + kb)[m1][:, None], (j2 - i2 + kb)[m2][None, :], i2[m2][None, :]), sub)
    return R


def _full_band(pairs, N, kb):
    """True when the in-band pairs of a radial geometry are the whole band |i - j| <= kb
    (the device projection writes every band entry)."""
    p = np.asarray(pairs)
    inside = p[np.abs(p[:, 1] - p[:, 0]) <= kb]
    return len({(int(i), int(j)) for i, j in inside}) == N * (2 * kb + 1) - kb * (kb + 1)


def gpu_setup_enabled():
    """Radial factors of two-electron terms are projected on the GPU when a CUDA device is
    present (PYPROP_GPU_SETUP=0 keeps the host projection, e.g. to compare the two)."""
    import os
    if os.environ.get("PYPROP_GPU_SETUP", "1") == "0":
        return False
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def _device_tables(bs):
    """Device copies of a B-spline basis's local tables: (first [nint] int32, values
    [nint][k][q], weights [nint*q]) as torch tensors, cached on the basis object."""
    import torch
    tabs = getattr(bs, "_gpu_tables", None)
    if tabs is None:
        idx, valid, cols, loc = bs._local()
        a0 = np.argmax(valid, axis=1)
        first = (idx[np.arange(idx.shape[0]), a0] - a0).astype(np.int32)
        tabs = (torch.as_tensor(first, device="cuda"), torch.as_tensor(np.ascontiguousarray(loc[0]), device="cuda"),
                torch.as_tensor(np.ascontiguousarray(bs.weights), device="cuda"))
        bs._gpu_tables = tabs
    return tabs


def radial_stencil_gpu(values, bs1, bs2):
    """The stencil [N1][2k-1][2k-1][N2] of a real function values[q1][q2] on the two radial
    quadrature grids (no derivatives), projected on the GPU by pg_bspline_band_project:
    along r2 for every r1 point, then along r1 for every (i2, d2) column. Equals the host
    ``_radial_stencil(_project(...))`` to rounding."""
    import torch
    from .gpu import Context, check, ptr
    ctx = Context.get()
    k = bs1.MaxSplineOrder
    if bs2.MaxSplineOrder != k:
        raise ValueError("both radial ranks need the same spline order")
    bw = 2 * k - 1
    N1, N2 = bs1.NumberOfBSplines, bs2.NumberOfBSplines
    nq1, nq2 = len(bs1.grid), len(bs2.grid)
    f1, B1, w1 = _device_tables(bs1)
    f2, B2, w2 = _device_tables(bs2)
    F = torch.as_tensor(np.ascontiguousarray(values, dtype=np.float64), device="cuda")
    if tuple(F.shape) != (nq1, nq2):
        raise ValueError("values must be given on the two quadrature grids")
    G = torch.empty((nq1, N2, bw), dtype=torch.float64, device="cuda")
    R = torch.empty((N1, bw, bw, N2), dtype=torch.float64, device="cuda")
    lib = ctx.lib
    ctx.bind_stream()
    check(lib.pg_bspline_band_project(ctx.h, ptr(F), nq1, 1, nq2, 1, B2.shape[0], k, B2.shape[2], ptr(f2), ptr(B2),
                                      ptr(w2), N2, ptr(G), N2 * bw, 0, bw, 1), "pg_bspline_band_project")
    check(lib.pg_bspline_band_project(ctx.h, ptr(G), N2 * bw, bw, 1, N2 * bw, B1.shape[0], k, B1.shape[2], ptr(f1),
                                      ptr(B1), ptr(w1), N1, ptr(R), 1, N2, bw * bw * N2, bw * N2),
          "pg_bspline_band_project")
    return R.cpu().numpy()


def factorize_potential(bases, geoms, conf, evaluator, pos):
    """FactoredPotential for a rank-3 term on a coupled angular rank and two banded B-spline
    ranks, or None (then the term is stored per pair as in the reference).

    Factors come from the evaluator's ``factors(pos)`` (a list of (radial function on the
    grid, coefficient per angular pair)); an evaluator that ignores the angular pair (no
    ``needs_basis``) is one factor with coefficient 1. Each radial function is projected with
    the section's geometries and differentiation exactly as the full potential would be, so
    the expansion equals the per-pair data up to rounding. ``factorize = False`` in the
    section keeps the per-pair form."""
    if len(bases) != 3 or not isinstance(bases[0], CoupledSphericalRankBasis):
        return None
    if conf.Exists("factorize") and not conf.Get("factorize"):
        return None
    if not all(isinstance(bases[r], BSplineRankBasis) for r in (1, 2)):
        return None
    if any(geoms[r].StorageId not in ("Simp", "BandNH") or not geoms[r].UseGrid for r in (1, 2)):
        return None
    kbs = [bases[r].BSplineObject.MaxSplineOrder - 1 for r in (1, 2)]
    if kbs[0] != kbs[1]:
        return None
    kb = kbs[0]
    for r in (1, 2):
        p = geoms[r].Pairs
        if geoms[r].StorageId == "Simp" and np.any(np.abs(p[:, 1] - p[:, 0]) > kb):
            return None
    g0 = geoms[0]
    npairs = 1 if g0.Pairs is None else len(g0.Pairs)
    if hasattr(evaluator, "factors"):
        facs = evaluator.factors(pos)
    elif not getattr(evaluator, "needs_basis", False):
        single = tuple(np.asarray(x)[:1] if i == 0 else x for i, x in enumerate(pos))
        facs = [(np.asarray(evaluator(single)), np.ones(npairs))]
    else:
        return None
    shape = (1, len(bases[1].grid(geoms[1])), len(bases[2].grid(geoms[2])))
    N1, N2 = bases[1].size, bases[2].size
    diffs = [conf.Get("differentiation%d" % r) if conf.Exists("differentiation%d" % r) else 0 for r in (1, 2)]
    on_gpu = diffs == [0, 0] and all(_full_band(geoms[r].Pairs, bases[r].size, kb) for r in (1, 2)) \
        and gpu_setup_enabled()
    stencils, coefs, weights = [], [], []
    for values, c in facs:
        c = np.asarray(c, dtype=np.float64).reshape(-1)
        if c.size != npairs or not np.any(c):
            continue
        v = np.broadcast_to(np.asarray(values, dtype=np.complex128), shape).copy()
        if on_gpu:
            # projection on the GPU (pg_bspline_band_project), real and imaginary parts
            bs1, bs2 = bases[1].BSplineObject, bases[2].BSplineObject
            parts = [(radial_stencil_gpu(p, bs1, bs2), w) for p, w in ((v[0].real, 1.0), (v[0].imag, 1j)) if np.any(p)]
        else:
            data2 = _project(bases, geoms, conf, v, [1, 2])[0]
            parts = [(_radial_stencil(p, geoms[1].Pairs, geoms[2].Pairs, N1, N2, kb), w)
                     for p, w in ((data2.real, 1.0), (data2.imag, 1j)) if np.any(p)]
        for stencil, w in parts:
            stencils.append(stencil)
            coefs.append(c)
            weights.append(w)
    if not stencils:
        return None
    return FactoredPotential(None if g0.Pairs is None else np.asarray(g0.Pairs, dtype=np.int32), np.asarray(coefs),
                             np.asarray(weights, dtype=np.complex128), np.asarray(stencils),
                             (geoms[1].Pairs, geoms[2].Pairs), kb, bases[0].size)


class TensorPotential:
    """A potential stored in the basis (``pyprop/tensorpotential/TensorPotential.py``).

    ``PotentialData`` has one axis per rank, each indexed by that rank's basis pairs;
    ``MultiplyPotential`` adds ``f(t) * V * src`` to ``dst`` (``:92-112``).
    """

    def __init__(self, psi):
        self.psi = psi
        self.GeometryList = None
        self._data = None
        self.Factors = None
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
        self.GeometryList, data = generate_potential(bases, conf)
        if isinstance(data, FactoredPotential):
            self.Factors = data
        else:
            self.PotentialData = data

    @property
    def PotentialData(self):
        """Reference-layout data; a factorized term expands on first use (small cases)."""
        if self._data is None and self.Factors is not None:
            self._data = self.Factors.reference_data()
        return self._data

    @PotentialData.setter
    def PotentialData(self, value):
        self._data = value

    def SetupStep(self, timestep):
        self.BasisPairs = [g.GetBasisPairs() for g in self.GeometryList]
        self.StorageIds = "_".join(g.GetStorageId() for g in self.GeometryList)

    def GetTimeScaling(self, t):
        return float(self.TimeFunction(t)) if self.IsTimeDependent else 1.0

    def _device_operator(self):
        """This potential alone as a device operator (FP64), built on first use."""
        if getattr(self, "_op", None) is None:
            from . import _native as nat
            from .gpu import Context, DeviceOperator
            repr_ = self.psi.GetRepresentation()
            if getattr(self, "BasisPairs", None) is None:
                self.SetupStep(0.0)
            self._op = DeviceOperator(Context.get(), [self], repr_.GetFullShape(), repr_.kb, nat.PG_FP64)
        return self._op

    def MultiplyPotential(self, srcPsi, destPsi, t, timeStep):
        """destPsi += f(t) V srcPsi on the device (TensorPotential.py:92-112)."""
        op = self._device_operator()
        op.matvec(op.scales(t), srcPsi.GetData(), destPsi.GetData(), accumulate=True)

    def GetExpectationValue(self, psi, tmpPsi, t, timeStep):
        """<psi|V|psi>: tmpPsi = S^-1 V psi, then the S-weighted inner product with psi
        (TensorPotential.py:117-125)."""
        tmpPsi.Clear()
        self.MultiplyPotential(psi, tmpPsi, t, timeStep)
        repr_ = psi.GetRepresentation()
        repr_.SolveOverlap(tmpPsi)
        return psi.InnerProduct(tmpPsi)

    def CanConsolidate(self, other):
        """Same time dependence, same storage and basis pairs in every rank (``:128-163``)."""
        if self.Factors is not None or other.Factors is not None:
            return False  # factorized terms stay separate (their factors are merged on the device)
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
