"""Combined representation and device wavefunction.

``CombinedRepresentation`` holds one basis per rank (angular, radial) and the overlap of
the non-orthogonal B-spline rank; its overlap operations run on the GPU and follow
``core/representation/combinedrepresentation.cpp:164-238`` (MultiplyOverlap, SolveOverlap,
MultiplySqrtOverlap, SolveSqrtOverlap with S = U^H U) and the S-weighted inner product of
``:423-474``. ``Wavefunction`` mirrors ``core/wavefunction.h`` (GetData, GetNorm,
InnerProduct, Normalize, Copy) with its data a complex128 CUDA tensor.
"""
from __future__ import annotations

import numpy as np

from . import _native as nat
from .gpu import Banded, Context, DeviceOperator, torch, vec_dot
from .tensorpotential import BSplineRankBasis


class CombinedRepresentation:
    def __init__(self, bases):
        self.bases = list(bases)
        self.radial = self.bases[-1]
        if not isinstance(self.radial, BSplineRankBasis):
            raise ValueError("the last rank must be the B-spline radial rank")
        bs = self.radial.BSplineObject
        self.kb = bs.MaxSplineOrder - 1
        self.overlap_rows = bs.overlap_band().real.copy()
        self._ovl = None

    def GetFullShape(self):
        return tuple(b.size for b in self.bases)

    def GetRank(self):
        return len(self.bases)

    def IsOrthogonalBasis(self, rank):
        return bool(self.bases[rank].orthogonal)

    def GetRepresentation(self, rank):
        return self.bases[rank]

    # -- device overlap -------------------------------------------------------------------
    def _overlap(self):
        if self._ovl is None:
            ctx = Context.get()
            shape = self.GetFullShape()
            if len(shape) == 3 and (shape[1] != shape[2] or not isinstance(self.bases[1], BSplineRankBasis)):
                raise ValueError("two-electron ranks must share one B-spline basis")
            # an empty operator only carries the shape/precision for the banded object
            self._ovl_op = _ShapeOp(ctx, shape, self.kb)
            self._ovl = Banded.overlap(self._ovl_op, self.overlap_rows)
        return self._ovl

    def _radial(self, which, data):
        """A banded overlap operation along every B-spline rank (for two electrons the library
        applies it along both radial ranks)."""
        self._overlap().apply(which, data)

    def MultiplyOverlap(self, psi):
        self._radial(nat.PG_BAND_MUL_S, psi.GetData())

    def MultiplyIntegrationWeights(self, psi):
        """The integration weights of every rank (combinedrepresentation.cpp:93-130): the overlap
        on the B-spline ranks, 1 on the angular basis ranks."""
        self._radial(nat.PG_BAND_MUL_S, psi.GetData())

    def SolveOverlap(self, psi):
        self._radial(nat.PG_BAND_SOLVE_S, psi.GetData())

    def MultiplySqrtOverlap(self, conj, psi):
        self._radial(nat.PG_BAND_MUL_UT if conj else nat.PG_BAND_MUL_U, psi.GetData())

    def SolveSqrtOverlap(self, conj, psi):
        self._radial(nat.PG_BAND_SOLVE_UT if conj else nat.PG_BAND_SOLVE_U, psi.GetData())

    def InnerProduct(self, psi1, psi2):
        """<psi1 | S | psi2> over the B-spline ranks (Euclidean over the angular rank)."""
        tmp = psi2.GetData().clone()
        self._radial(nat.PG_BAND_MUL_S, tmp)
        return vec_dot(Context.get(), psi1.GetData(), tmp)


class _ShapeOp(DeviceOperator):
    """A finalized operator with no terms: gives banded objects their shape and precision."""

    def __init__(self, ctx, shape, kb, precision=nat.PG_FP64):
        super().__init__(ctx, [], shape, kb, precision)


class Wavefunction:
    def __init__(self, representation, data=None):
        self.Representation = representation
        self._data = data

    @property
    def data(self):
        """complex128 CUDA tensor [Nang][N], allocated on first use."""
        if self._data is None:
            t = torch()
            self._data = t.zeros(self.Representation.GetFullShape(), dtype=t.complex128, device="cuda")
        return self._data

    @data.setter
    def data(self, value):
        self._data = value

    def GetData(self):
        return self.data

    def SetData(self, array):
        t = torch()
        self.data.copy_(t.as_tensor(np.asarray(array), dtype=t.complex128))

    def GetRepresentation(self):
        return self.Representation

    def GetRank(self):
        return self.Representation.GetRank()

    def Copy(self):
        return Wavefunction(self.Representation, self.data.clone())

    CopyDeep = Copy

    def Clear(self):
        self.data.zero_()

    def InnerProduct(self, other):
        return self.Representation.InnerProduct(self, other)

    def GetNorm(self):
        return float(np.sqrt(max(self.InnerProduct(self).real, 0.0)))

    def Normalize(self):
        n = self.GetNorm()
        if n > 0:
            self.data /= n
        return n

    def numpy(self):
        return self.data.detach().cpu().numpy()
