"""Angular ranks: reduced spherical harmonics (fixed m) and coupled two-electron harmonics.

Reduced spherical harmonics follow ``core/transform/reducedspherical/reducedsphericaltools.cpp``:
an (lmax+1)-point Gauss-Legendre rule in cos(theta) (``:283-305``) and associated Legendre
functions normalised so that the theta integral of P_lm P_l'm with the rule's weights is
delta_ll' (``:311-364``, norm ``sqrt((2l+1)/(4pi) (l-|m|)!/(l+|m|)!) * sqrt(2pi)``).
The l grid of the basis representation is ``|m|, |m|+1, ..., lmax``
(``core/representation/reducedspherical/lrange.h``).
"""
from __future__ import annotations

import math

import numpy as np

from .bspline import gauss_legendre


def normalized_legendre(lmax, m, x):
    """sqrt((2l+1)/2 (l-m)!/(l+m)!) P_l^m(x) for l = m..lmax (columns), Condon-Shortley phase
    included (as scipy's lpmv), by the three-term recurrence in l of the normalised functions,
    which stays finite where the factorials overflow (l > 170)."""
    x = np.asarray(x, dtype=np.float64)
    s = np.sqrt(np.maximum(0.0, 1.0 - x * x))
    q = np.full_like(x, math.sqrt(0.5))
    for k in range(1, m + 1):  # Q_k^k = -sqrt((2k+1)/(2k)) sin(theta) Q_{k-1}^{k-1}
        q = -math.sqrt((2.0 * k + 1.0) / (2.0 * k)) * s * q
    out = np.empty((len(x), lmax - m + 1))
    out[:, 0] = q
    if lmax > m:
        out[:, 1] = math.sqrt(2.0 * m + 3.0) * x * q
    for l in range(m + 2, lmax + 1):
        a = math.sqrt((4.0 * l * l - 1.0) / (l * l - m * m))
        b = math.sqrt(((l - 1.0) ** 2 - m * m) / (4.0 * (l - 1.0) ** 2 - 1.0))
        out[:, l - m] = a * (x * out[:, l - m - 1] - b * out[:, l - m - 2])
    return out


class ReducedSphericalTools:
    """Theta quadrature and normalised associated Legendre tables for one m."""

    def __init__(self, lmax, m=0):
        self.LMax = int(lmax)
        self.M = int(m)
        x, w = gauss_legendre(self.LMax + 1)
        self.ThetaGrid = np.arccos(x)
        self.Weights = w
        ls = np.arange(abs(self.M), self.LMax + 1)
        self.l_values = ls
        cos_t = np.cos(self.ThetaGrid)
        sign = (-1.0) ** self.M if self.M > 0 else 1.0
        P = sign * normalized_legendre(self.LMax, abs(self.M), cos_t)
        self.AssocLegendrePoly = P
        D = np.zeros_like(P)
        for idx, l in enumerate(ls):
            if idx > 0:
                nrm = math.sqrt((2 * l + 1.0) / (2 * l - 1.0) * (l - abs(self.M)) / float(l + abs(self.M)))
                D[:, idx] = l * cos_t * P[:, idx] - (l + self.M) * nrm * P[:, idx - 1]
        self.AssocLegendrePolyDerivative = D

    def GetSize(self):
        """Number of l channels minus one (``reducedsphericaltools.h:53``)."""
        return self.LMax - abs(self.M)

    def project_pairs(self, values, pairs, differentiation=0):
        """Angular matrix elements ``sum_theta P_row f P_col w`` for each (row, col) pair.

        ``values`` has theta as its first axis; the result has the pair index first
        (``core/tensorpotential/basis_reducedspherical.h:12-73``).
        """
        left = self.AssocLegendrePoly
        right = self.AssocLegendrePoly if differentiation == 0 else self.AssocLegendrePolyDerivative
        if differentiation not in (0, 1):
            raise ValueError("Reduced spherical harmonics support differentiation 0 or 1")
        coef = left[:, pairs[:, 0]] * right[:, pairs[:, 1]] * self.Weights[:, None]  # (ntheta, npairs)
        return np.tensordot(coef, values, axes=([0], [0]))


def dipole_selection_pairs(nchannels):
    """Pairs (l, l-1), (l, l+1) in the order of ``GeometryInfoReducedSphHarmSelectionRule``
    (``pyprop/tensorpotential/basis/ReducedSphericalHarmonic.py:20-34``)."""
    pairs = []
    for i in range(nchannels):
        if i > 0:
            pairs.append((i, i - 1))
        if i < nchannels - 1:
            pairs.append((i, i + 1))
    return np.asarray(pairs, dtype=np.int32).reshape(-1, 2)


# ---------------------------------------------------------------------------------------
# coupled spherical harmonics for two electrons
# ---------------------------------------------------------------------------------------


class CoupledIndex:
    __slots__ = ("l1", "l2", "L", "M")

    def __init__(self, l1, l2, L, M):
        self.l1, self.l2, self.L, self.M = l1, l2, L, M

    def __repr__(self):
        return "CoupledIndex(l1=%d, l2=%d, L=%d, M=%d)" % (self.l1, self.l2, self.L, self.M)


class DefaultCoupledIndexIterator:
    """All (l1, l2, L, M) with l1, l2 <= lmax, |l1-l2| <= L <= l1+l2, |M| <= L, in the order of
    ``pyprop/CoupledSphericalHarmonics.py:14-83``: M outer, then L, then l1, then l2.
    L defaults to ``range(lmax+1)``; L and M are made unique and sorted."""

    def __init__(self, lmax, L=None, M=(0,), fullTensor=False):
        if L is None:
            L = range(lmax + 1)
        if not hasattr(L, "__iter__"):
            L = [L]
        if not hasattr(M, "__iter__"):
            M = [M]
        self.lmax = lmax
        self.L = sorted(set(int(x) for x in L))
        self.M = sorted(set(int(x) for x in M))
        self.fullTensor = fullTensor

    def __iter__(self):
        for M in self.M:
            for L in self.L:
                if abs(M) > L and not self.fullTensor:
                    continue
                for l1 in range(self.lmax + 1):
                    for l2 in range(self.lmax + 1):
                        if self.fullTensor or abs(l1 - l2) <= L <= l1 + l2:
                            yield CoupledIndex(l1, l2, L, M)

    def __repr__(self):
        return "DefaultCoupledIndexIterator(lmax=%d, L=%r, M=%r)" % (self.lmax, self.L, self.M)
