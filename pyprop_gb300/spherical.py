"""Angular ranks: reduced spherical harmonics (fixed m) and coupled two-electron harmonics.

Reduced spherical harmonics follow ``core/transform/reducedspherical/reducedsphericaltools.cpp``:
an (lmax+1)-point Gauss-Legendre rule in cos(theta) (``:283-305``) and associated Legendre
functions normalised so that the theta integral of P_lm P_l'm with the rule's weights is
delta_ll' (``:311-364``, norm ``sqrt((2l+1)/(4pi) (l-|m|)!/(l+|m|)!) * sqrt(2pi)``).
The l grid of the basis representation is ``|m|, |m|+1, ..., lmax``
(``core/representation/reducedspherical/lrange.h``).
"""
from __future__ import annotations

import functools
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


def clebsch_gordan(j1, j2, m1, m2, J, M):
    """<j1 m1 j2 m2 | J M> for integer angular momenta (Racah's closed form, evaluated with
    log-factorials), the coefficient ``CoupledSpherical::ClebschGordan`` returns as
    ``cg(j1, j2, m1, m2, J, M)``. Zero outside the selection rules."""
    if m1 + m2 != M or abs(m1) > j1 or abs(m2) > j2 or abs(M) > J:
        return 0.0
    if J < abs(j1 - j2) or J > j1 + j2:
        return 0.0
    lf = math.lgamma

    def f(n):
        return lf(n + 1.0)

    pre = 0.5 * (math.log(2.0 * J + 1.0) + f(J + j1 - j2) + f(J - j1 + j2) + f(j1 + j2 - J) - f(j1 + j2 + J + 1)
                 + f(J + M) + f(J - M) + f(j1 - m1) + f(j1 + m1) + f(j2 - m2) + f(j2 + m2))
    total = 0.0
    kmin = max(0, j2 - J - m1, j1 - J + m2)
    kmax = min(j1 + j2 - J, j1 - m1, j2 + m2)
    for k in range(kmin, kmax + 1):
        den = (f(k) + f(j1 + j2 - J - k) + f(j1 - m1 - k) + f(j2 + m2 - k) + f(J - j2 + m1 + k)
               + f(J - j1 - m2 + k))
        total += (-1.0) ** k * math.exp(pre - den)
    return total


class CoupledSphericalBasis:
    """The coupled two-electron angular basis ``CoupledSphericalHarmonicRepresentation``:
    an ordered list of (l1, l2, L, M) from an index iterator."""

    def __init__(self, index_iterator):
        self.indices = list(index_iterator)
        self.size = len(self.indices)

    def pairs(self, rule):
        """(left, right) pairs accepted by ``rule(left, right)``, left-major
        (core/tensorpotential/coupledsphericalselectionrule.h:16-52)."""
        out = [(i, j) for i, a in enumerate(self.indices) for j, b in enumerate(self.indices) if rule(a, b)]
        return np.asarray(out, dtype=np.int32).reshape(-1, 2)


def rule_diagonal(a, b):
    """``CoupledSphericalSelectionRuleDiagonal`` (coupledsphericalselectionrule.h:357-367)."""
    return a.L == b.L and a.M == b.M and a.l1 == b.l1 and a.l2 == b.l2


def rule_r12_old(a, b):
    """``CoupledSphericalSelectionRuleR12Old`` (:58-86): equal L, M and both triangles."""
    return (a.L == b.L and a.M == b.M and a.L <= a.l1 + a.l2 and abs(a.l1 - a.l2) <= a.L
            and b.L <= b.l1 + b.l2 and abs(b.l1 - b.l2) <= b.L)


def r12_angular_sum(left, right, l3):
    """The angular factor of the multipole l3 of 1/|r1 - r2| between coupled states
    (examples/tensor/helium_stabilization/coupledspherical.cpp:63-92): the m-sum over four
    Clebsch-Gordan coefficients times the l3 coefficient, without the radial r<^l3/r>^(l3+1)."""
    L, M = left.L, left.M
    l1p, l2p, l1, l2 = left.l1, left.l2, right.l1, right.l2
    coef = (math.sqrt((2.0 * l1p + 1.0) * (2.0 * l1 + 1.0) / (2.0 * l3 + 1.0))
            * math.sqrt((2.0 * l2p + 1.0) * (2.0 * l2 + 1.0) / (2.0 * l3 + 1.0)) / (2.0 * l3 + 1.0)
            * clebsch_gordan(l1p, l1, 0, 0, l3, 0) * clebsch_gordan(l2p, l2, 0, 0, l3, 0))
    if coef == 0.0:
        return 0.0
    stop = max(l1, l1p, l2, l2p)
    s = 0.0
    for m1p in range(-stop, stop + 1):
        m2p = M - m1p
        for m1 in range(-stop, stop + 1):
            m2 = M - m1
            m3 = m1 - m1p
            cur = (clebsch_gordan(l1p, l2p, m1p, m2p, L, M) * clebsch_gordan(l1, l2, m1, m2, L, M)
                   * clebsch_gordan(l1p, l1, -m1p, m1, l3, m3) * clebsch_gordan(l2p, l2, -m2p, m2, l3, -m3))
            if cur != 0.0:
                s += cur * (-1.0) ** (m1p + m2p + m3)
    return s * coef


@functools.lru_cache(maxsize=None)
def wigner_6j(j1, j2, j3, j4, j5, j6):
    """{j1 j2 j3; j4 j5 j6} for integer arguments (Racah's single sum, log-factorials)."""
    def ok(a, b, c):
        return abs(a - b) <= c <= a + b

    if not (ok(j1, j2, j3) and ok(j1, j5, j6) and ok(j4, j2, j6) and ok(j4, j5, j3)):
        return 0.0
    f = _log_factorial

    def tri(a, b, c):
        return 0.5 * (f(a + b - c) + f(a - b + c) + f(-a + b + c) - f(a + b + c + 1))

    pre = tri(j1, j2, j3) + tri(j1, j5, j6) + tri(j4, j2, j6) + tri(j4, j5, j3)
    tmin = max(j1 + j2 + j3, j1 + j5 + j6, j4 + j2 + j6, j4 + j5 + j3)
    tmax = min(j1 + j2 + j4 + j5, j2 + j3 + j5 + j6, j3 + j1 + j6 + j4)
    total = 0.0
    for t in range(tmin, tmax + 1):
        den = (f(t - j1 - j2 - j3) + f(t - j1 - j5 - j6) + f(t - j4 - j2 - j6) + f(t - j4 - j5 - j3)
               + f(j1 + j2 + j4 + j5 - t) + f(j2 + j3 + j5 + j6 - t) + f(j3 + j1 + j6 + j4 - t))
        total += (-1.0) ** t * math.exp(pre + f(t + 1) - den)
    return total


def _log_factorial(n):
    return math.lgamma(n + 1.0)


@functools.lru_cache(maxsize=None)
def reduced_c(lp, k, l):
    """<lp || C^k || l> = (-1)^lp sqrt((2lp+1)(2l+1)) (lp k l; 0 0 0), the reduced matrix
    element of the renormalised spherical harmonic C^k = sqrt(4 pi / (2k+1)) Y_k."""
    three_j = (-1.0) ** (lp - k) / math.sqrt(2.0 * l + 1.0) * clebsch_gordan(lp, k, 0, 0, l, 0)
    return (-1.0) ** lp * math.sqrt((2.0 * lp + 1.0) * (2.0 * l + 1.0)) * three_j


def r12_angular_factor(left, right, l3):
    """The same factor as :func:`r12_angular_sum`, in closed form: the matrix element of
    P_l3(cos theta_12) = C^l3(1) . C^l3(2) between coupled states,
    (-1)^(l1 + l2' + L) {l1' l2' L; l2 l1 l3} <l1'||C^l3||l1> <l2'||C^l3||l2>
    (left = (l1', l2', L), right = (l1, l2, L)). One 6j symbol instead of the double m-sum
    over four Clebsch-Gordan coefficients; the two agree to rounding."""
    if left.L != right.L or left.M != right.M:
        return 0.0
    L = left.L
    l1p, l2p, l1, l2 = left.l1, left.l2, right.l1, right.l2
    c = reduced_c(l1p, l3, l1)
    if c == 0.0:
        return 0.0
    c *= reduced_c(l2p, l3, l2)
    if c == 0.0:
        return 0.0
    return (-1.0) ** (l1 + l2p + L) * wigner_6j(l1p, l2p, L, l2, l1, l3) * c


def r12_multipoles(left, right):
    """l3 range of the multipole expansion between two coupled states (:60-61)."""
    if left.L != right.L or left.M != right.M:
        return range(0)
    return range(max(abs(right.l1 - left.l1), abs(right.l2 - left.l2)), min(right.l1 + left.l1, right.l2 + left.l2) + 1)


def rule_linear_polarized_field(a, b):
    """``CoupledSphericalSelectionRuleLinearPolarizedField`` (coupledsphericalselectionrule.h:
    333-355): L changes by one, M kept, one electron's l changes by one, the other's is kept."""
    if abs(a.L - b.L) != 1 or a.M != b.M:
        return False
    return (abs(a.l1 - b.l1) == 1 and a.l2 == b.l2) or (abs(a.l2 - b.l2) == 1 and a.l1 == b.l1)


def laser_length_factors(left, right):
    """(I1, I2): the angular factors of the length-gauge coupling r1 I1 + r2 I2 between coupled
    states (examples/tensor/helium_stabilization/coupledlength.cpp:44-124). As in the reference,
    the single-electron factor is <l m|Y_10|l' m> (cos(theta) = sqrt(4 pi / 3) Y_10) with its
    sign convention (the m >= 0 Condon-Shortley phase divided out)."""
    if abs(left.L - right.L) != 1 or left.M != right.M:
        return 0.0, 0.0
    L, M, l1, l2 = left.L, left.M, left.l1, left.l2
    Lp, l1p, l2p = right.L, right.l1, right.l2

    def coef(l, lp):
        return math.sqrt((2 * l + 1.0) * (2 * lp + 1.0) / (12 * math.pi))

    def cs(m):
        return 1.0 if m < 0 else (-1.0) ** m

    I1 = I2 = 0.0
    stop = max(l1, l1p, l2, l2p)
    for m1 in range(-stop, stop + 1):
        m2 = M - m1
        if abs(m1) > l1 or abs(m1) > l1p or abs(m2) > l2 or abs(m2) > l2p:
            continue
        base = clebsch_gordan(l1, l2, m1, m2, L, M) * clebsch_gordan(l1p, l2p, m1, m2, Lp, M)
        if base == 0.0:
            continue
        I1 += base * coef(l1, l1p) * clebsch_gordan(l1, l1p, 0, 0, 1, 0) * clebsch_gordan(l1, l1p, -m1, m1, 1, 0) / cs(m1)
        I2 += base * coef(l2, l2p) * clebsch_gordan(l2, l2p, 0, 0, 1, 0) * clebsch_gordan(l2, l2p, -m2, m2, 1, 0) / cs(m2)
    return I1, I2
