"""Potential evaluators and laser time functions used by the tensor-potential generator.

Each evaluator mirrors a C++ ``GetPotentialValue(pos)`` class of the reference examples
(``examples/tensor/helium_stabilization_sae/potential.cpp``) but is evaluated on the whole
tensor grid at once: ``pos`` is a tuple with one broadcastable numpy array per rank. A rank
represented in its basis (geometry "Diagonal") passes basis values (the l of each
channel); a rank on its grid passes grid points (theta, r).
"""
from __future__ import annotations

import numpy as np


class PotentialBase:
    def ApplyConfigSection(self, conf):
        for key in getattr(self, "_keys", ()):
            if conf.Exists(key):
                setattr(self, key, conf.Get(key))

    def __call__(self, pos, t=0.0):
        return self.GetPotentialValue(pos)


class KineticEnergyPotential(PotentialBase):
    """Constant ``-1/(2 mass)``, used with ``differentiation=2`` (potential.cpp:6-35)."""
    _keys = ("mass",)
    mass = 1.0

    def GetPotentialValue(self, pos):
        shape = np.broadcast(*pos).shape
        return np.full(shape, -1.0 / (2.0 * self.mass))


class AngularKineticEnergyPotential(PotentialBase):
    """``l(l+1) / (2 mass r^2)`` with l from the angular rank's basis values
    (potential.cpp:219-253)."""
    _keys = ("mass", "angular_rank", "radial_rank")
    mass = 1.0
    angular_rank = 0
    radial_rank = 1

    def GetPotentialValue(self, pos):
        l = pos[self.angular_rank]
        r = pos[self.radial_rank]
        return l * (l + 1.0) / (2.0 * self.mass * r * r)


class CoulombPotential(PotentialBase):
    """Nuclear attraction ``-z / sqrt(r^2 + soft^2)``; ``soft = 0`` gives the pure ``-z/r``."""
    _keys = ("z", "soft", "radial_rank", "charge")
    z = 1.0
    soft = 0.0
    radial_rank = 1

    def GetPotentialValue(self, pos):
        r = pos[self.radial_rank]
        return -self.z / np.sqrt(r * r + self.soft * self.soft) + 0.0 * np.broadcast_to(0.0, np.broadcast(*pos).shape)


class SingleActiveElectronPotential(PotentialBase):
    """Model potential ``-(Z + a1 e^{-a2 r} + a3 r e^{-a4 r} + a5 e^{-a6 r}) / sqrt(r^2+soft^2)``
    (potential.cpp:256-314)."""
    _keys = ("z", "a1", "a2", "a3", "a4", "a5", "a6", "soft", "radial_rank")
    z = 1.0
    a1 = a2 = a3 = a4 = a5 = a6 = 0.0
    soft = 0.0
    radial_rank = 1

    def GetPotentialValue(self, pos):
        r = np.abs(pos[self.radial_rank])
        V = -(self.z + self.a1 * np.exp(-self.a2 * r) + self.a3 * r * np.exp(-self.a4 * r)
              + self.a5 * np.exp(-self.a6 * r)) / np.sqrt(r * r + self.soft * self.soft)
        return V + 0.0 * np.broadcast_to(0.0, np.broadcast(*pos).shape)


class DipoleLaserPotentialLength(PotentialBase):
    """Length-gauge dipole ``-charge * r * cos(theta)`` (potential.cpp:75-109)."""
    _keys = ("angular_rank", "radial_rank", "charge")
    angular_rank = 0
    radial_rank = 1
    charge = -1.0

    def GetPotentialValue(self, pos):
        theta = pos[self.angular_rank]
        r = pos[self.radial_rank]
        return -self.charge * r * np.cos(theta)


class OverlapPotential(PotentialBase):
    """Constant 1 with ``differentiation=0``: represents S itself in a rank."""

    def GetPotentialValue(self, pos):
        return np.ones(np.broadcast(*pos).shape)


class ComplexAbsorbingPotential(PotentialBase):
    """Complex absorber ``factor_real x^scaling_real + i factor_imag x^scaling_imag`` with
    ``x = (r - absorber_start)/absorber_length`` on ``start < r <= start + length``, zero
    elsewhere (potential.cpp ``ComplexAbsorbingPotential``)."""
    _keys = ("radial_rank", "scaling_real", "scaling_imag", "factor_real", "factor_imag",
             "absorber_start", "absorber_length")
    radial_rank = 1
    scaling_real = 1.0
    scaling_imag = 1.0
    factor_real = 0.0
    factor_imag = -1.0
    absorber_start = 0.0
    absorber_length = 1.0

    def GetPotentialValue(self, pos):
        r = pos[self.radial_rank]
        inside = (self.absorber_start < r) & (r <= self.absorber_start + self.absorber_length)
        x = np.where(inside, (r - self.absorber_start) / self.absorber_length, 0.0)
        val = np.where(inside, self.factor_real * x ** self.scaling_real
                       + 1j * self.factor_imag * x ** self.scaling_imag, 0.0)
        return np.broadcast_to(val, np.broadcast(*pos).shape).astype(np.complex128)


# ---------------------------------------------------------------------------------------
# laser time functions (examples/tensor/helium_stabilization_sae/example.py:220-273)
# ---------------------------------------------------------------------------------------


def LaserFunctionSimpleLength(conf, t):
    """``E0 sin^2(pi t / T) cos(w t)`` for 0 <= t < T, else 0."""
    if 0 <= t < conf.pulse_duration:
        return conf.amplitude * np.sin(t * np.pi / conf.pulse_duration) ** 2 * np.cos(t * conf.frequency)
    return 0.0


def LaserFunctionVelocity(conf, t):
    """``-E0 sin^2(pi t / T) cos(w t + phase)`` for 0 <= t < T, else 0."""
    phase = getattr(conf, "phase", 0.0)
    if 0 <= t < conf.pulse_duration:
        return -conf.amplitude * np.sin(t * np.pi / conf.pulse_duration) ** 2 * np.cos(t * conf.frequency + phase)
    return 0.0


def LaserFunctionLength(conf, t):
    """Time derivative of the velocity-gauge sin^2 pulse (example.py:243-252)."""
    if 0 <= t < conf.pulse_duration:
        T = conf.pulse_duration
        w = conf.frequency
        return conf.amplitude * np.sin(np.pi * t / T) * (
            -2 * np.pi / T * np.cos(np.pi * t / T) * np.cos(w * t) + w * np.sin(np.pi * t / T) * np.sin(w * t))
    return 0.0


def LaserFunctionFlatTop(conf, t):
    """Flat-top pulse with sin^2 ramps (example.py:254-273)."""
    start = getattr(conf, "pulse_start", 0.0)
    field = conf.amplitude * np.cos(t * conf.frequency)
    if t > conf.pulse_duration or t < start:
        return 0.0
    if 0 <= t < conf.ramp_on_time:
        return field * np.sin(t * np.pi / (2 * conf.ramp_on_time)) ** 2
    if t > conf.pulse_duration - conf.ramp_off_time:
        return field * np.sin((conf.pulse_duration - t) * np.pi / (2 * conf.ramp_off_time)) ** 2
    return field


POTENTIAL_CLASSES = {cls.__name__: cls for cls in (
    KineticEnergyPotential, AngularKineticEnergyPotential, CoulombPotential,
    SingleActiveElectronPotential, DipoleLaserPotentialLength, OverlapPotential,
    ComplexAbsorbingPotential)}

TIME_FUNCTIONS = {f.__name__: f for f in (
    LaserFunctionSimpleLength, LaserFunctionVelocity, LaserFunctionLength, LaserFunctionFlatTop)}


class SingleIonizationBox(PotentialBase):
    """1 where one electron is beyond ``inner_box_size`` and the other within ``width``, else 0
    (examples/tensor/helium_stabilization/potential.cpp:190-218): its expectation value is the
    probability of single ionization."""
    _keys = ("radial_rank_1", "radial_rank_2", "inner_box_size", "width")
    radial_rank_1 = 1
    radial_rank_2 = 2
    inner_box_size = 20.0
    width = 20.0

    def GetPotentialValue(self, pos):
        r1, r2 = pos[self.radial_rank_1], pos[self.radial_rank_2]
        inside = ((r1 > self.inner_box_size) & (r2 < self.width)) | ((r2 > self.inner_box_size) & (r1 < self.width))
        return np.broadcast_to(inside.astype(np.float64), np.broadcast(*pos).shape)


class DoubleIonizationBox(SingleIonizationBox):
    """1 where both electrons are beyond ``inner_box_size``, else 0 (potential.cpp:220-247):
    its expectation value is the probability of double ionization."""

    def GetPotentialValue(self, pos):
        r1, r2 = pos[self.radial_rank_1], pos[self.radial_rank_2]
        inside = (r1 > self.inner_box_size) & (r2 > self.inner_box_size)
        return np.broadcast_to(inside.astype(np.float64), np.broadcast(*pos).shape)


def register_potential(cls):
    """Make a user evaluator class available to ``classname = "..."`` in configs."""
    POTENTIAL_CLASSES[cls.__name__] = cls
    return cls


# ---------------------------------------------------------------------------------------
# two-electron (coupled spherical harmonics) evaluators
# ---------------------------------------------------------------------------------------
# The coupled angular rank is never on a grid: its "coordinate" is the index of an angular
# basis pair, and these evaluators are bound to the angular basis and its pair list before
# they are evaluated (``bind``), as the reference's custom evaluators receive the basis pairs
# (examples/tensor/helium_stabilization/coupledspherical.cpp, coupledbase.h).


class CoupledPotentialBase(PotentialBase):
    _keys = ("angular_rank", "radial_rank1", "radial_rank2", "mass", "z")
    angular_rank = 0
    radial_rank1 = 1
    radial_rank2 = 2
    mass = 1.0
    needs_basis = True

    def bind(self, bases, geoms):
        self.basis = bases[self.angular_rank]
        self.pairs = geoms[self.angular_rank].GetBasisPairs()

    def _left_right(self):
        idx = self.basis.indices
        return [(idx[int(a)], idx[int(b)]) for a, b in self.pairs]


class CoupledSphericalCoulombPotential(PotentialBase):
    """Nuclear attraction of both electrons, ``-z/r1 - z/r2`` (potential.cpp:44-78)."""
    _keys = ("z", "radial_rank1", "radial_rank2")
    z = 2.0
    radial_rank1 = 1
    radial_rank2 = 2

    def GetPotentialValue(self, pos):
        r1, r2 = pos[self.radial_rank1], pos[self.radial_rank2]
        return np.broadcast_to(-self.z / r1 - self.z / r2, np.broadcast(*pos).shape)


class CoupledSphericalKineticEnergyEvaluator(CoupledPotentialBase):
    """Angular kinetic energy ``l1(l1+1)/(2 m r1^2) + l2(l2+1)/(2 m r2^2)`` on pairs of equal
    coupled indices, zero on others (coupledspherical.cpp:132-210)."""

    def GetPotentialValue(self, pos):
        r1, r2 = pos[self.radial_rank1], pos[self.radial_rank2]
        lr = self._left_right()
        shape = np.broadcast(*pos).shape
        out = np.zeros(shape)
        for p, (a, b) in enumerate(lr):
            if (a.L, a.M, a.l1, a.l2) != (b.L, b.M, b.l1, b.l2):
                continue
            sl = [slice(None)] * len(shape)
            sl[self.angular_rank] = p
            v = a.l1 * (a.l1 + 1.0) / (2.0 * self.mass * r1 * r1) + a.l2 * (a.l2 + 1.0) / (2.0 * self.mass * r2 * r2)
            out[tuple(sl)] = np.squeeze(np.broadcast_to(v, shape)[tuple(sl)])
        return out

    def factors(self, pos):
        """Angular coefficient x radial function pairs that sum to the potential:
        l1(l1+1) x 1/(2 m r1^2) and l2(l2+1) x 1/(2 m r2^2) on pairs of equal indices."""
        r1, r2 = pos[self.radial_rank1], pos[self.radial_rank2]
        lr = self._left_right()
        same = np.array([(a.L, a.M, a.l1, a.l2) == (b.L, b.M, b.l1, b.l2) for a, b in lr], dtype=bool)
        c1 = np.array([a.l1 * (a.l1 + 1.0) for a, _ in lr]) * same
        c2 = np.array([a.l2 * (a.l2 + 1.0) for a, _ in lr]) * same
        return [(1.0 / (2.0 * self.mass * r1 * r1), c1), (1.0 / (2.0 * self.mass * r2 * r2), c2)]


class CustomPotentialEvaluationR12(CoupledPotentialBase):
    """Electron-electron repulsion ``1/|r1 - r2|`` in the multipole expansion
    (coupledspherical.cpp:7-127): for each angular pair, sum over l3 of the angular factor
    times r<^l3 / r>^(l3+1)."""

    def GetPotentialValue(self, pos):
        from .spherical import r12_angular_factor, r12_multipoles
        r1, r2 = pos[self.radial_rank1], pos[self.radial_rank2]
        rmin, rmax = np.minimum(r1, r2), np.maximum(r1, r2)
        frac = rmin / rmax
        shape = np.broadcast(*pos).shape
        out = np.zeros(shape)
        for p, (left, right) in enumerate(self._left_right()):
            v = 0.0
            for l3 in r12_multipoles(left, right):
                c = r12_angular_factor(left, right, l3)
                if c != 0.0:
                    v = v + c * frac ** l3 / rmax
            if np.isscalar(v) and v == 0.0:
                continue
            sl = [slice(None)] * len(shape)
            sl[self.angular_rank] = p
            out[tuple(sl)] = np.squeeze(np.broadcast_to(v, shape)[tuple(sl)])
        return out

    def factors(self, pos):
        """One (radial function, angular coefficients) pair per multipole l3:
        r<^l3 / r>^(l3+1) and the coefficient of each angular pair (zero outside its l3 range)."""
        from .spherical import r12_angular_factor, r12_multipoles
        r1, r2 = pos[self.radial_rank1], pos[self.radial_rank2]
        rmin, rmax = np.minimum(r1, r2), np.maximum(r1, r2)
        frac = rmin / rmax
        lr = self._left_right()
        table = {}
        for p, (left, right) in enumerate(lr):
            for l3 in r12_multipoles(left, right):
                c = r12_angular_factor(left, right, l3)
                if c != 0.0:
                    table.setdefault(l3, np.zeros(len(lr)))[p] = c
        # even multipoles first, then odd: an angular pair's nonzero multipoles share a parity,
        # so each pair's factors are contiguous in this order
        return [(frac ** l3 / rmax, table[l3]) for l3 in sorted(table, key=lambda l: (l % 2, l))]


class CustomPotential_LaserLength(CoupledPotentialBase):
    """Length-gauge laser coupling of both electrons on ``SelectionRule_LinearPolarizedField``
    pairs, I1 r1 + I2 r2 (coupledlength.cpp:9-124); the field strength comes from the
    section's time function."""

    def GetPotentialValue(self, pos):
        from .spherical import laser_length_factors
        r1, r2 = pos[self.radial_rank1], pos[self.radial_rank2]
        shape = np.broadcast(*pos).shape
        out = np.zeros(shape)
        for p, (left, right) in enumerate(self._left_right()):
            I1, I2 = laser_length_factors(left, right)
            if I1 == 0.0 and I2 == 0.0:
                continue
            sl = [slice(None)] * len(shape)
            sl[self.angular_rank] = p
            out[tuple(sl)] = np.squeeze(np.broadcast_to(I1 * r1 + I2 * r2, shape)[tuple(sl)])
        return out

    def factors(self, pos):
        """(r1, I1) and (r2, I2) over the angular pairs."""
        from .spherical import laser_length_factors
        r1, r2 = pos[self.radial_rank1], pos[self.radial_rank2]
        II = np.array([laser_length_factors(left, right) for left, right in self._left_right()]).reshape(-1, 2)
        return [(r1 + 0.0 * r2, II[:, 0].copy()), (r2 + 0.0 * r1, II[:, 1].copy())]


for _cls in (CoupledSphericalCoulombPotential, CoupledSphericalKineticEnergyEvaluator, CustomPotentialEvaluationR12,
             CustomPotential_LaserLength, SingleIonizationBox, DoubleIonizationBox):
    POTENTIAL_CLASSES[_cls.__name__] = _cls
