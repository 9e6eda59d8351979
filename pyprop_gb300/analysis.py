"""Analysis of final two-electron states: populations of products of single-electron states.

The functions follow examples/tensor/helium_stabilization/analysis.cpp (the projections, on
the GPU through ``pg_radial_products_project`` / ``pg_radial_products_remove``) and
analysis.py (their drivers) of the reference:

* ``CalculateProjectionRadialProductStates(l1, V1, l2, V2, psiData, angularIndices)``:
  <V1_i(1) V2_j(2) | psi> for the angular indices of one (l1, l2) pair (analysis.cpp:39-81);
* ``RemoveProjectionRadialProductStates(...)`` (analysis.cpp:91-121);
* ``CalculatePopulationRadialProductStates(...)``: (i1, i2, |proj|^2 summed over the angular
  indices) (analysis.cpp:133-152);
* ``GetPopulationProductStates`` / ``RemoveProductStatesProjection`` over every (l1, l2) of
  lists of radial states per l (analysis.py:694-782);
* ``SetupRadialEigenstates``: single-electron radial eigenstates per l of -1/2 d^2/dr^2 +
  l(l+1)/2r^2 - Z/r in the B-spline basis (the reference computes them the same way in its
  helium examples), and ``GetFilteredSingleParticleStates`` selecting them by energy;
* ``ProductStateIonization``: bound, single- and double-ionization populations of a
  state, as analysis.py:391-462 reports them.

``psiData`` is the wavefunction with the integration weights applied (the overlap on both
radial ranks): ``MultiplyIntegrationWeights`` of the representation, as the reference's
callers do before projecting.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as nat
from .gpu import Context, check, ptr


def _states(V):
    V = np.ascontiguousarray(np.asarray(V, dtype=np.complex128))
    if V.ndim != 2:
        raise ValueError("radial states must be a 2-D array [N][nstates]")
    return V


def _indices(angularIndices):
    return np.ascontiguousarray(np.asarray(angularIndices, dtype=np.int32).ravel())


def CalculateProjectionRadialProductStates(l1, V1, l2, V2, psiData, angularIndices):
    """proj[q][i1][i2] = sum_{r1,r2} conj(V1[r1][i1]) psiData[a_q][r1][r2] conj(V2[r2][i2]),
    complex128 [len(angularIndices)][n1][n2] (host). psiData: [Nang][N][N] device tensor."""
    V1, V2 = _states(V1), _states(V2)
    idx = _indices(angularIndices)
    nang, N1, N2 = psiData.shape
    if V1.shape[0] != N1 or V2.shape[0] != N2:
        raise ValueError("radial states do not match the wavefunction's radial size")
    ctx = Context.get()
    out = np.zeros((len(idx), V1.shape[1], V2.shape[1]), dtype=np.complex128)
    _, ip = nat.iptr(idx)
    check(ctx.lib.pg_radial_products_project(ctx.h, ptr(psiData), nang, N1, N2, ip, len(idx),
                                             V1.view(np.float64).ctypes.data_as(nat._DP), V1.shape[1],
                                             V2.view(np.float64).ctypes.data_as(nat._DP), V2.shape[1],
                                             out.view(np.float64).ctypes.data_as(nat._DP)),
          "pg_radial_products_project")
    return out


def RemoveProjectionRadialProductStates(l1, V1, l2, V2, psiData, angularIndices, outputPsi):
    """outputPsi[a_q] -= V1 proj_q V2^T with proj from psiData (both [Nang][N][N] device
    tensors; outputPsi without the integration weights)."""
    V1, V2 = _states(V1), _states(V2)
    idx = _indices(angularIndices)
    if len(set(idx.tolist())) != len(idx):
        raise ValueError("angular indices must be distinct")
    nang, N1, N2 = psiData.shape
    ctx = Context.get()
    _, ip = nat.iptr(idx)
    check(ctx.lib.pg_radial_products_remove(ctx.h, ptr(psiData), ptr(outputPsi), nang, N1, N2, ip, len(idx),
                                            V1.view(np.float64).ctypes.data_as(nat._DP), V1.shape[1],
                                            V2.view(np.float64).ctypes.data_as(nat._DP), V2.shape[1]),
          "pg_radial_products_remove")


def CalculatePopulationRadialProductStates(l1, V1, l2, V2, psiData, angularIndices):
    """[(i1, i2, pop)]: |proj|^2 summed over the angular indices for every state pair."""
    proj = CalculateProjectionRadialProductStates(l1, V1, l2, V2, psiData, angularIndices)
    pop = np.sum(np.abs(proj) ** 2, axis=0)
    return [(i1, i2, float(pop[i1, i2])) for i1 in range(pop.shape[0]) for i2 in range(pop.shape[1])]


def GetLocalCoupledSphericalHarmonicIndices(psi, coupledIndexFilter):
    """Angular indices of psi's coupled basis whose CoupledIndex passes the filter
    (analysis.py:35-62)."""
    basis = psi.GetRepresentation().GetRepresentation(0)
    return [i for i, c in enumerate(basis.indices) if coupledIndexFilter(c)]


def _weighted(psi):
    tmp = psi.Copy()
    psi.GetRepresentation().MultiplyIntegrationWeights(tmp)
    return tmp


def GetPopulationProductStates(psi, singleStates1, singleStates2):
    """[(l1, l2, [(i1, i2, pop)])] over every (l1, l2) with states on both sides and coupled
    indices in psi (analysis.py:694-739)."""
    data = _weighted(psi).GetData()
    population = []
    for l1, V1 in enumerate(singleStates1):
        if np.asarray(V1).size == 0:
            continue
        for l2, V2 in enumerate(singleStates2):
            if np.asarray(V2).size == 0:
                continue
            idx = GetLocalCoupledSphericalHarmonicIndices(psi, lambda c: c.l1 == l1 and c.l2 == l2)
            if not idx:
                continue
            population.append((l1, l2, CalculatePopulationRadialProductStates(l1, V1, l2, V2, data, idx)))
    return population


def RemoveProductStatesProjection(psi, singleStates1, singleStates2):
    """psi <- (1 - sum_ij |i(1) j(2)><i(1) j(2)|) psi over every (l1, l2) (analysis.py:742-781)."""
    data = _weighted(psi).GetData()
    for l1, V1 in enumerate(singleStates1):
        if np.asarray(V1).size == 0:
            continue
        for l2, V2 in enumerate(singleStates2):
            if np.asarray(V2).size == 0:
                continue
            idx = GetLocalCoupledSphericalHarmonicIndices(psi, lambda c: c.l1 == l1 and c.l2 == l2)
            if idx:
                RemoveProjectionRadialProductStates(l1, V1, l2, V2, data, idx, psi.GetData())


def SetupRadialEigenstates(bspline, Z, lmax, mass=1.0):
    """(energies, states) per l <= lmax: the generalized eigenpairs of the radial Hamiltonian
    -1/(2 mass) d^2/dr^2 + l(l+1)/(2 mass r^2) - Z/r against the overlap in the B-spline basis
    ``bspline`` (host, setup only); states are columns [N][N] with unit S-norm."""
    import scipy.linalg as sl
    r = bspline.grid
    S = bspline.dense(bspline.overlap_band())
    T = bspline.dense(bspline.band_elements(np.full_like(r, -1.0 / (2.0 * mass)), 2))
    V = bspline.dense(bspline.band_elements(-Z / r, 0))
    C2 = bspline.dense(bspline.band_elements(1.0 / (2.0 * mass * r * r), 0))
    energies, states = [], []
    for l in range(lmax + 1):
        H = T + V + l * (l + 1) * C2
        H = 0.5 * (H + H.T)
        w, v = sl.eigh(H, S)
        energies.append(w)
        states.append(v.astype(np.complex128))
    return energies, states


def GetFilteredSingleParticleStates(energies, states, energyFilter):
    """The states (and energies) per l whose energy passes the filter (analysis.py:598-615)."""
    E, V = [], []
    for w, v in zip(energies, states):
        keep = np.array([bool(energyFilter(e)) for e in w], dtype=bool)
        E.append(w[keep])
        V.append(v[:, keep])
    return E, V


def ProductStateIonization(psi, Z, lmax, maxE=None):
    """Populations of psi in products of single-electron (charge Z) radial states
    (analysis.py:391-462): {"norm", "bound" (both electrons bound), "single" (one bound, one
    in the continuum, either way round), "double" (both in the continuum, energies below
    maxE when given)}."""
    bs = psi.GetRepresentation().GetRepresentation(1).BSplineObject
    energies, states = SetupRadialEigenstates(bs, Z, lmax)
    bound = GetFilteredSingleParticleStates(energies, states, lambda e: e <= 0.0)[1]
    cont = GetFilteredSingleParticleStates(energies, states,
                                           (lambda e: 0.0 < e) if maxE is None else (lambda e: 0.0 < e <= maxE))[1]

    def total(pop):
        return float(sum(p for _, _, lst in pop for _, _, p in lst))

    return {"norm": psi.GetNorm() ** 2,
            "bound": total(GetPopulationProductStates(psi, bound, bound)),
            "single": total(GetPopulationProductStates(psi, bound, cont)) +
            total(GetPopulationProductStates(psi, cont, bound)),
            "double": total(GetPopulationProductStates(psi, cont, cont))}
