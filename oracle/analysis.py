"""Oracle of the two-electron analysis - test infrastructure only.

Loop restatements of examples/tensor/helium_stabilization/analysis.cpp:
  * ``projection``  CalculateProjectionRadialProductStates (:39-81): for each angular index,
    tempProj = psi_a conj(V2) row by row, then proj = V1^H tempProj;
  * ``remove``      RemoveProjectionRadialProductStates (:91-121): psi_a -= sum proj V1 V2;
  * ``population``  CalculatePopulationRadialProductStates (:133-152).
psiData carries the integration weights (the overlap on both radial ranks)."""
from __future__ import annotations

import numpy as np


def projection(V1, V2, psiData, angularIndices):
    V1 = np.asarray(V1, dtype=np.complex128)
    V2 = np.asarray(V2, dtype=np.complex128)
    rcount, count1 = V1.shape
    count2 = V2.shape[1]
    proj = np.zeros((len(angularIndices), count1, count2), dtype=np.complex128)
    for i0, a in enumerate(angularIndices):
        psi = psiData[a]
        temp = np.zeros((rcount, count2), dtype=np.complex128)
        for r1 in range(rcount):
            for r2 in range(V2.shape[0]):
                temp[r1, :] += np.conj(V2[r2, :]) * psi[r1, r2]
        for r1 in range(rcount):
            proj[i0] += np.conj(V1[r1, :])[:, None] * temp[r1, None, :]
    return proj


def remove(V1, V2, psiData, angularIndices, outputPsi):
    proj = projection(V1, V2, psiData, angularIndices)
    V1 = np.asarray(V1, dtype=np.complex128)
    V2 = np.asarray(V2, dtype=np.complex128)
    for i0, a in enumerate(angularIndices):
        outputPsi[a] -= np.einsum("ij,ri,sj->rs", proj[i0], V1, V2)
    return outputPsi


def population(V1, V2, psiData, angularIndices):
    proj = projection(V1, V2, psiData, angularIndices)
    pop = np.sum(np.abs(proj) ** 2, axis=0)
    return [(i1, i2, float(pop[i1, i2])) for i1 in range(pop.shape[0]) for i2 in range(pop.shape[1])]
