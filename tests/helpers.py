"""Shared builders for the tests: hydrogen problems and their oracle Hamiltonians."""
from __future__ import annotations

import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def hydrogen_problem(lmax=3, nbsplines=40, rmax=40.0, propagator="PamPropagatorGPU", precision="fp64", **kw):
    import pyprop_gb300 as pp
    from pyprop_gb300.workloads import hydrogen
    conf = pp.LoadString(hydrogen(lmax=lmax, nbsplines=nbsplines, rmax=rmax, propagator=propagator,
                                  precision=precision, **kw))
    return pp.Problem(conf)


def oracle_terms(prob):
    bp = prob.Propagator.BasePropagator
    return [("_".join(g.GetStorageId() for g in p.GeometryList), p.PotentialData,
             p.GeometryList[0].GetBasisPairs(), p.TimeFunction) for p in bp.PotentialList]


def oracle_hamiltonian(prob):
    from oracle.propagators import OracleHamiltonian
    repr_ = prob.psi.GetRepresentation()
    nang, N = repr_.GetFullShape()
    return OracleHamiltonian(oracle_terms(prob), repr_.overlap_rows, nang, N)


def golden(name):
    return np.load(os.path.join(GOLDEN, name))


def relerr(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def infidelity(ref, psi, S=None):
    """1 - |<ref|psi>|^2 / (<ref|ref><psi|psi>), Euclidean or S-weighted (S per radial fibre)."""
    ref = np.asarray(ref)
    psi = np.asarray(psi)
    if S is None:
        ip = np.vdot(ref, psi)
        n1, n2 = np.vdot(ref, ref).real, np.vdot(psi, psi).real
    else:
        Sp = psi @ S.T
        Sr = ref @ S.T
        ip = np.vdot(ref, Sp)
        n1, n2 = np.vdot(ref, Sr).real, np.vdot(psi, Sp).real
    return float(1.0 - abs(ip) ** 2 / (n1 * n2))
