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
    """1 - |<ref|psi>|^2 / (<ref|ref><psi|psi>), Euclidean or S-weighted (S per radial fibre),
    evaluated as ||psi - P_ref psi||^2 / ||psi||^2 (P_ref the projector on ref in the same
    metric), which keeps its accuracy far below the 1e-16 that 1 - |<ref|psi>|^2/(...) can
    resolve."""
    ref = np.asarray(ref)
    psi = np.asarray(psi)
    if S is None:
        ip = lambda x, y: np.vdot(x, y)
    else:
        ip = lambda x, y: np.vdot(x, y @ S.T)
    r = psi - ref * (ip(ref, psi) / ip(ref, ref).real)
    return float(ip(r, r).real / ip(psi, psi).real)


# ---------------------------------------------------------------------------------------
# random potentials in every storage of the generated multiply kernels
# ---------------------------------------------------------------------------------------
OUTER_KINDS = ("Simp", "Herm", "Diag", "Ident", "Band", "BandNH", "Dense")
INNER_KINDS = ("BandNH", "Band", "Dense", "Diag", "Ident")


def radial_extent(inner, N, kb):
    return {"BandNH": N * (2 * kb + 1), "Band": N * (kb + 1), "Dense": N * N, "Diag": N, "Ident": 1}[inner]


def random_storage_term(outer, inner, nang, N, kb, seed, outer_band=3):
    """(storage id, potential [e0][e1] complex128, pairs or None) with seeded random values."""
    rng = np.random.default_rng(seed)
    pairs = None
    if outer in ("Simp", "Herm"):
        pairs = np.array([(r, c) for r in range(nang) for c in range(nang) if abs(r - c) <= 1 and (r + c) % 3 != 2],
                         dtype=np.int32)
        e0 = len(pairs)
    elif outer == "Diag":
        e0 = nang
    elif outer == "Ident":
        e0 = 1
    elif outer == "Dense":
        e0 = nang * nang
    elif outer == "Band":
        e0 = nang * outer_band
    else:  # BandNH, odd band count
        e0 = nang * (2 * (outer_band // 2) + 1)
    e1 = radial_extent(inner, N, kb)
    pot = rng.standard_normal((e0, e1)) + 1j * rng.standard_normal((e0, e1))
    return "%s_%s" % (outer, inner), pot, pairs


class FakeGeometry:
    def __init__(self, storage_id, pairs=None):
        self.sid, self.pairs = storage_id, pairs

    def GetStorageId(self):
        return self.sid

    def GetBasisPairs(self):
        return self.pairs


class FakePotential:
    """The parts of a consolidated TensorPotential the device operator reads."""

    def __init__(self, storage, data, pairs, factor=1.0):
        """pairs: the angular pair list (rank 2) or a per-rank list of pair arrays."""
        kinds = storage.split("_")
        if not isinstance(pairs, (list, tuple)):
            pairs = [pairs] + [None] * (len(kinds) - 1)
        self.GeometryList = [FakeGeometry(k, pr) for k, pr in zip(kinds, pairs)]
        self.PotentialData = data
        self.factor = factor

    def GetTimeScaling(self, t):
        return self.factor


def helium_problem(lmax=1, nbsplines=16, rmax=15.0, **kw):
    import pyprop_gb300 as pp
    from pyprop_gb300.workloads import helium
    return pp.Problem(pp.LoadString(helium(lmax=lmax, nbsplines=nbsplines, rmax=rmax, **kw)))


def helium_dense(prob):
    """Dense H and S (x) S of a two-electron problem from the oracle's rank-3 storage loops."""
    from oracle.operators import Overlap, TermOracle, dense_operator
    bp = prob.Propagator.BasePropagator
    repr_ = prob.psi.GetRepresentation()
    shape = repr_.GetFullShape()
    terms = [TermOracle("_".join(g.GetStorageId() for g in pot.GeometryList), pot.PotentialData,
                        [g.GetBasisPairs() for g in pot.GeometryList], None, None, repr_.kb, shape=shape)
             for pot in bp.PotentialList]
    H = dense_operator(terms, [1.0] * len(terms), shape[0] * shape[1], shape[2])
    S = Overlap(repr_.overlap_rows).S
    return H, np.kron(np.eye(shape[0]), np.kron(S, S)), terms
