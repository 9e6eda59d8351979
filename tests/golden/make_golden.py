"""Regenerate the golden fixtures under tests/golden/.

    python tests/golden/make_golden.py /path/to/reference

* qdot_piram.npz - the reference's own pIRAM test input (core/krylov/piram/piram/
  qdotmatrix.dat: "row col re im" lines, only the real part is used, piramtest.cpp:34-68;
  init.dat: the start vector, :103-140) and the five eigenvalues with the smallest real
  parts from a dense eigen-decomposition of that matrix. piramtest.cpp runs pIRAM with
  BasisSize 50, EigenvalueCount 5, MaxRestartCount 10, Tolerance 0 (:153-182).
* hydrogen_small.npz - oracle outputs on a small hydrogen problem (lmax 3, 40 B-splines,
  r in [0, 40]) with the field on: a seeded wavefunction, H(t) psi, one pAMP step and one
  Cayley step. They pin the oracle (CPU tests recompute them) and are the GPU tests'
  reference values.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def make_qdot(reference):
    base = os.path.join(reference, "core", "krylov", "piram", "piram")
    rows, cols, vals = [], [], []
    with open(os.path.join(base, "qdotmatrix.dat")) as fh:
        for line in fh:
            parts = line.split()
            if len(parts) < 3:
                continue
            rows.append(int(parts[0]))
            cols.append(int(parts[1]))
            vals.append(float(parts[2]))
    init = np.loadtxt(os.path.join(base, "init.dat"))
    rows = np.asarray(rows, dtype=np.int16)
    cols = np.asarray(cols, dtype=np.int16)
    vals = np.asarray(vals, dtype=np.float64)
    n = int(rows.max()) + 1
    A = np.zeros((n, n))
    np.add.at(A, (rows.astype(int), cols.astype(int)), vals)
    ev = np.linalg.eigvals(A)
    ev = ev[np.argsort(ev.real)][:5]
    np.savez_compressed(os.path.join(HERE, "qdot_piram.npz"), rows=rows, cols=cols, vals=vals, init=init,
                        lowest5=ev)
    return n, ev


def hydrogen_small_terms():
    import pyprop_gb300 as pp
    from pyprop_gb300.workloads import hydrogen
    conf = pp.LoadString(hydrogen(lmax=3, nbsplines=40, rmax=40.0, amplitude=0.05, pulse_duration=10.0))
    prob = pp.Problem(conf)
    bp = prob.Propagator.BasePropagator
    repr_ = prob.psi.GetRepresentation()
    terms = [("_".join(g.GetStorageId() for g in p.GeometryList), p.PotentialData,
              p.GeometryList[0].GetBasisPairs(), p.TimeFunction) for p in bp.PotentialList]
    return prob, repr_, terms


def make_hydrogen():
    from oracle.propagators import OracleCayley, OracleHamiltonian, OraclePam
    prob, repr_, terms = hydrogen_small_terms()
    nang, N = repr_.GetFullShape()
    ham = OracleHamiltonian(terms, repr_.overlap_rows, nang, N)
    rng = np.random.default_rng(20261203)
    psi = rng.normal(size=(nang, N)) + 1j * rng.normal(size=(nang, N))
    psi /= ham.norm(psi)
    t, dt = 2.5, 0.01
    Hpsi = ham.apply_H(psi, t)
    pam = OraclePam(ham, 20, double_ortho=True).step(psi, t, dt)
    cay = OracleCayley(ham, dt, [0], 20, 1e-13).step(psi, t, dt)
    np.savez_compressed(os.path.join(HERE, "hydrogen_small.npz"), psi=psi, t=t, dt=dt, Hpsi=Hpsi, pamp=pam,
                        cayley=cay, scalings=np.array(ham.scalings(t)))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py /path/to/reference  (the PyProp source tree)")
    reference = sys.argv[1]
    n, ev = make_qdot(reference)
    print("qdot", n, ev)
    make_hydrogen()
    print("hydrogen_small written")
