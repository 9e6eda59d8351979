"""Full-length complex128 oracle runs of the hydrogen workloads -> tests/golden/run_*.npz.

    python tests/golden/make_oracle_runs.py [--jobs J] [name ...]

Each run builds the model on the host (the package's B-spline and potential setup, the same
code the GPU path uses), starts from the field-free ground state of the l = 0 channel and
advances it in complex128 twice: with the reference's own pAMP / GMRES templates driven as
PamPropagator / CayleyPropagator drive them (oracle/refkrylov.py over oracle/_ref, built from
the PyProp source tree by oracle/ref/build_ref.py; the stored ``psi``), and with the numpy
restatement of the oracle (``psi_oracle``). Test infrastructure only; the reference tree must
be on this machine ($PYPROP_REFERENCE or the recipe's default). The runs:

* ``run_cayley_l40.npz``: Crank-Nicolson steps (CayleyPropagator.py:71-150, GMRES(20) with
  the block-diagonal LU, tolerance 1e-12), hydrogen lmax 40, 600 B-splines on [0, 400], dt
  0.01 through the whole 50 a.u. 800 nm pulse of peak 0.05 a.u.: 5000 steps (about 5 minutes
  on one core).
* ``run_pamp_l10.npz``: pAMP steps (PamPropagator.py:50-75, pamp.h:613-670, double
  orthogonalization), hydrogen lmax 10, 150 B-splines on [0, 100], dt 0.01 through a 10 a.u.
  800 nm pulse of 0.05 a.u.: 1000 steps with a Krylov basis of 40 (``psi``), and the first
  ``SHORT`` steps with the workload's basis of 20 (``psi_m20``). With 20 vectors the step is
  not converged for this model (dt times the largest eigenvalue is about 21): the error
  estimate |c_m|^2 reaches 1e-8 per step, the state after 300 steps differs from the
  converged one by an infidelity of 2e-3, and a relative perturbation of 1e-15 of the initial
  state changes it by 1e-2 - in any implementation, so that run is compared only over the
  first steps; with 40 vectors the estimate stays below 1e-30 and the whole run is
  well-conditioned.
* ``run_members.npz``: ensemble members of ``hydrogen_ensemble_params(256)``: 1000
  Crank-Nicolson steps for ``CAYLEY_MEMBERS`` and the first ``SHORT`` pAMP steps (basis 20,
  stiffer still) for ``MEMBERS``.

Stored per run: the initial state ``psi0``, the final state ``psi`` (reference templates) and
``psi_oracle``, the S-norm and energy <H(t_end)> / <S> of ``psi`` (Problem.py:257-279), the
step count, and (Crank-Nicolson) the GMRES iterations summed over the run. Ensemble members
are stepped by the oracle restatement only. The GPU tests compare their final states with
``psi``.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

MEMBERS = (0, 32, 64, 96, 128, 160, 192, 224)
CAYLEY_MEMBERS = (0, 64, 128, 192)
SHORT = 10


def _problem(kw, propagator):
    import pyprop_gb300 as pp
    from pyprop_gb300.workloads import hydrogen
    return pp.Problem(pp.LoadString(hydrogen(propagator=propagator, precision="fp64", **kw)))


def _oracle(prob):
    from oracle.propagators import OracleHamiltonian
    repr_ = prob.psi.GetRepresentation()
    nang, N = repr_.GetFullShape()
    bp = prob.Propagator.BasePropagator
    terms = [("_".join(g.GetStorageId() for g in p.GeometryList), p.PotentialData, p.GeometryList[0].GetBasisPairs(),
              p.TimeFunction) for p in bp.PotentialList]
    return OracleHamiltonian(terms, repr_.overlap_rows, nang, N)


def run_one(kw, method, engine="oracle", nsteps=None):
    """Run of the workload ``kw`` (keywords of ``workloads.hydrogen``) with "cayley" or "pamp"
    steps by the oracle restatement ("oracle") or the reference's templates ("ref"), for
    nsteps steps (default: the whole pulse); returns the arrays stored in the fixture."""
    from oracle.propagators import OracleCayley, OraclePam
    from pyprop_gb300.workloads import field_free_ground_state, run_steps
    prob = _problem(kw, "CayleyPropagatorGPU" if method == "cayley" else "PamPropagatorGPU")
    ham = _oracle(prob)
    psi0, e0 = field_free_ground_state(prob)
    dt = kw["timestep"]
    nsteps = run_steps(kw) if nsteps is None else nsteps
    m = kw["krylov_basis_size"]
    if engine == "ref":
        from oracle import refkrylov
        from oracle.ref import build_ref
        from tests.helpers import oracle_terms
        build_ref.build(build_ref.reference_tree())
        rh = refkrylov.RefHamiltonian(oracle_terms(prob), ham.nang, ham.N, ham.kb)
        if method == "cayley":
            prec = OracleCayley(ham, dt, [0], m, kw["gmres_tolerance"]).prec
            prop = refkrylov.RefCayley(rh, ham.overlap, prec, m, kw["gmres_tolerance"])
        else:
            prop = refkrylov.RefPam(rh, ham.overlap, m, True)
    elif method == "cayley":
        prop = OracleCayley(ham, dt, [0], m, kw["gmres_tolerance"])
    else:
        prop = OraclePam(ham, m, True)
    psi = psi0.copy()
    iters = 0
    t0 = time.perf_counter()
    for n in range(nsteps):
        psi = prop.step(psi, n * dt, dt)
        if method == "cayley":
            iters += prop.last_iterations
    t_end = nsteps * dt
    return dict(psi0=psi0, psi=psi, e0=e0, norm=ham.norm(psi), energy=ham.energy(psi, t_end), steps=nsteps,
                dt=dt, iterations=iters, workload=json.dumps(kw), method=method,
                seconds=time.perf_counter() - t0)


def _job(args):
    name, kw, method, engine, nsteps = args
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    return name + ("_ref" if engine == "ref" else ""), run_one(kw, method, engine, nsteps)


def jobs(names):
    from pyprop_gb300.ensemble import hydrogen_ensemble_params
    from pyprop_gb300.workloads import ENSEMBLE_MEMBER, HYDROGEN_L10_PAMP, HYDROGEN_L40_CAYLEY
    out = []
    for engine in ("ref", "oracle"):
        if "cayley_l40" in names:
            out.append(("cayley_l40", HYDROGEN_L40_CAYLEY, "cayley", engine, None))
        if "pamp_l10" in names:
            out.append(("pamp_l10", dict(HYDROGEN_L10_PAMP, krylov_basis_size=40), "pamp", engine, None))
    if "pamp_l10" in names:
        out.append(("pamp_l10_m20", HYDROGEN_L10_PAMP, "pamp", "ref", SHORT))
    if "members" in names:
        params = hydrogen_ensemble_params(256)
        for i in MEMBERS:
            out.append(("pamp_member%d" % i, dict(ENSEMBLE_MEMBER, **params[i]), "pamp", "ref", SHORT))
        for i in CAYLEY_MEMBERS:
            out.append(("cayley_member%d" % i, dict(ENSEMBLE_MEMBER, **params[i]), "cayley", "ref", None))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=os.cpu_count() or 1)
    ap.add_argument("names", nargs="*", default=["cayley_l40", "pamp_l10", "members"])
    args = ap.parse_args()
    os.environ["OPENBLAS_NUM_THREADS"] = "1"  # children inherit it before numpy loads
    todo = sorted(jobs(args.names), key=lambda j: j[0] != "cayley_l40")
    with mp.get_context("spawn").Pool(min(args.jobs, len(todo))) as pool:
        results = dict(pool.map(_job, todo))
    for name in ("cayley_l40", "pamp_l10"):
        if name in results:
            r = dict(results[name + "_ref"])
            r["psi_oracle"] = results[name]["psi"]
            r["iterations_oracle"] = results[name]["iterations"]
            if name == "pamp_l10":
                r["psi_m20"] = results["pamp_l10_m20_ref"]["psi"]
                r["steps_m20"] = SHORT
            np.savez_compressed(os.path.join(HERE, "run_%s.npz" % name), **r)
            d = r["psi"] - r["psi_oracle"]
            print(name, "%.1f s" % r["seconds"], "norm %.15f energy %.12f" % (r["norm"], r["energy"]),
                  "ref vs oracle %.2e" % (np.linalg.norm(d) / np.linalg.norm(r["psi"])))
    if "members" in args.names:
        arrays = {}
        for i in MEMBERS:
            r = results["pamp_member%d_ref" % i]
            arrays.update({"pamp%d_psi0" % i: r["psi0"], "pamp%d_psi" % i: r["psi"], "pamp%d_norm" % i: r["norm"],
                           "pamp%d_energy" % i: r["energy"], "pamp%d_workload" % i: r["workload"]})
        for i in CAYLEY_MEMBERS:
            r = results["cayley_member%d_ref" % i]
            arrays.update({"cayley%d_psi" % i: r["psi"], "cayley%d_norm" % i: r["norm"],
                           "cayley%d_energy" % i: r["energy"], "cayley%d_iterations" % i: r["iterations"],
                           "cayley%d_workload" % i: r["workload"]})
        np.savez_compressed(os.path.join(HERE, "run_members.npz"), members=np.array(MEMBERS),
                            cayley_members=np.array(CAYLEY_MEMBERS), pamp_steps=SHORT, cayley_steps=1000, dt=0.01,
                            **arrays)
        print("members", max(results["cayley_member%d_ref" % i]["seconds"] for i in CAYLEY_MEMBERS), "s")


if __name__ == "__main__":
    main()
