"""Ensemble stepping (one graph launch for many members) against members stepped alone."""
import numpy as np
import pytest

from tests.helpers import hydrogen_problem, oracle_hamiltonian, relerr

pytestmark = pytest.mark.gpu


def _members(precision, fused=True):
    specs = [dict(lmax=3, nbsplines=40, rmax=40.0, amplitude=0.05),
             dict(lmax=5, nbsplines=33, rmax=30.0, amplitude=0.08, wavelength_nm=400.0),
             dict(lmax=2, nbsplines=55, rmax=50.0, amplitude=0.02, wavelength_nm=1600.0)]
    probs = []
    for k, sp in enumerate(specs):
        p = hydrogen_problem(propagator="CayleyPropagatorGPU", precision=precision, gmres_tolerance=1e-12, **sp)
        p.Propagator.FusedStep = fused
        p.SetupStep(skipWavefunctionSetup=True)
        rng = np.random.default_rng(100 + k)
        shape = p.psi.GetRepresentation().GetFullShape()
        psi = rng.normal(size=shape) + 1j * rng.normal(size=shape)
        p.psi.SetData(psi / np.linalg.norm(psi))
        p.PropagatedTime = 1.0
        probs.append(p)
    return probs


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_ensemble_matches_single_members(gpu, precision):
    from pyprop_gb300.ensemble import CayleyEnsembleGPU
    # the ensemble graph runs the multi-kernel step of every member: members stepped alone on
    # that step agree to rounding; mixed-precision members on the single-kernel step agree
    # to the GMRES tolerance
    alone = _members(precision, fused=False)
    alone_fused = _members(precision) if precision == "fp32" else []
    together = _members(precision)
    for _ in range(3):
        for p in alone + alone_fused:
            p.AdvanceStep()
    ens = CayleyEnsembleGPU(together)
    for _ in range(3):
        ens.AdvanceStep()
    stats = ens.Stats()
    for a, b, st in zip(alone, together, stats):
        assert relerr(b.psi.numpy(), a.psi.numpy()) < 1e-13
        assert st["Iterations"] >= 1
        assert abs(a.PropagatedTime - b.PropagatedTime) < 1e-12
    for a, b in zip(alone_fused, together):
        assert a.Propagator.Fused
        assert relerr(b.psi.numpy(), a.psi.numpy()) < 1e-10


def test_ensemble_member_against_oracle(gpu):
    from pyprop_gb300.ensemble import CayleyEnsembleGPU
    from oracle.propagators import OracleCayley
    together = _members("fp64")
    psi0 = [p.psi.numpy() for p in together]
    ens = CayleyEnsembleGPU(together)
    for _ in range(2):
        ens.AdvanceStep()
    for p, start in zip(together, psi0):
        ham = oracle_hamiltonian(p)
        cay = OracleCayley(ham, 0.01, [0], 20, 1e-13)
        ref = cay.step(cay.step(start, 1.0, 0.01), 1.01, 0.01)
        assert relerr(p.psi.numpy(), ref) < 1e-10


def _pamp_members(precision, with_field=True):
    specs = [dict(lmax=3, nbsplines=40, rmax=40.0, amplitude=0.05 if with_field else 0.0),
             dict(lmax=5, nbsplines=33, rmax=30.0, amplitude=0.08 if with_field else 0.0, wavelength_nm=400.0),
             dict(lmax=2, nbsplines=55, rmax=50.0, amplitude=0.02 if with_field else 0.0, wavelength_nm=1600.0)]
    probs = []
    for k, sp in enumerate(specs):
        p = hydrogen_problem(propagator="PamPropagatorGPU", precision=precision, **sp)
        p.SetupStep(skipWavefunctionSetup=True)
        rng = np.random.default_rng(200 + k)
        shape = p.psi.GetRepresentation().GetFullShape()
        psi = rng.normal(size=shape) + 1j * rng.normal(size=shape)
        p.psi.SetData(psi / np.linalg.norm(psi))
        p.PropagatedTime = 1.0
        probs.append(p)
    return probs


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_pamp_ensemble_matches_single_members(gpu, precision):
    """pAMP members of different sizes and fields advanced by one launch per step (the m x m
    exponentials on the device, Pade of order 6) against the same members stepped alone
    (complex128: the graphs with the host exponential; complex64: the single-kernel step), and a
    second batch built on the same members after the first is destroyed."""
    from pyprop_gb300.ensemble import PamEnsembleGPU
    alone = _pamp_members(precision)
    together = _pamp_members(precision)
    exact = _pamp_members("fp64") if precision == "fp32" else []
    for _ in range(4):
        for p in alone + exact:
            p.AdvanceStep()
    ens = PamEnsembleGPU(together)
    for _ in range(4):
        ens.AdvanceStep()
    stats = ens.Stats()
    tol = 1e-11 if precision == "fp64" else 1e-6
    for k, (a, b, st) in enumerate(zip(alone, together, stats)):
        if precision == "fp64":
            assert relerr(b.psi.numpy(), a.psi.numpy()) < tol, relerr(b.psi.numpy(), a.psi.numpy())
        else:
            # complex64 bases (the ensemble's step; the lone member's single-kernel step, whose
            # Krylov vectors are U^-1 V in complex64): both within the FP32 Krylov error of the
            # complex128-basis result, which dt ||H_m|| scales
            e_lone = relerr(a.psi.numpy(), exact[k].psi.numpy())
            e_ens = relerr(b.psi.numpy(), exact[k].psi.numpy())
            assert e_lone < 5e-5 and e_ens < 5 * e_lone + 1e-7, (e_ens, e_lone)
        assert st["Iterations"] == 20
        assert 0.0 <= st["ErrorEstimate"] < 1e-6
        assert abs(a.PropagatedTime - b.PropagatedTime) < 1e-12
    del ens
    # members step alone again (their own slots back) and agree with the lone copies (complex64:
    # to the difference the two paths' rounding left after the ensemble steps)
    for p, q in zip(alone, together):
        before = relerr(q.psi.numpy(), p.psi.numpy())
        p.AdvanceStep()
        q.AdvanceStep()
        assert relerr(q.psi.numpy(), p.psi.numpy()) < (tol if precision == "fp64" else 2 * before + 1e-6)


def _pamp_members_kw(precision, specs, seed):
    probs = []
    for k, sp in enumerate(specs):
        p = hydrogen_problem(propagator="PamPropagatorGPU", precision=precision, **sp)
        p.SetupStep(skipWavefunctionSetup=True)
        rng = np.random.default_rng(seed + k)
        shape = p.psi.GetRepresentation().GetFullShape()
        psi = rng.normal(size=shape) + 1j * rng.normal(size=shape)
        p.psi.SetData(psi / np.linalg.norm(psi))
        p.PropagatedTime = 1.0
        probs.append(p)
    return probs


@pytest.mark.parametrize("order", [7, 5])
def test_pamp_persistent_step_matches_graph_and_single_members(gpu, order):
    """The persistent ensemble step (one CTA per member from a device work list, the whole pAMP
    step in one launch; order 7: the kernel instance unrolled for 13-diagonal bands, order 5:
    the generic one) against the graph of per-member kernels and the members stepped alone:
    complex64 bases agree to the FP32 rounding of the Krylov vectors, the Hessenberg statistics
    match, and the launch shape was autotuned. Both complex64 paths are judged against the same
    members on a complex128 basis (their own rounding differs: substitutions here, block
    inverses there)."""
    from pyprop_gb300.ensemble import PamEnsembleGPU
    specs = [dict(lmax=3, nbsplines=40, rmax=40.0, amplitude=0.05, order=order),
             dict(lmax=5, nbsplines=33, rmax=30.0, amplitude=0.08, wavelength_nm=400.0, order=order),
             dict(lmax=2, nbsplines=55, rmax=50.0, amplitude=0.02, wavelength_nm=1600.0, order=order),
             dict(lmax=8, nbsplines=36, rmax=36.0, amplitude=0.1, wavelength_nm=600.0, order=order)]
    alone = _pamp_members_kw("fp32", specs, 300)
    graph = _pamp_members_kw("fp32", specs, 300)
    pers = _pamp_members_kw("fp32", specs, 300)
    exact = _pamp_members_kw("fp64", specs, 300)
    eg = PamEnsembleGPU(graph)
    eg.set_persistent(False)
    ep = PamEnsembleGPU(pers)
    ep.set_persistent(True)
    for _ in range(5):
        for p in alone + exact:
            p.AdvanceStep()
        eg.AdvanceStep()
        ep.AdvanceStep()
    shape = ep.launch_shape()
    assert shape["persistent"] and shape["threads"] >= 128 and shape["ctas"] >= 1 and shape["persistent_ms"] > 0.0
    assert not eg.launch_shape()["persistent"]
    for a, g, q, x, sg, sq in zip(alone, graph, pers, exact, eg.Stats(), ep.Stats()):
        e_graph = relerr(g.psi.numpy(), x.psi.numpy())
        e_pers = relerr(q.psi.numpy(), x.psi.numpy())
        assert e_graph < 1e-4 and e_pers < 5 * e_graph + 1e-7, (e_pers, e_graph)
        assert relerr(q.psi.numpy(), a.psi.numpy()) < 3 * (e_graph + e_pers)
        assert sq["Iterations"] == sg["Iterations"] == 20
        assert 0.0 <= sq["ErrorEstimate"] < 1e-4
        assert abs(np.log10(max(sq["ErrorEstimate"], 1e-300)) - np.log10(max(sg["ErrorEstimate"], 1e-300))) < 1.0
        assert abs(q.PropagatedTime - a.PropagatedTime) < 1e-12


def test_pamp_persistent_step_norm_and_fp64_members(gpu):
    """Field-free members keep their norm under the persistent step (the exponential of a
    Hermitian Hessenberg), and an ensemble with a complex128 basis stays on the graph (the
    persistent kernel takes complex64 bases only)."""
    from pyprop_gb300.ensemble import PamEnsembleGPU
    specs = [dict(lmax=4, nbsplines=45, rmax=40.0, amplitude=0.0), dict(lmax=7, nbsplines=30, rmax=30.0, amplitude=0.0)]
    pers = _pamp_members_kw("fp32", specs, 400)
    ep = PamEnsembleGPU(pers)
    ep.set_persistent(True)
    n0 = [p.psi.GetNorm() for p in pers]
    for _ in range(20):
        ep.AdvanceStep()
    assert ep.launch_shape()["persistent"]
    for p, a in zip(pers, n0):
        assert abs(p.psi.GetNorm() - a) < 1e-6
    e64 = PamEnsembleGPU(_pamp_members_kw("fp64", specs, 400))
    assert not e64.launch_shape()["persistent"]
    with pytest.raises(RuntimeError):
        e64.set_persistent(True)


def test_pamp_batch_automatic_choice(gpu):
    """By default the first ensemble step times the persistent kernel and the graph on the
    members themselves (restoring their wavefunctions after each trial) and keeps the faster;
    the step it runs continues from the unchanged start."""
    from pyprop_gb300.ensemble import PamEnsembleGPU
    specs = [dict(lmax=3, nbsplines=40, rmax=40.0, amplitude=0.05), dict(lmax=6, nbsplines=50, rmax=40.0, amplitude=0.05)]
    auto = _pamp_members_kw("fp32", specs, 500)
    ref = _pamp_members_kw("fp32", specs, 500)
    ea = PamEnsembleGPU(auto)
    er = PamEnsembleGPU(ref)
    er.set_persistent(False)
    for _ in range(3):
        ea.AdvanceStep()
        er.AdvanceStep()
    shape = ea.launch_shape()
    assert shape["persistent_ms"] > 0.0 and shape["graph_ms"] > 0.0
    assert shape["persistent"] == (shape["persistent_ms"] <= shape["graph_ms"])
    for a, r in zip(auto, ref):
        assert relerr(a.psi.numpy(), r.psi.numpy()) < 1e-4
