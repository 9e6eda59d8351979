"""GPU parity of the Krylov propagators and solvers against the oracle."""
import numpy as np
import pytest

from pyprop_gb300 import _native as nat
from tests.helpers import golden, hydrogen_problem, infidelity, oracle_hamiltonian, relerr

pytestmark = pytest.mark.gpu


def _torch():
    import torch
    return torch


def _set_psi(prob, psi):
    t = _torch()
    prob.psi.GetData().copy_(t.as_tensor(psi, device="cuda"))


def test_pamp_step_fp64_matches_golden(gpu):
    g = golden("hydrogen_small.npz")
    prob = hydrogen_problem(propagator="PamPropagatorGPU", precision="fp64")
    prob.SetupStep(skipWavefunctionSetup=True)
    _set_psi(prob, g["psi"])
    prob.Propagator.AdvanceStep(float(g["t"]), float(g["dt"]))
    out = prob.psi.numpy()
    assert relerr(out, g["pamp"]) < 1e-12
    st = prob.Propagator.LastStats
    assert st.OpCount == 20 and st.ErrorEstimate < 1e-20


def test_pamp_steps_against_oracle_fp64_and_fp32(gpu):
    from oracle.propagators import OraclePam
    g = golden("hydrogen_small.npz")
    ref = hydrogen_problem()
    ham = oracle_hamiltonian(ref)
    pam = OraclePam(ham, 20, True)
    psi_ref = g["psi"].copy()
    t0, dt, nsteps = 1.0, 0.01, 10
    for n in range(nsteps):
        psi_ref = pam.step(psi_ref, t0 + n * dt, dt)
    S = ham.overlap.S
    for prec, tol_rel, tol_inf in [("fp64", 1e-11, 1e-14), ("fp32", 5e-5, 1e-9)]:
        prob = hydrogen_problem(propagator="PamPropagatorGPU", precision=prec)
        prob.SetupStep(skipWavefunctionSetup=True)
        _set_psi(prob, g["psi"])
        for n in range(nsteps):
            prob.Propagator.AdvanceStep(t0 + n * dt, dt)
        out = prob.psi.numpy()
        assert relerr(out, psi_ref) < tol_rel, prec
        assert infidelity(psi_ref, out, S) < tol_inf, prec
        assert abs(ham.norm(out) - ham.norm(psi_ref)) < 10 * tol_rel


def test_pamp_device_exponential_matches_host_exponential(gpu):
    """The step with the m x m exponential on the device (one graph, no wait) against the step
    that computes it on the host between two graphs: same states, same statistics, read on
    demand after steps that did not wait."""
    g = golden("hydrogen_small.npz")
    t0, dt, nsteps = 1.0, 0.01, 10
    outs, stats = {}, {}
    for dev in (True, False):
        prob = hydrogen_problem(propagator="PamPropagatorGPU", precision="fp64")
        prob.SetupStep(skipWavefunctionSetup=True)
        prob.Propagator.stepper.set_device_exp(dev)
        prob.Propagator.StepStats = False
        _set_psi(prob, g["psi"])
        for n in range(nsteps):
            prob.Propagator.AdvanceStep(t0 + n * dt, dt)
        st = prob.Propagator.LastStats
        stats[dev] = (st.OpCount, st.Iterations, st.ErrorEstimate)
        outs[dev] = prob.psi.numpy()
    # the host takes the Hermitian tridiagonal H_m by implicit QL, the device the scaled Pade:
    # both within rounding of the exact exponential
    assert relerr(outs[True], outs[False]) < 1e-11
    assert stats[True][:2] == stats[False][:2] == (20 * nsteps, 20)
    assert stats[True][2] < 1e-20 and stats[False][2] < 1e-20
    # a basis above the device exponential's limit keeps the host path
    big = hydrogen_problem(propagator="PamPropagatorGPU", precision="fp64", krylov_basis_size=60)
    big.SetupStep(skipWavefunctionSetup=True)
    with pytest.raises(nat.PygpuError):
        big.Propagator.stepper.set_device_exp(True)


def test_pamp_single_kernel_step_matches_graphs_and_oracle(gpu):
    """The single-kernel complex64-basis pAMP step (Arnoldi on T_j = U^-1 V_j, the exponential
    in every CTA, one launch per step) against the oracle's complex128 steps and against the
    captured graphs with the same complex64 basis, over 10 steps enqueued without waiting."""
    from oracle.propagators import OraclePam
    g = golden("hydrogen_small.npz")
    ref = hydrogen_problem()
    ham = oracle_hamiltonian(ref)
    pam = OraclePam(ham, 20, True)
    psi_ref = g["psi"].copy()
    t0, dt, nsteps = 1.0, 0.01, 10
    for n in range(nsteps):
        psi_ref = pam.step(psi_ref, t0 + n * dt, dt)
    S = ham.overlap.S
    outs = {}
    for fused in (True, False):
        prob = hydrogen_problem(propagator="PamPropagatorGPU", precision="fp32")
        prob.SetupStep(skipWavefunctionSetup=True)
        assert prob.Propagator.Fused
        if not fused:
            assert not prob.Propagator.stepper.set_fused(False)
        prob.Propagator.StepStats = False
        ctx = prob.Propagator.op64.ctx
        _set_psi(prob, g["psi"])
        l0 = ctx.launches()
        for n in range(nsteps):
            prob.Propagator.AdvanceStep(t0 + n * dt, dt)
        st = prob.Propagator.LastStats
        assert st.Iterations == 20 and 0.0 <= st.ErrorEstimate < 1e-10
        if fused:
            assert ctx.launches() - l0 == nsteps
        outs[fused] = prob.psi.numpy()
    for fused, out in outs.items():
        assert relerr(out, psi_ref) < 5e-5, fused
        assert infidelity(psi_ref, out, S) < 1e-9, fused
        assert abs(ham.norm(out) - ham.norm(psi_ref)) < 5e-6, fused
    assert relerr(outs[True], outs[False]) < 5e-5


@pytest.mark.parametrize("kw", [dict(lmax=3, nbsplines=40, rmax=40.0, order=5),
                                dict(lmax=3, nbsplines=300, rmax=150.0),
                                dict(lmax=5, nbsplines=600, rmax=300.0)])
def test_pamp_single_kernel_step_other_layouts(gpu, kw):
    """The single-kernel pAMP step on the generic band-width instance (B-splines of order 5, the
    dense S^-1 of a short fibre), with the blocked solve's factors in shared memory (300
    B-splines) and read through L2 (600 B-splines), against the graphs with the same complex64
    basis and the complex128-basis step: both complex64 paths within the FP32 Krylov error of
    the complex128 result."""
    t0, dt, nsteps = 1.0, 0.01, 5
    rng = np.random.default_rng(7)
    out = {}
    psi0 = None
    for name, prec, fused in (("fused", "fp32", True), ("graphs", "fp32", False), ("exact", "fp64", False)):
        prob = hydrogen_problem(propagator="PamPropagatorGPU", precision=prec, amplitude=0.05, **kw)
        prob.SetupStep(skipWavefunctionSetup=True)
        if prec == "fp32":
            assert prob.Propagator.stepper.set_fused(fused) == fused
        if psi0 is None:
            shape = prob.psi.GetRepresentation().GetFullShape()
            psi0 = rng.normal(size=shape) + 1j * rng.normal(size=shape)
            psi0 *= np.exp(-np.arange(shape[1]) * (10.0 / shape[1]))[None, :]  # weight on the inner splines
            psi0 /= np.linalg.norm(psi0)
        _set_psi(prob, psi0)
        for n in range(nsteps):
            prob.Propagator.AdvanceStep(t0 + n * dt, dt)
        out[name] = prob.psi.numpy()
    e_graph = relerr(out["graphs"], out["exact"])
    e_fused = relerr(out["fused"], out["exact"])
    assert e_graph < 1e-4 and e_fused < 5 * e_graph + 1e-7, (e_fused, e_graph)


@pytest.mark.parametrize("at_barrier", [0, 5])
def test_pamp_single_kernel_step_bounded_barrier_wait(gpu, at_barrier):
    """A grid barrier of the single-kernel pAMP step whose arrivals never all come (the test
    hook adds one that no CTA makes; barrier 0 is the norm's, barrier 5 the third Arnoldi
    step's first) gives up after its bounded polls: the call reports PG_ERR_NOT_CONVERGED, the
    device error word reads 2, psi is unchanged, and once the word is cleared the next step
    equals a fresh stepper's."""
    g = golden("hydrogen_small.npz")
    prob = hydrogen_problem(propagator="PamPropagatorGPU", precision="fp32")
    prob.SetupStep(skipWavefunctionSetup=True)
    assert prob.Propagator.Fused
    stepper = prob.Propagator.stepper
    ctx = prob.Propagator.op64.ctx
    _set_psi(prob, g["psi"])
    scales = prob.Propagator.op64.scales(1.0)
    ctx.clear_device_error()
    stepper.set_barrier_probe(1, at_barrier)
    with pytest.raises(nat.PygpuError) as exc:
        stepper.step(prob.psi.GetData(), 0.01, scales)
    assert exc.value.code == nat.PG_ERR_NOT_CONVERGED
    assert ctx.device_error() == 2
    assert relerr(prob.psi.numpy(), g["psi"]) == 0.0
    stepper.set_barrier_probe(0, 0)
    ctx.clear_device_error()
    stepper.step(prob.psi.GetData(), 0.01, scales)
    assert ctx.device_error() == 0
    ref = hydrogen_problem(propagator="PamPropagatorGPU", precision="fp32")
    ref.SetupStep(skipWavefunctionSetup=True)
    _set_psi(ref, g["psi"])
    ref.Propagator.stepper.step(ref.psi.GetData(), 0.01, scales)
    assert relerr(prob.psi.numpy(), ref.psi.numpy()) < 1e-13


def test_cayley_step_fp64_matches_golden(gpu):
    g = golden("hydrogen_small.npz")
    prob = hydrogen_problem(propagator="CayleyPropagatorGPU", precision="fp64", gmres_tolerance=1e-13)
    prob.Propagator.TrueResidual = True
    prob.SetupStep(skipWavefunctionSetup=True)
    _set_psi(prob, g["psi"])
    prob.Propagator.AdvanceStep(float(g["t"]), float(g["dt"]))
    out = prob.psi.numpy()
    assert relerr(out, g["cayley"]) < 1e-11
    st = prob.Propagator.LastStats
    assert 0 <= st.TrueResidual < 1e-10 and 1 <= st.Iterations <= 20
    # the same step enqueued without waiting gives the same state (graph replay)
    prob.Propagator.StepStats = False
    _set_psi(prob, g["psi"])
    prob.Propagator.AdvanceStep(float(g["t"]), float(g["dt"]))
    assert relerr(prob.psi.numpy(), out) < 1e-15
    assert prob.Propagator.LastStats.Iterations == st.Iterations


def test_cayley_mixed_precision_against_oracle(gpu):
    from oracle.propagators import OracleCayley
    g = golden("hydrogen_small.npz")
    ham = oracle_hamiltonian(hydrogen_problem())
    cay = OracleCayley(ham, 0.01, [0], 20, 1e-13)
    psi_ref = g["psi"].copy()
    t0, dt, nsteps = 1.0, 0.01, 10
    for n in range(nsteps):
        psi_ref = cay.step(psi_ref, t0 + n * dt, dt)
    prob = hydrogen_problem(propagator="CayleyPropagatorGPU", precision="fp32", gmres_tolerance=1e-12)
    prob.SetupStep(skipWavefunctionSetup=True)
    _set_psi(prob, g["psi"])
    for n in range(nsteps):
        prob.Propagator.AdvanceStep(t0 + n * dt, dt)
        assert prob.Propagator.LastStats.TrueResidual < 1e-12
    out = prob.psi.numpy()
    assert relerr(out, psi_ref) < 1e-9
    assert infidelity(psi_ref, out, ham.overlap.S) < 1e-14


def test_cayley_single_kernel_step_matches_multi_kernel_step(gpu):
    """The mixed step of a one-electron banded operator runs as one cooperative kernel by
    default; the captured multi-kernel step runs the same scheme. Both reach the FP64 true
    residual bound every step and agree to the GMRES tolerance; the single-kernel stepper
    counts one kernel per step and leaves the device error flag clear."""
    g = golden("hydrogen_small.npz")
    t0, dt, nsteps = 1.0, 0.01, 10
    states = {}
    for fused in (True, False):
        prob = hydrogen_problem(propagator="CayleyPropagatorGPU", precision="fp32", gmres_tolerance=1e-12)
        prob.Propagator.FusedStep = fused
        prob.SetupStep(skipWavefunctionSetup=True)
        assert prob.Propagator.Fused == fused, prob.Propagator.stepper.fused_status
        _set_psi(prob, g["psi"])
        ctx = prob.Propagator.op64.ctx
        k0 = ctx.launches()
        for n in range(nsteps):
            prob.Propagator.AdvanceStep(t0 + n * dt, dt)
            st = prob.Propagator.LastStats
            assert st.TrueResidual < 1e-12 and 1 <= st.Iterations <= 40
        if fused:
            assert ctx.launches() - k0 == nsteps
            assert ctx.device_error() == 0
        states[fused] = prob.psi.numpy()
    assert relerr(states[True], states[False]) < 1e-10


def test_cayley_single_kernel_step_long_fibres_and_basis_bound(gpu):
    """Fibres longer than one CTA's threads (N = 1000: several rows per thread) step on the
    single-kernel path to the same bound; a Krylov basis above its bound (32) keeps the
    multi-kernel step."""
    nang, N = 6, 1000
    i = np.arange(N)
    psi = np.zeros((nang, N), complex)
    psi[0] = np.exp(-((i - 150.0) / 60.0) ** 2)
    psi[1] = 0.3j * np.exp(-((i - 200.0) / 80.0) ** 2)
    psi /= np.linalg.norm(psi)
    prob = hydrogen_problem(lmax=nang - 1, nbsplines=N, rmax=200.0, propagator="CayleyPropagatorGPU",
                            precision="fp32", gmres_tolerance=1e-12)
    prob.SetupStep(skipWavefunctionSetup=True)
    assert prob.Propagator.Fused
    ref = hydrogen_problem(lmax=nang - 1, nbsplines=N, rmax=200.0, propagator="CayleyPropagatorGPU",
                           precision="fp32", gmres_tolerance=1e-12)
    ref.Propagator.FusedStep = False
    ref.SetupStep(skipWavefunctionSetup=True)
    _set_psi(prob, psi)
    _set_psi(ref, psi)
    for n in range(4):
        for p in (prob, ref):
            p.Propagator.AdvanceStep(1.0 + 0.01 * n, 0.01)
            assert p.Propagator.LastStats.TrueResidual < 1e-12
    assert relerr(prob.psi.numpy(), ref.psi.numpy()) < 1e-10
    big = hydrogen_problem(propagator="CayleyPropagatorGPU", precision="fp32", krylov_basis_size=40)
    big.SetupStep(skipWavefunctionSetup=True)
    assert not big.Propagator.Fused


def test_cayley_single_kernel_step_full_size_properties(gpu):
    """At the benchmark's full size (lmax 40, 600 B-splines, 41 x 600 coefficients, dt 0.01 in
    the 800 nm pulse) size-independent properties of 40 mixed single-kernel steps: every step
    meets the FP64 true-residual bound, the S-norm is conserved (Crank-Nicolson is unitary in
    the S metric) to 1e-10, and the state equals the plain FP64 path's to 1e-12 infidelity."""
    import pyprop_gb300 as pp
    from pyprop_gb300.workloads import hydrogen
    kw = dict(lmax=40, nbsplines=600, rmax=400.0, timestep=0.01, pulse_duration=50.0, amplitude=0.05,
              wavelength_nm=800.0, krylov_basis_size=20, gmres_tolerance=1e-12, duration=50.0)
    out = {}
    for prec in ("fp32", "fp64"):
        prob = pp.Problem(pp.LoadString(hydrogen(propagator="CayleyPropagatorGPU", precision=prec, **kw)))
        prob.SetupStep(skipWavefunctionSetup=True)
        assert prob.Propagator.Fused == (prec == "fp32")
        shape = prob.psi.GetRepresentation().GetFullShape()
        rng = np.random.default_rng(40)
        psi = np.zeros(shape, complex)
        i = np.arange(shape[1])
        psi[0] = np.exp(-((i - 60.0) / 25.0) ** 2)
        psi[1] = 0.2 * np.exp(-((i - 80.0) / 30.0) ** 2) * (1 + 0.1j * rng.normal(size=shape[1]))
        prob.psi.SetData(psi / np.linalg.norm(psi))
        prob.PropagatedTime = 20.0  # near the pulse maximum
        S = prob.psi.GetRepresentation().radial.BSplineObject.dense(prob.psi.GetRepresentation().overlap_rows)
        n0 = np.vdot(prob.psi.numpy(), prob.psi.numpy() @ S.T).real
        for _ in range(40):
            prob.AdvanceStep()
            if prec == "fp32":
                assert prob.Propagator.LastStats.TrueResidual < 1e-12
        final = prob.psi.numpy()
        assert abs(np.vdot(final, final @ S.T).real / n0 - 1.0) < 1e-10, prec
        out[prec] = final
    assert infidelity(out["fp64"], out["fp32"], S) < 1e-12


@pytest.mark.parametrize("variant", [1, 2])
def test_cayley_single_kernel_step_bounded_barrier_wait(gpu, variant):
    """A grid barrier of the single-kernel step whose arrivals never all come (the test hook
    adds one arrival that no CTA makes) gives up after its bounded polls: the step returns, the
    device error word reads 2, the step call reports it, psi is unchanged, and the next normal
    step is correct. Both layouts (one CTA per channel; three-CTA clusters)."""
    g = golden("hydrogen_small.npz")
    prob = hydrogen_problem(propagator="CayleyPropagatorGPU", precision="fp32", gmres_tolerance=1e-12)
    prob.SetupStep(skipWavefunctionSetup=True)
    assert prob.Propagator.Fused
    stepper = prob.Propagator.stepper
    stepper.set_fused_variant(variant)
    assert stepper.fused_variant() == variant
    ctx = prob.Propagator.op64.ctx
    _set_psi(prob, g["psi"])
    scales = prob.Propagator.op64.scales(1.005)
    ctx.clear_device_error()
    stepper.set_barrier_probe(1)
    with pytest.raises(nat.PygpuError) as exc:
        stepper.step(prob.psi.GetData(), 0.01, scales)
    assert exc.value.code == -7  # PG_ERR_NOT_CONVERGED: the step was abandoned
    assert ctx.device_error() == 2
    assert relerr(prob.psi.numpy(), g["psi"]) == 0.0
    stepper.set_barrier_probe(0)
    ctx.clear_device_error()
    st = stepper.step(prob.psi.GetData(), 0.01, scales)
    assert ctx.device_error() == 0
    assert st.TrueResidual < 1e-12
    ref = hydrogen_problem(propagator="CayleyPropagatorGPU", precision="fp32", gmres_tolerance=1e-12)
    ref.SetupStep(skipWavefunctionSetup=True)
    _set_psi(ref, g["psi"])
    ref.Propagator.stepper.step(ref.psi.GetData(), 0.01, scales)
    assert relerr(prob.psi.numpy(), ref.psi.numpy()) < 1e-13


@pytest.mark.parametrize("variant", [1, 2])
def test_cayley_single_kernel_step_abandoned_after_first_pass_started(gpu, variant):
    """A bounded wait that runs out at a later grid barrier (barrier 4, after the first
    refinement pass and its first GMRES iteration have started) is reported too: the step call
    fails with PG_ERR_NOT_CONVERGED, the error word reads 2 and stays set, so a step enqueued
    without statistics and read afterwards reports it as well; once the word is cleared, steps
    from the original state are correct again. Both layouts."""
    g = golden("hydrogen_small.npz")
    prob = hydrogen_problem(propagator="CayleyPropagatorGPU", precision="fp32", gmres_tolerance=1e-12)
    prob.SetupStep(skipWavefunctionSetup=True)
    assert prob.Propagator.Fused
    stepper = prob.Propagator.stepper
    stepper.set_fused_variant(variant)
    ctx = prob.Propagator.op64.ctx
    _set_psi(prob, g["psi"])
    scales = prob.Propagator.op64.scales(1.005)
    ctx.clear_device_error()
    stepper.set_barrier_probe(1, 4)
    with pytest.raises(nat.PygpuError) as exc:
        stepper.step(prob.psi.GetData(), 0.01, scales)
    assert exc.value.code == -7
    assert ctx.device_error() == 2
    # the word is sticky: a normal step enqueued now still reads as abandoned
    stepper.set_barrier_probe(0)
    stepper.step(prob.psi.GetData(), 0.01, scales, want_stats=False)
    with pytest.raises(nat.PygpuError) as exc:
        stepper.last_stats()
    assert exc.value.code == -7
    ctx.clear_device_error()
    _set_psi(prob, g["psi"])
    st = stepper.step(prob.psi.GetData(), 0.01, scales)
    assert ctx.device_error() == 0 and st.TrueResidual < 1e-12
    ref = hydrogen_problem(propagator="CayleyPropagatorGPU", precision="fp32", gmres_tolerance=1e-12)
    ref.SetupStep(skipWavefunctionSetup=True)
    _set_psi(ref, g["psi"])
    ref.Propagator.stepper.step(ref.psi.GetData(), 0.01, scales)
    assert relerr(prob.psi.numpy(), ref.psi.numpy()) < 1e-13


@pytest.mark.parametrize("lmax,nbsplines,rmax,nsteps", [(3, 40, 40.0, 10), (40, 600, 400.0, 40), (8, 267, 100.0, 20)])
def test_cayley_cluster_layout_matches_one_cta_per_channel(gpu, lmax, nbsplines, rmax, nsteps):
    """The single-kernel step with each channel on a three-CTA cluster (the solve factors in
    shared memory, boundary values through distributed shared memory) and with one CTA per
    channel: the same states to the GMRES tolerance after steps in the field, the FP64 true
    residual bound every step, one kernel per step. Shapes: the small model (the third CTA of
    each cluster owns no fibre block, only boundary rows), the benchmark's lmax 40 / 600
    B-splines, and an ensemble member's lmax 8 / 267 B-splines."""
    out = {}
    for variant in (1, 2):
        prob = hydrogen_problem(lmax=lmax, nbsplines=nbsplines, rmax=rmax, propagator="CayleyPropagatorGPU",
                                precision="fp32", gmres_tolerance=1e-12, amplitude=0.05, pulse_duration=50.0)
        prob.SetupStep(skipWavefunctionSetup=True)
        assert prob.Propagator.Fused
        prob.Propagator.stepper.set_fused_variant(variant)
        assert prob.Propagator.stepper.fused_variant() == variant
        shape = prob.psi.GetRepresentation().GetFullShape()
        rng = np.random.default_rng(11)
        psi = np.zeros(shape, complex)
        i = np.arange(shape[1])
        psi[0] = np.exp(-((i - shape[1] / 8.0) / (shape[1] / 20.0)) ** 2)
        psi[1] = 0.3 * np.exp(-((i - shape[1] / 6.0) / (shape[1] / 15.0)) ** 2) * (1 + 0.1j * rng.normal(size=shape[1]))
        _set_psi(prob, psi / np.linalg.norm(psi))
        ctx = prob.Propagator.op64.ctx
        k0 = ctx.launches()
        for n in range(nsteps):
            prob.Propagator.AdvanceStep(20.0 + 0.01 * n, 0.01)
            assert prob.Propagator.LastStats.TrueResidual < 1e-12
        assert ctx.launches() - k0 == nsteps and ctx.device_error() == 0
        out[variant] = prob.psi.numpy()
    assert relerr(out[2], out[1]) < 1e-10


def test_cayley_single_kernel_step_other_spline_order(gpu):
    """B-splines of order 5 (9 diagonals) take the generic-width instance of the single-kernel
    step: the same states as the multi-kernel step to the GMRES tolerance."""
    out = {}
    for fused in (True, False):
        prob = hydrogen_problem(lmax=4, nbsplines=50, rmax=40.0, propagator="CayleyPropagatorGPU", precision="fp32",
                                gmres_tolerance=1e-12, order=5)
        prob.Propagator.FusedStep = fused
        prob.SetupStep(skipWavefunctionSetup=True)
        assert prob.Propagator.Fused == fused
        shape = prob.psi.GetRepresentation().GetFullShape()
        rng = np.random.default_rng(5)
        psi = rng.normal(size=shape) + 1j * rng.normal(size=shape)
        _set_psi(prob, psi / np.linalg.norm(psi))
        for n in range(5):
            prob.Propagator.AdvanceStep(1.0 + 0.01 * n, 0.01)
            assert prob.Propagator.LastStats.TrueResidual < 1e-12
        out[fused] = prob.psi.numpy()
    assert relerr(out[True], out[False]) < 1e-10


def test_piram_ground_state_shift_invert(gpu):
    """Config-1 model (lmax 10, N 150): shift-invert pIRAM ground state E = -1/2."""
    import pyprop_gb300 as pp
    prob = hydrogen_problem(lmax=10, nbsplines=150, rmax=100.0)
    prob.Config.Arpack.inverse_iterations = True
    prob.Config.Arpack.krylov_eigenvalue_shift = -0.7
    solver = pp.PiramSolverGPU(prob, seed=1234)
    solver.Solve()
    ev = solver.GetEigenvalues()
    assert abs(ev[0] + 0.5) < 1e-10 and abs(ev[1] + 0.125) < 1e-9
    solver.SetEigenvector(prob.psi, 0)
    E = prob.GetEnergyExpectationValue()
    assert abs(E + 0.5) < 1e-10
    assert abs(prob.psi.GetNorm() - 1.0) < 1e-12


def test_piram_plain_mode_small_operator(gpu):
    """Plain pIRAM (S^-1 H, smallest real parts) on lmax 0: matches the oracle's pIRAM."""
    import pyprop_gb300 as pp
    from oracle.krylov import piram_solve
    prob = hydrogen_problem(lmax=0, nbsplines=30, rmax=30.0)
    prob.Config.Arpack.krylov_basis_size = 29
    prob.Config.Arpack.krylov_max_iteration_count = 5
    solver = pp.PiramSolverGPU(prob, seed=1234)
    solver.Solve()
    ham = oracle_hamiltonian(prob)
    op = lambda v: ham.overlap.solve(ham.apply_H(v.reshape(1, -1), 0.0)).ravel()
    start = np.random.default_rng(1234).uniform(0.0, 1.0, 30).astype(complex)
    vals, vecs, rs, conv = piram_solve(op, start, 29, 2, 1e-12, 5)
    ev = solver.GetEigenvalues()
    # the lowest Ritz value is converged in both; the second is not yet, so the two runs
    # (CGS2 on the GPU, DGKS in the oracle) agree only to the Ritz error bound
    assert abs(ev[0] - vals[0].real) < 1e-9
    assert abs(ev[1] - vals[1].real) < 1e-3
    assert abs(ev[0] + 0.5) < 1e-6


def test_problem_energy_and_norm(gpu):
    """Problem API: energy <H> of a state and S-norm, GPU vs oracle."""
    g = golden("hydrogen_small.npz")
    prob = hydrogen_problem()
    prob.SetupStep(skipWavefunctionSetup=True)
    _set_psi(prob, g["psi"])
    ham = oracle_hamiltonian(prob)
    assert abs(prob.psi.GetNorm() - ham.norm(g["psi"])) < 1e-13
    E = prob.GetEnergyExpectationValue()
    assert abs(E - ham.energy(g["psi"], 0.0)) < 1e-10 * abs(E)
