"""Two-electron (helium) model on the GPU: rank-3 operator, overlap on both radial ranks,
energy and pAMP propagation of the ground state, against the CPU oracle."""
import numpy as np
import pytest
import scipy.linalg as sl

from pyprop_gb300 import _native as nat
from tests.helpers import helium_dense, helium_problem, relerr

pytestmark = pytest.mark.gpu


def _setup():
    prob = helium_problem(lmax=1, nbsplines=16, rmax=15.0)
    H, S3, terms = helium_dense(prob)
    w, v = sl.eigh(H, S3, subset_by_index=[0, 0])
    return prob, H, S3, terms, w[0], v[:, 0]


def test_helium_operator_matvec(gpu):
    import torch
    prob, H, S3, terms, e0, v0 = _setup()
    bp = prob.Propagator.BasePropagator
    bp.SetupStep(0.01)
    shape = prob.psi.GetRepresentation().GetFullShape()
    x = np.random.default_rng(3).standard_normal(shape) + 1j * np.random.default_rng(4).standard_normal(shape)
    ref = (H @ x.ravel()).reshape(shape)
    for prec, dt, tol in [(nat.PG_FP64, torch.complex128, 1e-12), (nat.PG_FP32, torch.complex64, 2e-5)]:
        op = bp.device_operator(prec)
        src = torch.as_tensor(x, device="cuda").to(dt)
        dst = torch.zeros(shape, dtype=dt, device="cuda")
        op.matvec(op.scales(0.0), src, dst)
        assert relerr(dst.to(torch.complex128).cpu().numpy(), ref) < tol, prec


def test_helium_overlap_on_both_radial_ranks(gpu):
    import torch
    prob, H, S3, terms, e0, v0 = _setup()
    repr_ = prob.psi.GetRepresentation()
    shape = repr_.GetFullShape()
    x = np.random.default_rng(5).standard_normal(shape) + 0j
    prob.psi.GetData().copy_(torch.as_tensor(x, device="cuda"))
    repr_.MultiplyOverlap(prob.psi)
    assert relerr(prob.psi.numpy().ravel(), S3 @ x.ravel()) < 1e-13
    repr_.SolveOverlap(prob.psi)
    assert relerr(prob.psi.numpy(), x) < 1e-11


def test_helium_ground_state_energy_and_pamp_propagation(gpu):
    """The oracle's ground state: E on the GPU equals the eigenvalue; pAMP steps (balanced
    overlap on both radial ranks) only rotate its phase."""
    import torch
    prob, H, S3, terms, e0, v0 = _setup()
    prob.SetupStep(skipWavefunctionSetup=True)
    shape = prob.psi.GetRepresentation().GetFullShape()
    psi0 = v0.reshape(shape).astype(np.complex128)
    prob.psi.GetData().copy_(torch.as_tensor(psi0, device="cuda"))
    E = prob.GetEnergyExpectationValue()
    assert abs(E - e0) < 1e-10, (E, e0)
    assert abs(e0 + 2.9) < 0.01
    prob.psi.GetData().copy_(torch.as_tensor(psi0 / np.sqrt(np.vdot(psi0, (S3 @ psi0.ravel()).reshape(shape)).real),
                                             device="cuda"))
    dt, nsteps = 0.01, 10
    for _ in range(nsteps):
        prob.Propagator.AdvanceStep(0.0, dt)
    out = prob.psi.numpy().ravel()
    ref = np.exp(-1j * e0 * dt * nsteps) * psi0.ravel() / np.sqrt(np.vdot(psi0.ravel(), S3 @ psi0.ravel()).real)
    assert relerr(out, ref) < 1e-9
    assert abs(prob.psi.GetNorm() - 1.0) < 1e-12


def test_helium_in_a_laser_field_pamp_matches_dense_exponential(gpu):
    """Time-dependent two-electron propagation (length-gauge coupling on
    SelectionRule_LinearPolarizedField pairs): pAMP steps with H frozen at the step start
    against exp(-i dt S^-1 H(t)) of the dense oracle operator."""
    import torch
    from oracle.operators import dense_operator
    # the radial band (2k-1 = 13 diagonals) needs more than 12 B-splines on the device
    prob = helium_problem(lmax=1, nbsplines=14, rmax=12.0, L=(0, 1), amplitude=0.1, frequency=1.0,
                          pulse_duration=2.0)
    H, S3, terms = helium_dense(prob)
    pots = prob.Propagator.BasePropagator.PotentialList
    mats = [dense_operator([t], [1.0], terms[0].nang, terms[0].N) for t in terms]
    prob.SetupStep(skipWavefunctionSetup=True)
    shape = prob.psi.GetRepresentation().GetFullShape()
    rng = np.random.default_rng(8)
    psi = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    psi /= np.sqrt(np.vdot(psi.ravel(), S3 @ psi.ravel()).real)
    prob.psi.GetData().copy_(torch.as_tensor(psi, device="cuda"))
    Sinv = np.linalg.inv(S3)
    ref = psi.ravel().copy()
    t0, dt = 0.5, 0.01
    for n in range(5):
        t = t0 + n * dt
        Ht = sum(pot.GetTimeScaling(t) * M for pot, M in zip(pots, mats))
        ref = sl.expm(-1j * dt * Sinv @ Ht) @ ref
        prob.Propagator.AdvanceStep(t, dt)
    assert relerr(prob.psi.numpy().ravel(), ref) < 1e-10
    assert abs(prob.psi.GetNorm() - 1.0) < 1e-11


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_helium_cayley_steps_match_dense_crank_nicolson(gpu, precision):
    """Two-electron Cayley steps preconditioned by the fast-diagonalization radial block
    preconditioner, against the dense solve (S + i dt/2 H) psi' = (S - i dt/2 H) psi with H at
    t + dt/2; the GMRES true residual meets 1e-12."""
    import torch
    from oracle.operators import dense_operator
    prob = helium_problem(lmax=1, nbsplines=14, rmax=12.0, L=(0, 1), amplitude=0.1, frequency=1.0,
                          pulse_duration=2.0, propagator="CayleyPropagatorGPU", precision=precision)
    H, S3, terms = helium_dense(prob)
    pots = prob.Propagator.BasePropagator.PotentialList
    mats = [dense_operator([t], [1.0], terms[0].nang, terms[0].N) for t in terms]
    prob.SetupStep(skipWavefunctionSetup=True)
    if precision == "fp64":
        prob.Propagator.TrueResidual = True
        prob.Propagator.SetupStep(0.01)
    shape = prob.psi.GetRepresentation().GetFullShape()
    rng = np.random.default_rng(9)
    psi = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    psi /= np.sqrt(np.vdot(psi.ravel(), S3 @ psi.ravel()).real)
    prob.psi.GetData().copy_(torch.as_tensor(psi, device="cuda"))
    ref = psi.ravel().copy()
    t0, dt = 0.5, 0.01
    for n in range(5):
        t = t0 + n * dt
        Ht = sum(pot.GetTimeScaling(t + dt / 2) * M for pot, M in zip(pots, mats))
        ref = np.linalg.solve(S3 + 0.5j * dt * Ht, (S3 - 0.5j * dt * Ht) @ ref)
        prob.Propagator.AdvanceStep(t, dt)
        st = prob.Propagator.LastStats
        assert 0 <= st.TrueResidual < 1e-11, (precision, st.TrueResidual)
    assert relerr(prob.psi.numpy().ravel(), ref) < (1e-10 if precision == "fp64" else 1e-8)


def _factored_case(gpu_precisions, **kw):
    """(problem, x, {precision: GPU H(t) x}, oracle H(t) x) for a factorized two-electron model."""
    import torch
    from oracle.operators import factored_multiply
    prob = helium_problem(**kw)
    bp = prob.Propagator.BasePropagator
    bp.SetupStep(0.01)
    pots = bp.PotentialList
    assert all(p.Factors is not None for p in pots)
    shape = prob.psi.GetRepresentation().GetFullShape()
    rng = np.random.default_rng(21)
    x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    t = 0.37
    out = {}
    for prec, dt in gpu_precisions:
        op = bp.device_operator(prec)
        sc = op.scales(t)
        src = torch.as_tensor(x, device="cuda").to(dt)
        dst = torch.zeros(shape, dtype=dt, device="cuda")
        op.matvec(sc, src, dst)
        out[prec] = dst.to(torch.complex128).cpu().numpy()
    ref = factored_multiply([(p.Factors, 1 + i) for i, p in enumerate(pots)], sc, x, np.zeros(shape, complex))
    return prob, x, out, ref


def test_factored_two_electron_matvec_matches_oracle(gpu):
    """The factorized two-electron operator (multipoles of the repulsion, laser coupling,
    field-free terms; more than 32 coupled channels, so more than one channel tile of both
    radial kernels) on the GPU against the oracle's point-wise factored multiply, at a
    field-on time."""
    import torch
    prob, x, out, ref = _factored_case([(nat.PG_FP64, torch.complex128), (nat.PG_FP32, torch.complex64)],
                                       lmax=4, L=(0, 1, 2), nbsplines=14, rmax=12.0, amplitude=0.07,
                                       frequency=1.0, pulse_duration=2.0)
    assert prob.psi.GetRepresentation().GetFullShape()[0] > 32
    assert relerr(out[nat.PG_FP64], ref) < 1e-12
    assert relerr(out[nat.PG_FP32], ref) < 2e-5


def test_factored_matvec_long_radial_rank(gpu):
    """150 splines per electron: the last radial rank spans two point tiles (128 + 22) of the
    radial stencil kernel; FP64 and FP32 against the oracle."""
    import torch
    prob, x, out, ref = _factored_case([(nat.PG_FP64, torch.complex128), (nat.PG_FP32, torch.complex64)],
                                       lmax=1, L=(0,), nbsplines=150, rmax=30.0)
    assert relerr(out[nat.PG_FP64], ref) < 1e-12
    assert relerr(out[nat.PG_FP32], ref) < 2e-5


def test_factored_and_per_pair_operators_agree(gpu):
    """The same two-electron Hamiltonian, factorized and stored per angular pair as in the
    reference, gives the same matvec on the GPU (with the overlap slot)."""
    import torch
    res = []
    for fz in (True, False):
        prob = helium_problem(lmax=2, L=(0, 1), nbsplines=16, rmax=15.0, amplitude=0.05, factorize=fz)
        bp = prob.Propagator.BasePropagator
        bp.SetupStep(0.01)
        shape = prob.psi.GetRepresentation().GetFullShape()
        rng = np.random.default_rng(8)
        x = torch.as_tensor(rng.standard_normal(shape) + 1j * rng.standard_normal(shape), device="cuda")
        op = bp.device_operator(nat.PG_FP64, with_overlap=True)
        y = torch.zeros_like(x)
        op.matvec(op.scales(0.61, 0.5j * 0.01, 1.0), x, y)
        res.append(y.cpu().numpy())
    assert relerr(res[0], res[1]) < 1e-13


def test_fast_diagonalization_preconditioner_solves_the_separable_block(gpu):
    """PG_BAND_PREC_SOLVE of the fast-diagonalization preconditioner (FP64 and FP32) against
    the dense inverse of cS S x S + cH (h_l1 x S + S x h_l2) on every channel; and the Cayley
    GMRES needs fewer iterations with it than with the Kronecker-product preconditioner."""
    import scipy.linalg as sl
    import torch
    from pyprop_gb300.propagator import TwoElectronKroneckerPreconditioner
    prob = helium_problem(lmax=2, nbsplines=16, rmax=15.0, L=(0, 1), propagator="CayleyPropagatorGPU",
                          precision="fp32")
    prob.SetupStep(skipWavefunctionSetup=True)
    pre = prob.Propagator.Preconditioner
    assert pre.Method == "fast-diagonalization"
    repr_ = prob.psi.GetRepresentation()
    shape = repr_.GetFullShape()
    S = repr_.radial.BSplineObject.dense(repr_.overlap_rows)
    cS, cH = pre.OverlapScaling, pre.HamiltonianScaling
    rng = np.random.default_rng(4)
    x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    ref = np.empty_like(x)
    for a, ix in enumerate(repr_.bases[0].indices):
        h1, h2 = pre._dense(ix.l1), pre._dense(ix.l2)
        M = cS * np.kron(S, S) + cH * (np.kron(h1, S) + np.kron(S, h2))
        ref[a] = np.linalg.solve(M, x[a].ravel()).reshape(shape[1:])
    for prec, dt, tol in ((nat.PG_FP64, torch.complex128, 1e-10), (nat.PG_FP32, torch.complex64, 1e-4)):
        y = torch.as_tensor(x, device="cuda").to(dt)
        pre.solvers[prec].apply(nat.PG_BAND_PREC_SOLVE, y)
        assert relerr(y.to(torch.complex128).cpu().numpy(), ref) < tol, prec
    # GMRES iterations of one Cayley step: fast diagonalization against the Kronecker product
    psi = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    psi /= np.linalg.norm(psi)
    iters = {}
    for name in ("fd", "kron"):
        if name == "kron":
            kp = TwoElectronKroneckerPreconditioner(prob.psi)
            kp.Z, kp.Mass = pre.Z, pre.Mass
            kp.SetHamiltonianScaling(cH)
            kp.SetOverlapScaling(cS)
            prob.Propagator.Preconditioner = kp
            prob.Propagator.SetupStep(0.01)
        prob.psi.GetData().copy_(torch.as_tensor(psi, device="cuda"))
        prob.Propagator.AdvanceStep(0.0, 0.01)
        iters[name] = prob.Propagator.LastStats.Iterations
    print("GMRES iterations per Cayley step:", iters)
    assert iters["fd"] < iters["kron"]


def test_factored_fp64_emulation_matches_oracle(gpu):
    """The FP64 operator with its factorized terms in double-float arithmetic (FP32 pairs,
    error-free products and sums) meets the FP64 tolerance against the oracle, with and without
    the S x S overlap factor (the overlap slot of the Cayley residual operator)."""
    import torch
    from oracle.operators import factored_multiply
    prob = helium_problem(lmax=4, L=(0, 1, 2), nbsplines=14, rmax=12.0, amplitude=0.07, frequency=1.0,
                          pulse_duration=2.0)
    bp = prob.Propagator.BasePropagator
    bp.SetupStep(0.01)
    pots = bp.PotentialList
    repr_ = prob.psi.GetRepresentation()
    shape = repr_.GetFullShape()
    rng = np.random.default_rng(31)
    x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    S = repr_.radial.BSplineObject.dense(repr_.overlap_rows)
    for with_overlap in (False, True):
        op = bp.device_operator(nat.PG_FP64, with_overlap=with_overlap, fp64_emulation=True)
        assert op.fp64_emulation
        sc = op.scales(0.37, 0.5j * 0.01, 1.0 if with_overlap else 0.0)
        src = torch.as_tensor(x, device="cuda")
        dst = torch.zeros_like(src)
        op.matvec(sc, src, dst)
        ref = factored_multiply([(p.Factors, 1 + i) for i, p in enumerate(pots)], sc, x, np.zeros(shape, complex))
        if with_overlap:
            ref += np.einsum("ij,ajk,lk->ail", S, x, S)
        assert relerr(dst.cpu().numpy(), ref) < 1e-12, with_overlap


def test_fast_diagonalization_large_radial_rank(gpu):
    """130 splines per electron: beyond the shared-memory solve (FP64 at least), the four
    products as batched GEMMs; both precisions against the host evaluation of
    V1 (D o (V1^T X V2)) V2^T."""
    import scipy.linalg as sl
    import torch
    prob = helium_problem(lmax=1, nbsplines=130, rmax=40.0, L=(0,), propagator="CayleyPropagatorGPU",
                          precision="fp32")
    prob.SetupStep(skipWavefunctionSetup=True)
    pre = prob.Propagator.Preconditioner
    repr_ = prob.psi.GetRepresentation()
    shape = repr_.GetFullShape()
    S = repr_.radial.BSplineObject.dense(repr_.overlap_rows)
    cS, cH = pre.OverlapScaling, pre.HamiltonianScaling
    rng = np.random.default_rng(6)
    x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    ref = np.empty_like(x)
    for a, ix in enumerate(repr_.bases[0].indices):
        w1, v1 = sl.eigh(pre._dense(ix.l1), S)
        w2, v2 = sl.eigh(pre._dense(ix.l2), S)
        D = 1.0 / (cS + cH * (w1[:, None] + w2[None, :]))
        ref[a] = v1 @ (D * (v1.T @ x[a] @ v2)) @ v2.T
    for prec, dt, tol in ((nat.PG_FP64, torch.complex128, 1e-10), (nat.PG_FP32, torch.complex64, 1e-4)):
        y = torch.as_tensor(x, device="cuda").to(dt)
        pre.solvers[prec].apply(nat.PG_BAND_PREC_SOLVE, y)
        assert relerr(y.to(torch.complex128).cpu().numpy(), ref) < tol, prec
